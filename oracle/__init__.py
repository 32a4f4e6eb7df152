"""The oracle: a CPU restatement of the reference's semblance hot path.

Test infrastructure only -- imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py to check against, never by the product path.
"""
