"""GB300-native semblance engine for HighPerformanceSeismicStacking.

The compute path is the CUDA library ``lib/libhpss_gb300.so`` behind the C ABI
declared in ``include/hpss.h``; ``capi.Engine`` binds it with ctypes.  ``su``
reads and writes SU files with the reference's gather semantics and
``synthetic`` makes the seeded benchmark lines.
"""
__version__ = "0.1.0"
