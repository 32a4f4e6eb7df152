"""The C ABI library loads and exports every symbol include/hpss.h declares;
calls that need a device fail cleanly without one (CPU only)."""
import ctypes
import re
from pathlib import Path

import pytest

from highperformanceseismicstacking_gb300 import capi

HEADER = Path(__file__).resolve().parents[1] / "include" / "hpss.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(hpss_\w+)\s*\(", text, re.M)))


def test_header_symbols_all_exported():
    lib = capi.lib()
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(capi.EXPORTED) == syms


def test_version_string():
    assert b"sm_103a" in capi.lib().hpss_version()


def _has_gpu():
    n = ctypes.c_int(0)
    return capi.lib().hpss_device_count(ctypes.byref(n)) == 0 and n.value > 0


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device error path")
def test_create_without_device_reports_no_device():
    with pytest.raises(capi.HpssError) as e:
        capi.Engine(0)
    assert e.value.code == -4
    assert b"No CUDA devices" in capi.lib().hpss_last_error(None)


def test_null_handle_calls_are_rejected():
    lib = capi.lib()
    assert lib.hpss_destroy(None) == 0
    assert lib.hpss_set_window(None, 2) == -1
    assert lib.hpss_stream(None) is None
    assert lib.hpss_device_bytes(None) == 0
