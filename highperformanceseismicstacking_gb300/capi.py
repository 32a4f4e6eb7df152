"""ctypes binding of the C ABI in include/hpss.h (libhpss_gb300.so).

There is no fallback: if the CUDA engine is not built, importing this module
raises, and every call returns the engine's own error.  ``Engine`` is a thin
numpy-friendly wrapper that owns one ``hpss_handle``.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional, Sequence, Tuple

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "lib" / "libhpss_gb300.so"

HPSS_OK = 0
ERRORS = {
    -1: "HPSS_ERR_INVALID_ARGUMENT", -2: "HPSS_ERR_LOGIC", -3: "HPSS_ERR_CUDA",
    -4: "HPSS_ERR_NO_DEVICE", -5: "HPSS_ERR_OUT_OF_MEMORY", -6: "HPSS_ERR_NOT_READY",
    -7: "HPSS_ERR_TIMEOUT", -8: "HPSS_ERR_DEVICE_CHECK",
}
MODELS = {"cmp": 0, "zocrs": 1, "oct": 2}
STORAGE = {"fp32": 0, "bf16": 1, "fp16": 2}
KERNELS = {"plain": 0, "tuned": 1, "tuned_exact": 2}
GRID_MODES = {"reference": 0, "inclusive": 1}
PREC_FP64_TRAVELTIME, PREC_COMPENSATED, PREC_FP64 = 1, 2, 4
N_PARAMS = {"cmp": 1, "zocrs": 3, "oct": 2}

# Every symbol include/hpss.h declares.
EXPORTED = [
    "hpss_create", "hpss_destroy", "hpss_last_error", "hpss_version",
    "hpss_device_count", "hpss_upload_gather", "hpss_set_traveltime",
    "hpss_set_window", "hpss_set_grid_mode", "hpss_set_precision", "hpss_set_oct_half_offsets",
    "hpss_linear_search",
    "hpss_linear_search_device",
    "hpss_differential_evolution", "hpss_differential_evolution_device",
    "hpss_stretch_free", "hpss_select_traces", "hpss_stream", "hpss_device_bytes",
    "hpss_linear_search_noalloc", "hpss_noalloc_device_error", "hpss_linear_search_line",
    "hpss_write_result_files",
]


class Stats(C.Structure):
    _fields_ = [("evals", C.c_double), ("not_used", C.c_double),
                ("selected_traces", C.c_double), ("kernel_ms", C.c_double),
                ("selection_ms", C.c_double), ("device_error", C.c_uint32),
                ("kernel_variant", C.c_int32), ("near_ties", C.c_double),
                ("candidate_parts", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class HpssError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def load_library(path: Optional[Path] = None) -> C.CDLL:
    p = Path(path or _LIB_PATH)
    if not p.exists():
        raise ImportError(f"CUDA engine not built ({p} missing): run __graft_entry__.build()")
    lib = C.CDLL(str(p))
    vp, u32, f32, i32 = C.c_void_p, C.c_uint32, C.c_float, C.c_int
    fp, up = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
    sig = {
        "hpss_create": (i32, [i32, C.POINTER(vp)]),
        "hpss_destroy": (i32, [vp]),
        "hpss_last_error": (C.c_char_p, [vp]),
        "hpss_version": (C.c_char_p, []),
        "hpss_device_count": (i32, [C.POINTER(C.c_int)]),
        "hpss_upload_gather": (i32, [vp, fp, fp, fp, u32, u32, f32, i32]),
        "hpss_set_traveltime": (i32, [vp, i32, u32, fp, fp, f32, f32]),
        "hpss_set_window": (i32, [vp, i32]),
        "hpss_set_grid_mode": (i32, [vp, i32]),
        "hpss_set_precision": (i32, [vp, i32]),
        "hpss_set_oct_half_offsets": (i32, [vp, fp, u32]),
        "hpss_linear_search": (i32, [vp, fp, u32, up, i32, fp, C.POINTER(Stats)]),
        "hpss_linear_search_device": (i32, [vp, vp, u32, up, i32, vp, C.POINTER(Stats)]),
        "hpss_linear_search_line": (i32, [vp, fp, fp, fp, u32, u32, f32, i32, fp, u32, up, i32,
                                          fp, C.POINTER(Stats)]),
        "hpss_differential_evolution": (i32, [vp, fp, u32, u32, u32, f32, f32, C.c_uint64, fp,
                                              C.POINTER(Stats)]),
        "hpss_differential_evolution_device": (i32, [vp, vp, u32, u32, u32, f32, f32,
                                                     C.c_uint64, vp, C.POINTER(Stats)]),
        "hpss_stretch_free": (i32, [vp, fp, u32, fp, i32, fp, C.POINTER(Stats)]),
        "hpss_select_traces": (i32, [vp, fp, u32, up]),
        "hpss_stream": (vp, [vp]),
        "hpss_device_bytes": (C.c_size_t, [vp]),
        "hpss_linear_search_noalloc": (i32, [i32, vp, u32, vp, vp, u32, u32, f32, i32, fp, fp,
                                             up, f32, vp, u32, vp, vp]),
        "hpss_noalloc_device_error": (i32, [vp, up]),
        "hpss_write_result_files": (i32, [vp, i32, u32, u32, u32, vp, C.POINTER(C.c_char_p)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = load_library()
    return _lib


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _uptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


class Engine:
    """One device handle: upload a line once, then run searches over midpoints."""

    def __init__(self, device: int = 0, library: Optional[C.CDLL] = None):
        # library: another build of the engine (load_library(path)); default
        # the package's own
        self._lib = library if library is not None else lib()
        h = C.c_void_p()
        rc = self._lib.hpss_create(device, C.byref(h))
        if rc != HPSS_OK:
            raise HpssError(rc, self._lib.hpss_last_error(None).decode())
        self.h = h
        self.model = None
        self.S = 0
        self.np = 0
        self.n_h0 = 0  # OCT target half-offsets of set_oct_half_offsets (0: one h0)

    def close(self):
        if self.h:
            self._lib.hpss_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int):
        if rc != HPSS_OK:
            raise HpssError(rc, self._lib.hpss_last_error(self.h).decode())

    @property
    def stream(self) -> int:
        return int(self._lib.hpss_stream(self.h) or 0)

    def device_bytes(self) -> int:
        return int(self._lib.hpss_device_bytes(self.h))

    def upload_gather(self, samples: np.ndarray, midpoints: np.ndarray,
                      halfoffsets: np.ndarray, dt: float, storage: str = "fp32"):
        samples = np.ascontiguousarray(samples, dtype=np.float32)
        midpoints = np.ascontiguousarray(midpoints, dtype=np.float32)
        halfoffsets = np.ascontiguousarray(halfoffsets, dtype=np.float32)
        n, S = samples.shape
        self._check(self._lib.hpss_upload_gather(
            self.h, _fptr(samples), _fptr(midpoints), _fptr(halfoffsets), n, S,
            C.c_float(dt), STORAGE[storage]))
        self.S = S

    def set_traveltime(self, model: str, lower: Sequence[float], upper: Sequence[float],
                       apm: float = 0.0, h0: float = 0.0):
        lo = np.asarray(lower, np.float32)
        hi = np.asarray(upper, np.float32)
        self._check(self._lib.hpss_set_traveltime(self.h, MODELS[model], lo.size, _fptr(lo),
                                                   _fptr(hi), C.c_float(apm), C.c_float(h0)))
        self.model = model
        self.np = N_PARAMS[model]

    def set_oct_half_offsets(self, h0s: Sequence[float]):
        """OCT over several target half-offsets per call: results come back
        as [len(h0s) * nM0][...] blocks, h0-major; [] restores the single h0
        of set_traveltime."""
        a = np.ascontiguousarray(h0s, np.float32)
        self._check(self._lib.hpss_set_oct_half_offsets(self.h, _fptr(a) if a.size else None,
                                                         a.size))
        self.n_h0 = int(a.size)

    def _blocks(self) -> int:
        return self.n_h0 if (self.model == "oct" and self.n_h0) else 1

    def set_window(self, tau_index: int):
        self._check(self._lib.hpss_set_window(self.h, int(tau_index)))

    def set_precision(self, fp64_traveltime: bool = False, compensated: bool = False,
                      fp64: bool = False):
        """Precision modes of the linear search: FP64 traveltime (ZO-CRS /
        OCT), compensated window sums, or every step in FP64."""
        flags = (PREC_FP64_TRAVELTIME if fp64_traveltime else 0) | \
            (PREC_COMPENSATED if compensated else 0) | (PREC_FP64 if fp64 else 0)
        self._check(self._lib.hpss_set_precision(self.h, flags))

    def set_grid_mode(self, mode: str):
        """'reference' (uniform in v, upper bound excluded) or 'inclusive'
        (both bounds included, velocity uniform in 4/v^2)."""
        self._check(self._lib.hpss_set_grid_mode(self.h, GRID_MODES[mode]))

    def linear_search(self, m0s, granularity: Sequence[int], kernel: str = "tuned"
                      ) -> Tuple[np.ndarray, dict]:
        m0s = np.ascontiguousarray(m0s, dtype=np.float32)
        g = np.asarray(granularity, np.uint32)
        out = np.zeros((m0s.size * self._blocks(), 2 + self.np, self.S), np.float32)
        st = Stats()
        self._check(self._lib.hpss_linear_search(self.h, _fptr(m0s), m0s.size, _uptr(g),
                                                  KERNELS[kernel], _fptr(out), C.byref(st)))
        return out, st.as_dict()

    def linear_search_line(self, samples: np.ndarray, midpoints: np.ndarray,
                           halfoffsets: np.ndarray, dt: float, m0s, granularity: Sequence[int],
                           kernel: str = "tuned", storage: str = "fp32",
                           out: Optional[np.ndarray] = None) -> Tuple[np.ndarray, dict]:
        """Upload a line and search it in one call, the upload overlapped with
        the search (hpss_linear_search_line); the traveltime and the window
        must be set before.  The line stays resident afterwards, as after
        upload_gather.  `out` (optional): a C-contiguous float32 array of
        shape (len(m0s), 2 + nParams, S) to write into (e.g. page-locked)."""
        samples = np.ascontiguousarray(samples, dtype=np.float32)
        midpoints = np.ascontiguousarray(midpoints, dtype=np.float32)
        halfoffsets = np.ascontiguousarray(halfoffsets, dtype=np.float32)
        m0s = np.ascontiguousarray(m0s, dtype=np.float32)
        n, S = samples.shape
        g = np.asarray(granularity, np.uint32)
        shape = (m0s.size, 2 + self.np, S)
        if out is None:
            out = np.zeros(shape, np.float32)
        elif out.shape != shape or out.dtype != np.float32 or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous float32 array of shape {shape}")
        st = Stats()
        self._check(self._lib.hpss_linear_search_line(
            self.h, _fptr(samples), _fptr(midpoints), _fptr(halfoffsets), n, S, C.c_float(dt),
            STORAGE[storage], _fptr(m0s), m0s.size, _uptr(g), KERNELS[kernel], _fptr(out),
            C.byref(st)))
        self.S = S
        return out, st.as_dict()

    def linear_search_device(self, d_m0s: int, n_m0: int, granularity, d_out: int,
                             kernel: str = "tuned", stats: bool = False):
        g = np.asarray(granularity, np.uint32)
        st = Stats()
        self._check(self._lib.hpss_linear_search_device(
            self.h, C.c_void_p(d_m0s), n_m0, _uptr(g), KERNELS[kernel], C.c_void_p(d_out),
            C.byref(st) if stats else None))
        return st.as_dict() if stats else None

    def differential_evolution(self, m0s, population: int, generations: int, F: float,
                               CR: float, seed: int) -> Tuple[np.ndarray, dict]:
        m0s = np.ascontiguousarray(m0s, dtype=np.float32)
        out = np.zeros((m0s.size * self._blocks(), 2 + self.np, self.S), np.float32)
        st = Stats()
        self._check(self._lib.hpss_differential_evolution(
            self.h, _fptr(m0s), m0s.size, population, generations, C.c_float(F),
            C.c_float(CR), C.c_uint64(seed), _fptr(out), C.byref(st)))
        return out, st.as_dict()

    def stretch_free(self, m0s, params: np.ndarray, nmax: int = 10
                     ) -> Tuple[np.ndarray, dict]:
        m0s = np.ascontiguousarray(m0s, dtype=np.float32)
        params = np.ascontiguousarray(params, dtype=np.float32)
        if params.size != m0s.size * self._blocks() * self.np * self.S:
            raise ValueError("params must hold [blocks * nM0][nParams][S] values")
        out = np.zeros((m0s.size * self._blocks(), 3, self.S), np.float32)
        st = Stats()
        self._check(self._lib.hpss_stretch_free(self.h, _fptr(m0s), m0s.size, _fptr(params),
                                                 nmax, _fptr(out), C.byref(st)))
        return out, st.as_dict()

    def select_traces(self, m0s) -> np.ndarray:
        m0s = np.ascontiguousarray(m0s, dtype=np.float32)
        counts = np.zeros(m0s.size * self._blocks(), np.uint32)
        self._check(self._lib.hpss_select_traces(self.h, _fptr(m0s), m0s.size, _uptr(counts)))
        return counts


def write_result_files(slab, headers: np.ndarray, paths: Sequence[Optional[str]],
                       device_ptr: Optional[int] = None) -> None:
    """SU result files from a result slab [nM0][rows][S] (numpy array, or a
    device pointer with `slab` giving only the shape): file r holds, per
    midpoint, headers[i] (240-byte SU header) and slab[i][r]
    (hpss_write_result_files).  A None path skips its row."""
    n, rows, S = slab.shape
    hdr = np.ascontiguousarray(headers)
    if hdr.nbytes != n * 240:
        raise ValueError("headers must be nM0 SU trace headers (240 bytes each)")
    arr = (C.c_char_p * rows)(*[p.encode() if p else None for p in paths])
    if device_ptr is None:
        host = np.ascontiguousarray(slab, dtype=np.float32)
        rc = lib().hpss_write_result_files(host.ctypes.data, 0, n, rows, S, hdr.ctypes.data, arr)
    else:
        rc = lib().hpss_write_result_files(C.c_void_p(device_ptr), 1, n, rows, S,
                                           hdr.ctypes.data, arr)
    if rc != HPSS_OK:
        raise HpssError(rc, lib().hpss_last_error(None).decode())
