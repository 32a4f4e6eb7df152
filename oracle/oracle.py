"""numpy front end of the oracle's C restatement (hpss_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py to check or time the reference algorithm on the
host.  The product path never imports this module.

Parity: pinned against outputs of the reference's own CUDA kernels (compiled
from the reference sources, run on a GB300; fixtures in tests/golden/) and
against analytic known-answer cases.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

_HERE = Path(__file__).resolve().parent
MODELS = {"cmp": 0, "zocrs": 1, "oct": 2}
N_PARAMS = {"cmp": 1, "zocrs": 3, "oct": 2}

_lib = None


def lib():
    global _lib
    if _lib is None:
        p = _HERE / "liboracle.so"
        if not p.exists():
            from highperformanceseismicstacking_gb300 import build
            build.build_oracle()
        _lib = C.CDLL(str(p))
        fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
        up, u32, f32, i32 = C.POINTER(C.c_uint32), C.c_uint32, C.c_float, C.c_int
        common = [i32, fp, u32, u32, f32, i32, fp, fp, up, u32, f32, f32, f32]
        _lib.oracle_ls_eval_f32.argtypes = common + [fp, u32, fp, fp, fp, i32]
        _lib.oracle_ls_eval_f64.argtypes = common + [fp, u32, dp, dp, dp, i32]
        _lib.oracle_sf_eval_f32.argtypes = common + [fp, i32, fp, fp, fp, i32]
        _lib.oracle_sf_eval_f64.argtypes = common + [fp, i32, dp, dp, dp, i32]
        _lib.oracle_eval_raw_f32.argtypes = common + [fp, u32, fp, fp, i32]
        _lib.oracle_eval_raw_f64.argtypes = common + [fp, u32, dp, dp, i32]
        _lib.oracle_ls_eval_samples_f32.argtypes = common + [fp, u32, up, u32, fp, fp, i32]
        _lib.oracle_ls_eval_samples_f64.argtypes = common + [fp, u32, up, u32, dp, dp, i32]
        _lib.oracle_argmax_f32.argtypes = [fp, u32, u32, C.POINTER(C.c_int32)]
        _lib.oracle_argmax_f64.argtypes = [dp, u32, u32, C.POINTER(C.c_int32)]
        _lib.oracle_build_grid.argtypes = [i32, fp, fp, up, fp]
        _lib.oracle_build_grid_inclusive.argtypes = [i32, fp, fp, up, fp]
        _lib.oracle_select.argtypes = [i32, fp, fp, u32, f32, f32, f32, u32, f32, fp, u32,
                                       C.POINTER(C.c_uint8)]
        _lib.oracle_max_threads.restype = i32
    return _lib


def _f(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _u(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def build_grid(model: str, lower, upper, gran, mode: str = "reference") -> np.ndarray:
    lo = np.asarray(lower, np.float32)
    hi = np.asarray(upper, np.float32)
    g = np.asarray(gran, np.uint32)
    P = int(np.prod(g))
    out = np.zeros(P * N_PARAMS[model], np.float32)
    fn = lib().oracle_build_grid if mode == "reference" else lib().oracle_build_grid_inclusive
    fn(MODELS[model], _f(lo), _f(hi), _u(g), _f(out))
    return out.reshape(P, N_PARAMS[model])


def oct_selection_candidates(lower, upper, n: int = 1024) -> np.ndarray:
    """The reference's sampled OCT selection candidates
    (CudaLinearSearchAlgorithm.cu:269-292): a default-constructed
    std::default_random_engine and std::uniform_real_distribution<float> per
    parameter, velocity converted to 4/v^2.

    Third-party algorithm (GNU libstdc++, GCC 13): default_random_engine is
    minstd_rand0 (x <- 16807 x mod 2^31-1, seed 1); generate_canonical<float, 24>
    takes one draw, u = float(x - 1) / 2^31 (nudged below 1); the distribution
    returns u * (b - a) + a in float.  Restated here from that published
    definition; returns [n][2] = (4/v^2, slope)."""
    x = 1
    f32 = np.float32
    out = np.zeros((n, 2), np.float32)
    for prm in range(2):
        a, b = f32(lower[prm]), f32(upper[prm])
        for i in range(n):
            x = (16807 * x) % 2147483647
            u = f32(x - 1) / f32(2147483648.0)
            if u >= f32(1):
                u = np.nextafter(f32(1), f32(0))
            v = f32(u * f32(b - a)) + a
            if prm == 0:
                v = f32(4.0) / f32(v * v)
            out[i, prm] = v
    return out


def select(model: str, mid, hoff, m0: float, apm: float = 0.0, h0: float = 0.0,
           S: int = 0, dt: float = 0.0, cands: Optional[np.ndarray] = None) -> np.ndarray:
    mid = np.ascontiguousarray(mid, np.float32)
    hoff = np.ascontiguousarray(hoff, np.float32)
    mask = np.zeros(mid.size, np.uint8)
    c = np.ascontiguousarray(cands if cands is not None else np.zeros((0, 2)), np.float32)
    lib().oracle_select(MODELS[model], _f(mid), _f(hoff), mid.size, C.c_float(m0),
                        C.c_float(apm), C.c_float(h0), S, C.c_float(dt), _f(c),
                        c.shape[0] if c.ndim == 2 else 0,
                        mask.ctypes.data_as(C.POINTER(C.c_uint8)))
    return mask.astype(bool)


def ls_eval(model: str, samples: np.ndarray, mid, hoff, sel, m0: float, dt: float,
            tau: int, params: np.ndarray, apm: float = 0.0, h0: float = 0.0,
            precision: str = "f32", nthreads: int = 0):
    """Semblance and stack [S][P] for one midpoint (computeSemblancesFor*)."""
    samples = np.ascontiguousarray(samples, np.float32)
    mid = np.ascontiguousarray(mid, np.float32)
    hoff = np.ascontiguousarray(hoff, np.float32)
    sel = np.ascontiguousarray(sel, np.uint32)
    params = np.ascontiguousarray(params, np.float32)
    S = samples.shape[1]
    P = params.shape[0]
    dtype = np.float32 if precision == "f32" else np.float64
    sembl = np.zeros((S, P), dtype)
    stack = np.zeros((S, P), dtype)
    nu = np.zeros((S, P), dtype)
    fn = lib().oracle_ls_eval_f32 if precision == "f32" else lib().oracle_ls_eval_f64
    cv = _f if precision == "f32" else _d
    fn(MODELS[model], _f(samples), S, S, C.c_float(dt), tau, _f(mid), _f(hoff), _u(sel),
       sel.size, C.c_float(m0), C.c_float(apm), C.c_float(h0), _f(params), P, cv(sembl),
       cv(stack), cv(nu), nthreads)
    return sembl, stack, nu


def ls_eval_samples(model: str, samples: np.ndarray, mid, hoff, sel, m0: float, dt: float,
                    tau: int, params: np.ndarray, sidx, apm: float = 0.0, h0: float = 0.0,
                    precision: str = "f32", nthreads: int = 0):
    """ls_eval on the t0 samples sidx only: semblance and stack [len(sidx)][P]."""
    samples = np.ascontiguousarray(samples, np.float32)
    mid = np.ascontiguousarray(mid, np.float32)
    hoff = np.ascontiguousarray(hoff, np.float32)
    sel = np.ascontiguousarray(sel, np.uint32)
    params = np.ascontiguousarray(params, np.float32)
    sidx = np.ascontiguousarray(sidx, np.uint32)
    S = samples.shape[1]
    P = params.shape[0]
    dtype = np.float32 if precision == "f32" else np.float64
    sembl = np.zeros((sidx.size, P), dtype)
    stack = np.zeros((sidx.size, P), dtype)
    fn = lib().oracle_ls_eval_samples_f32 if precision == "f32" else \
        lib().oracle_ls_eval_samples_f64
    cv = _f if precision == "f32" else _d
    fn(MODELS[model], _f(samples), S, S, C.c_float(dt), tau, _f(mid), _f(hoff), _u(sel),
       sel.size, C.c_float(m0), C.c_float(apm), C.c_float(h0), _f(params), P, _u(sidx),
       sidx.size, cv(sembl), cv(stack), nthreads)
    return sembl, stack


def argmax(sembl: np.ndarray) -> np.ndarray:
    S, P = sembl.shape
    out = np.zeros(S, np.int32)
    if sembl.dtype == np.float32:
        lib().oracle_argmax_f32(_f(np.ascontiguousarray(sembl)), S, P,
                                out.ctypes.data_as(C.POINTER(C.c_int32)))
    else:
        lib().oracle_argmax_f64(_d(np.ascontiguousarray(sembl)), S, P,
                                out.ctypes.data_as(C.POINTER(C.c_int32)))
    return out


def ls_result(model: str, sembl, stack, params) -> tuple:
    """Result block [(2+np)][S] as selectBestSemblancesFor* writes it (velocity
    reported as 2/sqrt(c)), plus the chosen candidate index per sample."""
    idx = argmax(sembl)
    S = sembl.shape[0]
    npar = params.shape[1]
    out = np.zeros((2 + npar, S), np.float64 if sembl.dtype == np.float64 else np.float32)
    ok = idx >= 0
    rows = np.arange(S)
    out[0] = np.where(ok, sembl[rows, np.maximum(idx, 0)], -1)
    out[1] = np.where(ok, stack[rows, np.maximum(idx, 0)], 0)
    c = params[np.maximum(idx, 0), 0].astype(out.dtype)
    out[2] = np.where(ok, out.dtype.type(2) / np.sqrt(c), 0)
    for j in range(1, npar):
        out[2 + j] = np.where(ok, params[np.maximum(idx, 0), j], 0)
    return out, idx


def sf_eval(model: str, samples, mid, hoff, sel, m0: float, dt: float, tau: int,
            prior: np.ndarray, nmax: int = 10, apm: float = 0.0, h0: float = 0.0,
            precision: str = "f32", nthreads: int = 0):
    samples = np.ascontiguousarray(samples, np.float32)
    S = samples.shape[1]
    nn = 2 * nmax + 1
    dtype = np.float32 if precision == "f32" else np.float64
    sembl = np.zeros((S, nn), dtype)
    stack = np.zeros((S, nn), dtype)
    nu = np.zeros((S, nn), dtype)
    fn = lib().oracle_sf_eval_f32 if precision == "f32" else lib().oracle_sf_eval_f64
    cv = _f if precision == "f32" else _d
    sel = np.ascontiguousarray(sel, np.uint32)
    prior = np.ascontiguousarray(prior, np.float32)
    fn(MODELS[model], _f(samples), S, S, C.c_float(dt), tau,
       _f(np.ascontiguousarray(mid, np.float32)), _f(np.ascontiguousarray(hoff, np.float32)),
       _u(sel), sel.size, C.c_float(m0), C.c_float(apm), C.c_float(h0), _f(prior), nmax,
       cv(sembl), cv(stack), cv(nu), nthreads)
    return sembl, stack, nu


def eval_raw(model: str, samples, mid, hoff, sel, m0: float, dt: float, tau: int,
             cands: np.ndarray, apm: float = 0.0, h0: float = 0.0, precision: str = "f64",
             nthreads: int = 0):
    """Semblance of explicit raw candidates cands [S][n][np] (velocity first)."""
    samples = np.ascontiguousarray(samples, np.float32)
    S = samples.shape[1]
    cands = np.ascontiguousarray(cands, np.float32)
    n = cands.shape[1]
    dtype = np.float32 if precision == "f32" else np.float64
    sembl = np.zeros((S, n), dtype)
    stack = np.zeros((S, n), dtype)
    fn = lib().oracle_eval_raw_f32 if precision == "f32" else lib().oracle_eval_raw_f64
    cv = _f if precision == "f32" else _d
    sel = np.ascontiguousarray(sel, np.uint32)
    fn(MODELS[model], _f(samples), S, S, C.c_float(dt), tau,
       _f(np.ascontiguousarray(mid, np.float32)), _f(np.ascontiguousarray(hoff, np.float32)),
       _u(sel), sel.size, C.c_float(m0), C.c_float(apm), C.c_float(h0), _f(cands), n,
       cv(sembl), cv(stack), nthreads)
    return sembl, stack


def linear_search(model: str, samples, mid, hoff, m0s: Sequence[float], dt: float, tau: int,
                  lower, upper, gran, apm: float = 0.0, h0: float = 0.0,
                  precision: str = "f32", oct_cands: Optional[np.ndarray] = None,
                  nthreads: int = 0, grid_mode: str = "reference"):
    """Whole reference linear-search flow for a list of midpoints: selection,
    grid, evaluation, argmax.  Returns out [nM0][2+np][S], idx [nM0][S],
    counts [nM0]."""
    params = build_grid(model, lower, upper, gran, grid_mode)
    S = samples.shape[1]
    outs, idxs, counts = [], [], []
    for m0 in m0s:
        mask = select(model, mid, hoff, m0, apm, h0, S, dt, oct_cands)
        sel = np.nonzero(mask)[0].astype(np.uint32)
        counts.append(sel.size)
        if sel.size == 0:
            outs.append(np.zeros((2 + params.shape[1], S), np.float32 if precision == "f32"
                                 else np.float64))
            idxs.append(np.full(S, -2, np.int32))
            continue
        sembl, stack, _ = ls_eval(model, samples, mid, hoff, sel, m0, dt, tau, params, apm, h0,
                                  precision, nthreads)
        o, i = ls_result(model, sembl, stack, params)
        outs.append(o)
        idxs.append(i)
    return np.stack(outs), np.stack(idxs), np.asarray(counts)


# ---- differential evolution helpers ------------------------------------

def _de_sigs():
    L = lib()
    if getattr(L, "_de_ready", False):
        return L
    fp, u32 = C.POINTER(C.c_float), C.c_uint32
    L.oracle_de_uniforms.argtypes = [C.c_uint64, u32, u32, u32, u32, u32, fp]
    L.oracle_de_initial_population.argtypes = [C.c_uint64, u32, u32, u32, C.c_int, fp, fp, fp]
    L.oracle_select_oct_per_sample.argtypes = [fp, fp, u32, C.c_float, C.c_float, C.c_float,
                                               u32, C.c_float, fp, u32, C.POINTER(C.c_uint8)]
    L._de_ready = True
    return L


def de_key(m0: float) -> int:
    """The DE random stream's midpoint key: the midpoint's FP32 bit pattern."""
    return int(np.asarray(m0, np.float32).view(np.uint32))


def de_uniforms(seed: int, m0i: int, s: int, ind: int, gen: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    _de_sigs().oracle_de_uniforms(seed, m0i, s, ind, gen, n, _f(out))
    return out


def de_initial_population(seed: int, m0i: int, S: int, pop: int, lower, upper) -> np.ndarray:
    """[S][pop][np] raw initial individuals of the midpoint whose stream key
    is m0i (de_key(m0))."""
    lo = np.asarray(lower, np.float32)
    hi = np.asarray(upper, np.float32)
    out = np.zeros((S, pop, lo.size), np.float32)
    _de_sigs().oracle_de_initial_population(seed, m0i, S, pop, lo.size, _f(lo), _f(hi), _f(out))
    return out


def select_oct_per_sample(mid, hoff, m0: float, apm: float, h0: float, S: int, dt: float,
                          cands: np.ndarray) -> np.ndarray:
    mid = np.ascontiguousarray(mid, np.float32)
    hoff = np.ascontiguousarray(hoff, np.float32)
    c = np.ascontiguousarray(cands, np.float32)
    mask = np.zeros(mid.size, np.uint8)
    _de_sigs().oracle_select_oct_per_sample(_f(mid), _f(hoff), mid.size, C.c_float(m0),
                                            C.c_float(apm), C.c_float(h0), S, C.c_float(dt),
                                            _f(c), c.shape[1],
                                            mask.ctypes.data_as(C.POINTER(C.c_uint8)))
    return mask.astype(bool)
