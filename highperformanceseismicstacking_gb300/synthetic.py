"""Seeded synthetic seismic lines with the shapes of the five benchmark workloads.

The reference ships no data (its ``data/*.su`` files are not in the source
tree), so every test and benchmark input is generated here from a fixed seed.
Each line is a set of CMP gathers on a 2-D line along y (azimuth 0, scalco 1,
integer coordinates, midpoints > 0) so the reference geometry
(common/src/model/Utils.cpp:8-52) reproduces midpoints and half-offsets
exactly.

Signal model: reflection events with a Ricker wavelet and hyperbolic moveout
t(m, h) = sqrt(t0(m)^2 + 4 h^2 / v_nmo^2), plus Gaussian noise.  The noise
standard deviation is ``mean event amplitude / snr``.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .su import SU_HEADER_DTYPE


@dataclasses.dataclass
class Line:
    samples: np.ndarray        # [N][S] float32, CMP-major, h ascending
    midpoints: np.ndarray      # [N] float32 (exact)
    halfoffsets: np.ndarray    # [N] float32 (exact)
    headers: np.ndarray        # [N] SU headers
    cdp_midpoints: np.ndarray  # [nCMP] float32, ascending
    dt_us: int
    seed: int

    @property
    def dt(self) -> np.float32:
        return np.float32(np.float32(self.dt_us) * np.float32(1e-6))

    @property
    def samples_per_trace(self) -> int:
        return int(self.samples.shape[1])


def ricker(t: np.ndarray, f: float) -> np.ndarray:
    a = (math.pi * f * t) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def _headers(m: np.ndarray, h: np.ndarray, cdp: np.ndarray, ns: int, dt_us: int) -> np.ndarray:
    n = m.size
    hdr = np.zeros(n, SU_HEADER_DTYPE)
    hdr["tracl"] = np.arange(1, n + 1)
    hdr["tracr"] = np.arange(1, n + 1)
    hdr["cdp"] = cdp
    hdr["offset"] = (2 * h).astype(np.int32)
    hdr["scalco"] = 1
    hdr["sx"] = 0
    hdr["gx"] = 0
    hdr["sy"] = (m - h).astype(np.int32)
    hdr["gy"] = (m + h).astype(np.int32)
    hdr["ns"] = ns
    hdr["dt"] = dt_us
    return hdr


def _add_events(samples: np.ndarray, t_ev: np.ndarray, amp: np.ndarray, dt: float, f: float) -> None:
    """Add one wavelet per trace centred at t_ev[trace] (vectorised over traces)."""
    n, S = samples.shape
    nw = int(math.ceil(1.6 / (f * dt)))
    rows = np.arange(n)
    base = np.floor(t_ev / dt).astype(np.int64)
    for o in range(-nw, nw + 1):
        idx = base + o
        ok = (idx >= 0) & (idx < S) & np.isfinite(t_ev)
        if not ok.any():
            continue
        val = ricker(idx[ok] * dt - t_ev[ok], f) * amp[ok]
        samples[rows[ok], idx[ok]] += val.astype(np.float32)


def _finish(samples, rng, mean_amp, snr):
    sigma = mean_amp / snr
    noise = rng.standard_normal(samples.shape, dtype=np.float32)
    noise *= np.float32(sigma)
    samples += noise


def cmp_line(n_cmp: int, halfoffsets: Sequence[float], ns: int, dt_us: int,
             n_reflectors: int, n_multiples: int, f: float, snr: float,
             seed: int, m_start: int = 1000, dm: int = 25,
             v_top: float = 1500.0, v_bottom: float = 3500.0) -> Line:
    """Flat-reflector CMP line: hyperbolic moveout with v increasing with depth.

    Multiples reuse a primary's moveout with 0.8x its velocity at a later time.
    """
    rng = np.random.default_rng(seed)
    dt = float(np.float32(np.float32(dt_us) * np.float32(1e-6)))
    tmax = ns * dt
    h = np.asarray(halfoffsets, dtype=np.int64)
    fold = h.size
    cm = (m_start + dm * np.arange(n_cmp)).astype(np.int64)
    m = np.repeat(cm, fold)
    hh = np.tile(h, n_cmp)
    N = m.size
    samples = np.zeros((N, ns), np.float32)
    t0s = np.sort(rng.uniform(0.1 * tmax, 0.9 * tmax, n_reflectors))
    vs = v_top + (v_bottom - v_top) * (t0s - t0s.min()) / max(t0s.max() - t0s.min(), 1e-9)
    amps = rng.uniform(0.5, 1.0, n_reflectors)
    events: List[Tuple[float, float, float]] = [(t0s[i], vs[i], amps[i]) for i in range(n_reflectors)]
    for j in range(n_multiples):
        i = int(rng.integers(0, n_reflectors))
        events.append((min(1.6 * t0s[i], 0.95 * tmax), 0.8 * vs[i], 0.6 * amps[i]))
    hf = hh.astype(np.float64)
    for t0, v, a in events:
        t_ev = np.sqrt(t0 * t0 + 4.0 * hf * hf / (v * v))
        _add_events(samples, t_ev, np.full(N, a), dt, f)
    _finish(samples, rng, float(np.mean([e[2] for e in events])), snr)
    hdr = _headers(m, hh, np.repeat(np.arange(1, n_cmp + 1), fold), ns, dt_us)
    return Line(samples, m.astype(np.float32), hh.astype(np.float32), hdr,
                cm.astype(np.float32), dt_us, seed)


def structured_line(n_cmp: int, fold_range: Tuple[int, int], h_max: int, ns: int,
                    dt_us: int, n_reflectors: int, f: float, snr: float, seed: int,
                    v0: float = 1500.0, kz: float = 0.6, kx: float = 0.0,
                    dip_deg: float = 20.0, radius: Tuple[float, float] = (500.0, 5000.0),
                    m_start: int = 1000, dm: int = 25) -> Line:
    """Line of uneven fold with dipping, curved reflectors in v = v0 + kz z + kx x.

    Reflector depth z(x) = z0 + tan(dip) (x - xc) + a cos(2 pi (x - xc) / L),
    with a chosen so the crest curvature radius is ``radius``.  Zero-offset
    time 2 * int dz / v(z); NMO velocity is the RMS velocity of the column.
    """
    rng = np.random.default_rng(seed)
    dt = float(np.float32(np.float32(dt_us) * np.float32(1e-6)))
    tmax = ns * dt
    folds = rng.integers(fold_range[0], fold_range[1] + 1, n_cmp)
    cm = (m_start + dm * np.arange(n_cmp)).astype(np.int64)
    m = np.repeat(cm, folds)
    hh = np.concatenate([np.sort(rng.integers(0, h_max + 1, k)) for k in folds]).astype(np.int64)
    cdp = np.repeat(np.arange(1, n_cmp + 1), folds)
    N = m.size
    samples = np.zeros((N, ns), np.float32)
    x_mid = 0.5 * (cm[0] + cm[-1])
    L = 4000.0
    mf = m.astype(np.float64)
    hf = hh.astype(np.float64)
    amps = rng.uniform(0.5, 1.0, n_reflectors)
    for r in range(n_reflectors):
        dip = math.radians(rng.uniform(-dip_deg, dip_deg))
        R = rng.uniform(*radius)
        a = (L / (2 * math.pi)) ** 2 / R * (1 if rng.random() < 0.5 else -1)
        xc = rng.uniform(cm[0], cm[-1])
        # pick a target zero-offset time, then the depth that gives it at xc
        t_target = rng.uniform(0.12 * tmax, 0.85 * tmax)
        vloc = v0 + kx * xc
        z0 = (math.exp(t_target * kz / 2.0) - 1.0) * vloc / kz
        z = z0 + math.tan(dip) * (mf - xc) * 0.05 + a * np.cos(2 * math.pi * (mf - xc) / L) * 0.05
        z = np.maximum(z, 50.0)
        vtop = v0 + kx * mf
        t0 = (2.0 / kz) * np.log1p(kz * z / vtop)
        vbot = vtop + kz * z
        vrms = np.sqrt((vbot ** 2 - vtop ** 2) / (2.0 * kz * np.maximum(np.log(vbot / vtop), 1e-12)) / 1.0)
        vnmo = vrms / max(math.cos(dip), 0.3)
        t_ev = np.sqrt(t0 * t0 + 4.0 * hf * hf / (vnmo * vnmo))
        _add_events(samples, t_ev, np.full(N, amps[r]), dt, f)
    _finish(samples, rng, float(np.mean(amps)), snr)
    hdr = _headers(m, hh, cdp, ns, dt_us)
    return Line(samples, m.astype(np.float32), hh.astype(np.float32), hdr,
                cm.astype(np.float32), dt_us, seed)


# ---------------------------------------------------------------------------
# Workloads: the five benchmark configurations, expressed as reference CLI
# settings (lower/upper bounds, granularity, tau, apm, ...).
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Workload:
    name: str
    model: str                      # "cmp" | "zocrs" | "oct"
    algorithm: str                  # "linear-search" | "de" | "stretch-free"
    lower: List[float]
    upper: List[float]
    granularity: Optional[List[int]]
    tau: float
    apm: float
    aph: float
    h0: float = 0.0
    v0: float = 0.0
    ain: float = 0.0
    bpctg: float = 0.0
    population: int = 0
    generations: int = 0
    de_f: float = 0.85
    de_cr: float = 0.5
    line_args: dict = dataclasses.field(default_factory=dict)
    line_kind: str = "cmp"

    def make_line(self, seed: Optional[int] = None, n_cmp: Optional[int] = None) -> Line:
        args = dict(self.line_args)
        if seed is not None:
            args["seed"] = seed
        if n_cmp is not None:
            args["n_cmp"] = n_cmp
        if self.line_kind == "cmp":
            return cmp_line(**args)
        return structured_line(**args)


def zocrs_bounds(v_lower: float, v0: float, ain: float, bpctg: float):
    """TraveltimeBuilder::buildZeroOffsetCommonReflectionSurface
    (common/src/traveltime/TraveltimeBuilder.cpp:45-76): A and B bounds are
    derived, A_max = 2 sin(ain)/v0 and B_max = bpctg * 4 / vmin^2, in float32."""
    f32 = np.float32
    ain_rad = f32(f32(ain) * f32(math.pi)) / f32(180.0)
    a_max = f32(f32(2.0) * f32(math.sin(float(ain_rad)))) / f32(v0)
    b_max = f32(f32(bpctg) * f32(4)) / f32(f32(v_lower) * f32(v_lower))
    return float(a_max), float(b_max)


WORKLOADS = {
    # C1: CMP linear search, small 2-D line.
    "cmp-small": Workload(
        name="cmp-small", model="cmp", algorithm="linear-search",
        lower=[1000.0], upper=[5040.0], granularity=[101],
        tau=0.010, apm=0.0, aph=2000.0,
        line_args=dict(n_cmp=50, halfoffsets=list(range(25, 1176, 50)), ns=1000,
                       dt_us=4000, n_reflectors=5, n_multiples=0, f=25.0, snr=10.0,
                       seed=1001)),
    # C2: CMP linear search at production size (bench workload).
    "cmp-production": Workload(
        name="cmp-production", model="cmp", algorithm="linear-search",
        lower=[1000.0], upper=[6012.5], granularity=[401],
        tau=0.007, apm=0.0, aph=4000.0,
        line_args=dict(n_cmp=2000, halfoffsets=list(range(0, 2951, 50)), ns=2000,
                       dt_us=2000, n_reflectors=12, n_multiples=3, f=25.0, snr=10.0,
                       seed=1002)),
    # C3: ZO-CRS linear search over uneven fold, +-15 CMP aperture.
    "zocrs-ls": Workload(
        name="zocrs-ls", model="zocrs", algorithm="linear-search",
        lower=[1414.2136], upper=[6324.5553], granularity=[41, 21, 21],
        tau=0.010, apm=375.0, aph=4000.0, v0=2000.0, ain=90.0, bpctg=0.05,
        line_kind="structured",
        line_args=dict(n_cmp=1000, fold_range=(30, 90), h_max=2000, ns=1500,
                       dt_us=4000, n_reflectors=8, f=20.0, snr=5.0, seed=1003)),
    # C4: ZO-CRS differential evolution.
    "zocrs-de": Workload(
        name="zocrs-de", model="zocrs", algorithm="de",
        lower=[1414.2136], upper=[6324.5553], granularity=None,
        tau=0.010, apm=375.0, aph=4000.0, v0=2000.0, ain=90.0, bpctg=0.05,
        population=32, generations=60, de_f=0.5, de_cr=0.9,
        line_kind="structured",
        line_args=dict(n_cmp=500, fold_range=(30, 90), h_max=2000, ns=1500,
                       dt_us=4000, n_reflectors=8, f=20.0, snr=5.0, seed=1004)),
    # C5: OCT differential evolution (+ stretch-free stack afterwards).
    "oct-de": Workload(
        name="oct-de", model="oct", algorithm="de",
        lower=[1200.0, -1e-3], upper=[5000.0, 1e-3], granularity=None,
        tau=0.009, apm=375.0, aph=4000.0, h0=0.0,
        population=48, generations=80, de_f=0.5, de_cr=0.9,
        line_kind="structured",
        line_args=dict(n_cmp=800, fold_range=(40, 120), h_max=3000, ns=3000,
                       dt_us=2000, n_reflectors=10, f=30.0, snr=8.0, seed=1005,
                       v0=1800.0, kz=0.5, kx=0.1)),
}


def workload_bounds(w: Workload):
    """Lower/upper bounds of every model parameter as the reference builds them."""
    if w.model == "zocrs":
        a, b = zocrs_bounds(w.lower[0], w.v0, w.ain, w.bpctg)
        return [w.lower[0], -a, -b], [w.upper[0], a, b]
    return list(w.lower), list(w.upper)
