"""SU (Seismic Unix) trace files and the gather model of the reference.

The 240-byte trace header is the reference's ``trace_info_t``
(common/include/model/Trace.hpp:9-91): native byte order, naturally aligned
C struct, followed by ``ns`` float32 samples.  The layout is a file format,
so it is reproduced field for field.

``read_gather`` restates ``Gather::readGatherFromFile``
(common/src/model/Gather.cpp:49-126), ``Trace::read`` (Trace.cpp:45-61) and the
geometry of ``Utils::midpoint/halfoffset`` (common/src/model/Utils.cpp:8-52) in
float32 arithmetic with the same operation order, so the midpoints, half
offsets, window size and CDP map are bit-identical to the reference's.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional

import numpy as np

SU_HEADER_FIELDS = [
    ("tracl", "<i4"), ("tracr", "<i4"), ("fldr", "<i4"), ("tracf", "<i4"),
    ("ep", "<i4"), ("cdp", "<i4"), ("cdpt", "<i4"), ("trid", "<i2"),
    ("nvs", "<i2"), ("nhs", "<i2"), ("duse", "<i2"), ("offset", "<i4"),
    ("gelev", "<i4"), ("selev", "<i4"), ("sdepth", "<i4"), ("gdel", "<i4"),
    ("sdel", "<i4"), ("swdep", "<i4"), ("gwdep", "<i4"), ("scalel", "<i2"),
    ("scalco", "<i2"), ("sx", "<i4"), ("sy", "<i4"), ("gx", "<i4"),
    ("gy", "<i4"), ("counit", "<i2"), ("wevel", "<i2"), ("swevel", "<i2"),
    ("sut", "<i2"), ("gut", "<i2"), ("sstat", "<i2"), ("gstat", "<i2"),
    ("tstat", "<i2"), ("laga", "<i2"), ("lagb", "<i2"), ("delrt", "<i2"),
    ("muts", "<i2"), ("mute", "<i2"), ("ns", "<u2"), ("dt", "<u2"),
    ("gain", "<i2"), ("igc", "<i2"), ("igi", "<i2"), ("corr", "<i2"),
    ("sfs", "<i2"), ("sfe", "<i2"), ("slen", "<i2"), ("styp", "<i2"),
    ("stas", "<i2"), ("stae", "<i2"), ("tatyp", "<i2"), ("afilf", "<i2"),
    ("afils", "<i2"), ("nofilf", "<i2"), ("nofils", "<i2"), ("lcf", "<i2"),
    ("hcf", "<i2"), ("lcs", "<i2"), ("hcs", "<i2"), ("year", "<i2"),
    ("day", "<i2"), ("hour", "<i2"), ("minute", "<i2"), ("sec", "<i2"),
    ("timbas", "<i2"), ("trwf", "<i2"), ("grnors", "<i2"), ("grnofr", "<i2"),
    ("grnlof", "<i2"), ("gaps", "<i2"), ("otrav", "<i2"), ("d1", "<f4"),
    ("f1", "<f4"), ("d2", "<f4"), ("f2", "<f4"), ("ungpow", "<f4"),
    ("unscale", "<f4"), ("ntr", "<i4"), ("mark", "<i2"), ("shortpad", "<i2"),
    ("unass", "<i2", (14,)),
]
SU_HEADER_DTYPE = np.dtype(SU_HEADER_FIELDS)
assert SU_HEADER_DTYPE.itemsize == 240

MICRO2SECONDS = np.float32(1e-6)


def _f32(x) -> np.float32:
    return np.float32(x)


def fscalco(scalco: np.ndarray) -> np.ndarray:
    """Coordinate scale (Utils.cpp:9-10): scalco >= 0 multiplies, < 0 divides."""
    sc = scalco.astype(np.float32)
    with np.errstate(divide="ignore"):
        neg = np.float32(-1.0) / sc
    return np.where(scalco >= 0, sc, neg).astype(np.float32)


def _axis_values(hdr: np.ndarray, plus: bool):
    fs = fscalco(hdr["scalco"])
    half = np.float32(0.5)
    if plus:
        ix = (hdr["gx"].astype(np.int32) + hdr["sx"].astype(np.int32))
        iy = (hdr["gy"].astype(np.int32) + hdr["sy"].astype(np.int32))
    else:
        ix = (hdr["gx"].astype(np.int32) - hdr["sx"].astype(np.int32))
        iy = (hdr["gy"].astype(np.int32) - hdr["sy"].astype(np.int32))
    vx = (fs * ix.astype(np.float32)) * half
    vy = (fs * iy.astype(np.float32)) * half
    return vx.astype(np.float32), vy.astype(np.float32)


def azimuth_rad(az_deg: float) -> np.float32:
    """Utils::degreesToRad (Utils.cpp:54-56) in float32."""
    return np.float32(np.float32(az_deg) * np.float32(math.pi)) / np.float32(180.0)


def midpoint_halfoffset(hdr: np.ndarray, az_rad: np.float32):
    """Utils::midpoint / Utils::halfoffset (Utils.cpp:40-52).

    Azimuth 0 gives sin = 0 and cos = 1 exactly, so the value is the y-axis
    coordinate bit for bit; other azimuths depend on the libm's sinf/cosf.
    """
    s = np.float32(math.sin(float(az_rad)))
    c = np.float32(math.cos(float(az_rad)))
    mx, my = _axis_values(hdr, True)
    hx, hy = _axis_values(hdr, False)
    m = (mx * s + my * c).astype(np.float32)
    h = (hx * s + hy * c).astype(np.float32)
    return m, h


def read_su(path: str):
    """Raw SU read: headers [N] and samples [N][ns] (all traces must share ns)."""
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size == 0:
        return np.zeros(0, SU_HEADER_DTYPE), np.zeros((0, 0), np.float32)
    hdr0 = np.frombuffer(raw[:240].tobytes(), SU_HEADER_DTYPE)[0]
    ns = int(hdr0["ns"])
    rec = 240 + 4 * ns
    if raw.size % rec != 0:
        raise RuntimeError("end of file reached before reading all samples.")
    n = raw.size // rec
    rows = raw.reshape(n, rec)
    hdr = np.frombuffer(rows[:, :240].copy().tobytes(), SU_HEADER_DTYPE)
    if np.any(hdr["ns"] != ns):
        raise ValueError("mixed ns: use read_gather for reference semantics")
    samples = np.frombuffer(rows[:, 240:].copy().tobytes(), np.float32).reshape(n, ns)
    return hdr.copy(), samples.copy()


def write_su(path: str, headers: np.ndarray, samples: np.ndarray) -> None:
    """Write headers [N] + samples [N][ns] as one SU file (Dumper.cpp:96-110)."""
    samples = np.ascontiguousarray(samples, dtype=np.float32)
    n, ns = samples.shape
    rec = np.zeros((n, 240 + 4 * ns), np.uint8)
    rec[:, :240] = np.frombuffer(headers.astype(SU_HEADER_DTYPE).tobytes(), np.uint8).reshape(n, 240)
    rec[:, 240:] = samples.view(np.uint8).reshape(n, 4 * ns)
    rec.tofile(path)


@dataclasses.dataclass
class Cdp:
    midpoint: float
    info: np.void
    trace_count: int = 0
    sample_count: int = 0


@dataclasses.dataclass
class Gather:
    """The reference's ``Gather`` after ``readGatherFromFile``.

    Traces are sorted by (midpoint, half-offset) as ``std::sort`` with
    ``Trace::operator<`` (Trace.cpp:63-74); equal keys keep file order here
    (the reference's order for equal keys is unspecified).
    """
    samples: np.ndarray          # [N][S] float32, sorted
    midpoints: np.ndarray        # [N] float32
    halfoffsets: np.ndarray      # [N] float32
    headers: np.ndarray          # [N] trace_info_t, sorted
    cdps: Dict[float, Cdp]       # ordered by midpoint ascending (std::map)
    samples_per_trace: int
    dt_us: int
    dt: np.float32               # seconds, float(dt) * 1e-6f
    tau: np.float32
    tau_index: int
    window_size: int
    apm: np.float32
    aph: np.float32
    azimuth_rad: np.float32

    @property
    def trace_count(self) -> int:
        return int(self.samples.shape[0])

    def cdp_midpoints(self) -> List[float]:
        return sorted(self.cdps.keys())


def _cdp_info(hdr: np.void) -> np.void:
    """CDP header as Gather.cpp:89-92 builds it from the CDP's first trace."""
    info = hdr.copy()
    info["offset"] = 0
    x = (int(info["sx"]) + int(info["gx"])) >> 1
    y = (int(info["sy"]) + int(info["gy"])) >> 1
    info["sx"] = info["gx"] = x
    info["sy"] = info["gy"] = y
    return info


def tau_index(tau: float, dt: np.float32) -> int:
    """tauIndexDisplacement = (int)(tau / dtInSeconds) (Gather.cpp:75)."""
    return int(np.float32(tau) / np.float32(dt))


def read_gather(path: str, *, aph: float, apm: float, tau: float,
                azimuth_deg: float = 0.0, lowest_midpoint: Optional[float] = None,
                biggest_midpoint: Optional[float] = None,
                emulate_eof_cdp: bool = True) -> Gather:
    """``Gather::readGatherFromFile`` with the reference's filters.

    * traces with a different ``ns`` than the first are dropped;
    * traces with |h| > aph are dropped (the CDP entry is still created);
    * midpoints outside [lowest, biggest] are dropped; the default lowest
      is FLT_MIN, so midpoints <= 0 are dropped;
    * ``emulate_eof_cdp``: the reference's ``while (!eof)`` loop runs once
      more after the last trace and inserts a CDP at midpoint 0 with an
      uninitialised header; it is emulated with a zeroed header.
    """
    raw = np.fromfile(path, dtype=np.uint8)
    az = azimuth_rad(azimuth_deg)
    lo = np.float32(np.finfo(np.float32).tiny if lowest_midpoint is None else lowest_midpoint)
    hi = np.float32(np.finfo(np.float32).max if biggest_midpoint is None else biggest_midpoint)
    cdps: Dict[float, Cdp] = {}
    spt = 0
    dt_us = 0
    uniform = False
    if raw.size >= 240:
        hdr0 = np.frombuffer(raw[:240].tobytes(), SU_HEADER_DTYPE)[0]
        rec = 240 + 4 * int(hdr0["ns"])
        if raw.size % rec == 0:
            rows = raw.reshape(-1, rec)
            all_hdr = np.frombuffer(rows[:, :240].copy().tobytes(), SU_HEADER_DTYPE).copy()
            uniform = bool(np.all(all_hdr["ns"] == hdr0["ns"]))
    if uniform:
        spt = int(hdr0["ns"])
        dt_us = int(hdr0["dt"])
        m_all, h_all = midpoint_halfoffset(all_hdr, az)
        _, first = np.unique(m_all, return_index=True)
        for i in sorted(first.tolist()):
            key = float(m_all[i])
            cdps[key] = Cdp(key, _cdp_info(all_hdr[i]))
        keep = ~(np.abs(h_all) > np.float32(aph)) & (m_all >= lo) & (m_all <= hi)
        keep_idx = np.nonzero(keep)[0]
        headers = all_hdr[keep_idx]
        samples = np.frombuffer(rows[keep_idx, 240:].tobytes(), np.float32).reshape(-1, spt).copy()
        uniq, counts = np.unique(m_all[keep_idx], return_counts=True)
        for k, c in zip(uniq.tolist(), counts.tolist()):
            cdps[float(k)].trace_count = int(c)
            cdps[float(k)].sample_count = int(c) * spt
    else:
        keep_hdr, keep_smp = [], []
        pos = 0
        while pos < raw.size:
            if raw.size - pos < 240:
                break
            hdr = np.frombuffer(raw[pos:pos + 240].tobytes(), SU_HEADER_DTYPE).copy()
            ns = int(hdr["ns"][0])
            if raw.size - (pos + 240) < 4 * ns:
                raise RuntimeError("end of file reached before reading all samples.")
            smp = np.frombuffer(raw[pos + 240:pos + 240 + 4 * ns].tobytes(), np.float32).copy()
            pos += 240 + 4 * ns
            m, h = midpoint_halfoffset(hdr, az)
            m, h = m[0], h[0]
            if spt == 0:
                spt = ns
                dt_us = int(hdr["dt"][0])
            key = float(m)
            if key not in cdps:
                cdps[key] = Cdp(key, _cdp_info(hdr[0]))
            if ns != spt:
                continue
            if abs(h) > np.float32(aph):
                continue
            if not (m >= lo and m <= hi):
                continue
            keep_hdr.append(hdr)
            keep_smp.append(smp)
            cdps[key].trace_count += 1
            cdps[key].sample_count += ns
        if keep_hdr:
            headers = np.concatenate(keep_hdr)
            samples = np.stack(keep_smp).astype(np.float32)
        else:
            headers = np.zeros(0, SU_HEADER_DTYPE)
            samples = np.zeros((0, spt), np.float32)
    if emulate_eof_cdp and 0.0 not in cdps:
        cdps[0.0] = Cdp(0.0, np.zeros(1, SU_HEADER_DTYPE)[0])
    m, h = midpoint_halfoffset(headers, az)
    order = np.lexsort((h, m))
    dt = np.float32(np.float32(dt_us) * MICRO2SECONDS)
    ti = tau_index(tau, dt) if dt_us else 0
    cdps_sorted = {k: cdps[k] for k in sorted(cdps)}
    return Gather(samples=np.ascontiguousarray(samples[order]), midpoints=m[order],
                  halfoffsets=h[order], headers=headers[order], cdps=cdps_sorted,
                  samples_per_trace=spt, dt_us=dt_us, dt=dt, tau=np.float32(tau),
                  tau_index=ti, window_size=2 * ti + 1, apm=np.float32(apm),
                  aph=np.float32(aph), azimuth_rad=az)


def gather_from_arrays(samples: np.ndarray, headers: np.ndarray, *, aph: float,
                       apm: float, tau: float, azimuth_deg: float = 0.0,
                       emulate_eof_cdp: bool = False) -> Gather:
    """Same as ``read_gather`` for in-memory arrays (no file round trip)."""
    import os
    import tempfile
    fd, p = tempfile.mkstemp(suffix=".su")
    os.close(fd)
    try:
        write_su(p, headers, samples)
        return read_gather(p, aph=aph, apm=apm, tau=tau, azimuth_deg=azimuth_deg,
                           emulate_eof_cdp=emulate_eof_cdp)
    finally:
        os.unlink(p)
