"""The OCT displaced-midpoint box test (oct_warp_box, oct_box_may_pass and
oct_box_may_pass_h0 in csrc/hpss_device.cuh) against the per-sample test it
filters for, in an FP32 emulation on the CPU.

The per-sample side restates the reference's displaced-midpoint test
(cuda/include/semblance/kernel/oct/common.cuh:7-35) with the roundings of
oct_cand / oct_trace / oct_mh; the box side restates the kernels' test.  The
property checked is the one the kernels rely on: a trace the box test drops
fails the per-sample test of every member of the box.  Random lines, slopes
1e-8 to 3e-2, sample intervals 0.1 to 8 ms, h0 = 0 and h0 from 1e-3 to
3000 m, half-offsets of both signs and equal to +-h0.  The fused
multiply-adds are emulated in float64 and rounded once (exact for these
magnitudes up to a double rounding well inside the margin).
"""
import numpy as np

f32 = np.float32


def _fma(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64)
            + np.asarray(c, np.float64)).astype(f32)


def _mul(a, b):
    return (np.asarray(a, f32) * np.asarray(b, f32)).astype(f32)


def _add(a, b):
    return (np.asarray(a, f32) + np.asarray(b, f32)).astype(f32)


def _sqrt(x):
    return np.sqrt(np.asarray(x, f32)).astype(f32)


def _div(a, b):
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        return (np.asarray(a, f32) / np.asarray(b, f32)).astype(f32)


def _per_sample_pass(t0, s, c, h, h0, m, m0, apm):
    """[lanes][traces] True where the reference's displaced-midpoint test
    passes (no error and |m - mh| <= apm)."""
    hh = _mul(h, h)
    gs = _mul(_mul(f32(2), _sqrt(_fma(h0, h0, hh))), _mul(f32(2), _sqrt(_fma(h0, h0, hh))))
    p16h = _mul(_mul(_mul(_mul(f32(16), h), h), h0), h0)
    dif = _fma(-h0, h0, hh)
    theta = _mul(t0, s)[:, None]
    ts = _mul(theta, theta)
    tn0 = _fma(t0, t0, -_mul(_mul(c, h0), h0))[:, None]
    tq = _mul(tn0, tn0)
    arg = _fma(tq, tq, _mul(_mul(tq, ts), gs[None]))
    arg = _fma(_mul(p16h[None], ts), ts, arg)
    arg2 = _add(_add(_mul(ts, gs[None]), _mul(f32(2), tq)),
                _mul(f32(2), _sqrt(np.maximum(arg, f32(0)))))
    rc = _div(f32(1), _sqrt(arg2))
    with np.errstate(invalid="ignore", over="ignore"):
        mh = _fma(_mul(_mul(f32(2), theta), dif[None]), rc, np.full(rc.shape, m0, f32))
        return (arg >= 0) & (arg2 != 0) & ~(np.abs(_add(m[None], -mh)) > apm)


def _box_keep(t0, s, c, h, h0, m, m0, apm):
    """Per trace: kept by the warp's box test (or None: the box is off)."""
    if h0 == 0:
        inb = t0 > 0
        if not inb.any():
            return None
        aLo, aHi = t0[inb].min(), t0[inb].max()
        if not (aLo >= f32(1e-4)):
            return None
        sLo = sHi = s
        tHi = aLo if sHi > 0 else aHi
        tLo = aHi if sLo > 0 else aLo
        hh = _mul(h, h)
        gs = _mul(_mul(f32(2), _sqrt(hh)), _mul(f32(2), _sqrt(hh)))
        dif = hh
        hi = _div(_mul(_mul(f32(2), sHi), dif), _add(tHi, _sqrt(_fma(tHi, tHi, _mul(_mul(sHi, sHi), gs)))))
        lo = _div(_mul(_mul(f32(2), sLo), dif), _add(tLo, _sqrt(_fma(tLo, tLo, _mul(_mul(sLo, sLo), gs)))))
    else:
        theta = _mul(t0, s)
        T = _fma(t0, t0, -_mul(_mul(c, h0), h0))
        aLo, aHi, bLo, bHi = theta.min(), theta.max(), T.min(), T.max()
        if bHi < 0:
            bLo, bHi = -bHi, -bLo
        if not (bLo >= f32(1e-8) and bHi >= bLo):
            return None
        ad = np.abs(_fma(-h0, h0, _mul(h, h)))
        hh, hh0 = _mul(h, h), _mul(h0, h0)
        h4, l4 = _mul(f32(4), np.maximum(hh, hh0)), _mul(f32(4), np.minimum(hh, hh0))

        def g(th, T_):
            th2 = _mul(th, th)
            return _div(_mul(_mul(f32(2), th), ad),
                        _add(_sqrt(_fma(T_, T_, _mul(th2, h4))), _sqrt(_fma(T_, T_, _mul(th2, l4)))))
        gHi = g(aHi, bLo if aHi > 0 else bHi)
        gLo = g(aLo, bHi if aLo > 0 else bLo)
        dif = _fma(-h0, h0, _mul(h, h))
        lo = np.where(dif >= 0, gLo, -gHi)
        hi = np.where(dif >= 0, gHi, -gLo)
    marg = (f32(1e-4) * np.maximum(np.abs(lo), np.abs(hi))
            + f32(1e-5) * (abs(m0) + np.abs(m)) + f32(1e-3)).astype(f32)
    return ~((_add(m0, lo) - marg > m + apm) | (_add(m0, hi) + marg < m - apm))


def test_box_test_never_drops_a_passing_trace():
    rng = np.random.default_rng(2024)
    dropped = needed = kept = total = boxes = 0
    for it in range(400):
        dt = f32(10 ** rng.uniform(-4, np.log10(8e-3)))
        S = int(rng.integers(64, 4000))
        tile = int(rng.integers(0, (S + 31) // 32))
        h0 = f32(0) if it % 2 == 0 else f32(rng.choice([rng.uniform(1, 3000),
                                                        rng.uniform(1e-3, 10), 500.0]))
        c = f32(f32(4) / _mul(f32(rng.uniform(1000, 6000)), f32(rng.uniform(1000, 6000))))
        s = f32(0) if it % 7 == 3 else f32(rng.uniform(-1, 1) * 10 ** rng.uniform(-8, -1.5))
        n = 128
        h = rng.uniform(-5000, 5000, n).astype(f32)
        if it % 5 == 0:
            h[:10], h[10:20] = h0, -h0
        m0 = f32(rng.uniform(1, 1e5))
        m = (m0 + rng.uniform(-6000, 6000, n)).astype(f32)
        apm = f32(10 ** rng.uniform(1, 3.3))
        t0 = _mul(np.minimum(np.arange(tile * 32, tile * 32 + 32), S - 1).astype(f32), dt)
        keep = _box_keep(t0, s, c, h, h0, m, m0, apm)
        if keep is None:
            continue
        boxes += 1
        passing = _per_sample_pass(t0, s, c, h, h0, m, m0, apm).any(axis=0)
        dropped += int(np.sum(passing & ~keep))
        needed += int(passing.sum())
        kept += int(keep.sum())
        total += n
    assert boxes > 300
    assert dropped == 0
    # and the test is not vacuous: it keeps little more than what passes
    assert 0 < needed <= kept < needed + 0.05 * total, (needed, kept, total)
