"""The Courant kernel's FP32 filter, emulated on the CPU (numpy float32 with
one rounding per operation, as the kernel's non-contracted FP32 code; a
fused multiply-add on the GPU only rounds less).

The kernel (magic_gb300/csrc/courant.cu) skips a point when its FP32
estimate a of a Courant term is below (1 - 2^-13) M - 2^-49, M the largest
finite estimate seen; that is safe when |a - e| <= 2^-16 e + 2^-50 for the
FP64 term e of every point with a finite estimate.  These tests check that
bound on wide-range, near-tie and tiny inputs, and that a sequential run of
the filter returns the exact maximum of the terms (courant.f90:193-276,
evaluated like the oracle: one rounding per operation)."""
import numpy as np
import pytest

ETA, TAU = 2.0 ** -16, 2.0 ** -50


def hi_abs_f32(x):
    """|x| as float32 from the high word of x: mantissa truncated to 20 bits,
    below 2^-126 at most 2^-126, from 2^128 (and Inf / NaN) +Inf."""
    m = ((np.asarray(x, dtype=np.float64).view(np.uint64) >> np.uint64(32)) & np.uint64(0x7FFFFFFF)).astype(np.int64)
    m = np.clip(m, 0x38000000, 0x47F00000)
    return ((m - 0x38000000) << 3).astype(np.uint32).view(np.float32)


def constants(courfac, alffac, LFfac, opm, orho1, orho2, or2, or4, delxr2, delxh2, damp=True):
    cf2, af2 = courfac * courfac, alffac * alffac
    valri2 = valhi2 = 0.0
    if damp:
        h = 0.5 * (1.0 + opm)
        valri2, valhi2 = h * h / delxr2, h * h / delxh2
    f = np.float32
    return dict(cf2=cf2, af2=af2, LFfac=LFfac, orho1=orho1, orho2=orho2, o2=or2, o4=or4, valri2=valri2,
                valhi2=valhi2, A1=f(or4 * cf2 * orho2), A2=f(or4 * af2), B1=f(or2 * cf2 * orho2), B2=f(or2 * af2),
                KV=f(LFfac * orho1), RI=f(valri2), HI=f(valhi2))


def exact(c, vr, vt, vp, br, bt, bp, os2):
    """The two terms in FP64, one rounding per operation (the kernel's exact path)."""
    with np.errstate(all="ignore"):
        vflr2 = c["orho2"] * vr * vr
        valr = br * br * c["LFfac"] * c["orho1"]
        valr2 = valr * valr / (valr + c["valri2"])
        er = c["o4"] * (c["cf2"] * vflr2 + c["af2"] * valr2)
        vflh2 = (vt * vt + vp * vp) * os2 * c["orho2"]
        valh2 = (bt * bt + bp * bp) * c["LFfac"] * os2 * c["orho1"]
        valh2m = valh2 * valh2 / (valh2 + c["valhi2"])
        eh = c["o2"] * (c["cf2"] * vflh2 + c["af2"] * valh2m)
    return er, eh


def estimate(c, vr, vt, vp, br, bt, bp, os2):
    """The kernel's FP32 estimates (approx_r / approx_h)."""
    f = [hi_abs_f32(x) for x in (vr, vt, vp, br, bt, bp, os2)]
    vr, vt, vp, br, bt, bp, s = f
    with np.errstate(all="ignore"):
        v = c["KV"] * (br * br)
        ar = c["A1"] * (vr * vr) + c["A2"] * (v * (v / (v + c["RI"])))
        w = c["KV"] * (s * (bt * bt + bp * bp))
        ah = c["B1"] * (s * (vt * vt + vp * vp)) + c["B2"] * (w * (w / (w + c["HI"])))
    return ar.astype(np.float64), ah.astype(np.float64), s <= np.float32(2.0 ** 24)


def inputs(kind, n, rng):
    if kind == "normal":
        x = [rng.standard_normal(n) for _ in range(6)]
    elif kind == "wide":
        x = [rng.standard_normal(n) * np.exp(rng.standard_normal(n) * 20.0) for _ in range(6)]
    elif kind == "ties":
        x = [np.sign(rng.standard_normal(n)) * (1.0 + 1e-12 * rng.standard_normal(n)) for _ in range(6)]
    elif kind == "tiny":
        x = [1e-30 * rng.standard_normal(n) for _ in range(6)]
    else:  # "mixed": tiny B beside unit velocities, some exact zeros
        x = [rng.standard_normal(n) for _ in range(3)] + [1e-25 * rng.standard_normal(n) for _ in range(3)]
        x[3][::7] = 0.0
    os2 = 1.0 / np.sin(rng.uniform(0.005, np.pi / 2, n)) ** 2
    return x, os2


CASES = [dict(courfac=2.5, alffac=1.0, LFfac=1.3, opm=0.7, orho1=1.1, orho2=1.2, or2=0.6, or4=0.36,
              delxr2=1e-3, delxh2=2e-2),
         dict(courfac=2.5, alffac=1.0, LFfac=1e5, opm=1.0, orho1=1.0, orho2=1.0, or2=3.4, or4=11.6,
              delxr2=4e-6, delxh2=1e-4),
         dict(courfac=1.0, alffac=0.0, LFfac=1.0, opm=1.0, orho1=1.0, orho2=1.0, or2=1.0, or4=1.0,
              delxr2=1e-2, delxh2=1e-2)]


@pytest.mark.parametrize("kind", ["normal", "wide", "ties", "tiny", "mixed"])
@pytest.mark.parametrize("ci", range(len(CASES)))
@pytest.mark.parametrize("damp", [True, False])
def test_estimate_error_bound(kind, ci, damp):
    rng = np.random.default_rng(100 + ci)
    c = constants(damp=damp, **CASES[ci])
    (vr, vt, vp, br, bt, bp), os2 = inputs(kind, 200_000, rng)
    er, eh = exact(c, vr, vt, vp, br, bt, bp, os2)
    ar, ah, s_ok = estimate(c, vr, vt, vp, br, bt, bp, os2)
    for a, e, ok in ((ar, er, np.ones_like(s_ok)), (ah, eh, s_ok)):
        fin = np.isfinite(a) & ok
        # a finite estimate implies a finite exact term (0/0 gives NaN in both)
        assert np.all(np.isfinite(e[fin]))
        err = np.abs(a[fin] - e[fin])
        assert np.all(err <= ETA * e[fin] + TAU), float(np.max(err / (ETA * e[fin] + TAU)))


def filtered_max(a, e):
    """The kernel's filter run over the points in order: a point is evaluated
    exactly unless its estimate is below (1 - 2^-13) M - 2^-49."""
    kfac, tau2 = 1.0 - 2.0 ** -13, 2.0 ** -49
    M, best, evaluated = 0.0, 0.0, 0
    for ai, ei in zip(a, e):
        if np.isfinite(ai):
            M = max(M, ai)
        if not (ai < kfac * M - tau2):
            evaluated += 1
            if ei == ei:  # NaN terms do not enter the maximum
                best = max(best, ei)
    return best, evaluated


@pytest.mark.parametrize("kind", ["normal", "wide", "ties", "tiny", "mixed"])
def test_filter_keeps_the_exact_maximum(kind):
    rng = np.random.default_rng(7)
    c = constants(**CASES[0])
    (vr, vt, vp, br, bt, bp), os2 = inputs(kind, 20_000, rng)
    er, eh = exact(c, vr, vt, vp, br, bt, bp, os2)
    ar, ah, _ = estimate(c, vr, vt, vp, br, bt, bp, os2)
    for a, e in ((ar, er), (ah, eh)):
        got, evaluated = filtered_max(a, e)
        assert got == np.fmax.reduce(np.fmax(e, 0.0))
        if kind == "normal":
            assert evaluated < 0.01 * len(e)  # the filter does skip almost every point
        # ("wide" evaluates its beyond-FP32 points exactly: a few percent)
