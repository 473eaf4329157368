"""Known answers of the oracle's restatements of the radial-loop pieces that
have closed forms (no GPU)."""
import numpy as np
import pytest

from oracle import oracle as orc


@pytest.mark.parametrize("N,P", [(48, 96), (96, 192)])
@pytest.mark.parametrize("LFfac", [1.0, 2.5])
def test_lorentz_torque_known_answers(N, P, LFfac):
    """get_lorentz_torque (outRot.f90:423-483) is LFfac 2 pi / n_phi times a
    Gauss-quadrature sum over the sphere: for br = bp = 1 it is
    LFfac 2 pi * 2, for br = bp = cos(theta) LFfac 2 pi * 2/3, and the Grenoble
    term -b0 cos(theta) bp with bp = cos(theta) adds -b0 LFfac 2 pi * 2/3
    (the quadrature is exact for these polynomials)."""
    _, c = orc._row_trig(N)
    one = np.ones((P, N))
    cg = np.broadcast_to(c, (P, N))
    assert abs(orc.lorentz_torque(one, one, N, LFfac) - LFfac * 4.0 * np.pi) < 1e-12
    assert abs(orc.lorentz_torque(cg, cg, N, LFfac) - LFfac * 4.0 * np.pi / 3.0) < 1e-12
    b0 = 0.7
    got = orc.lorentz_torque(np.zeros((P, N)), cg, N, LFfac, b0)
    assert abs(got + b0 * LFfac * 4.0 * np.pi / 3.0) < 1e-12
    # only the phi average of br bp matters: a cos(phi) modulation of bp integrates to 0
    phi = 2.0 * np.pi * np.arange(P) / P
    assert abs(orc.lorentz_torque(one, np.cos(phi)[:, None] * one, N, LFfac)) < 1e-12


def test_get_nl_full_default_equals_boussinesq_restatement():
    """The restatement with the reference's switches, at the Boussinesq
    default (curl-form advection, Lorentz force, entropy advection, induction,
    unit constants), equals the single-configuration restatement on Adv, VS
    and VxB."""
    import numpy as np
    from oracle import oracle
    n, N, P = 3, 24, 48
    rng = np.random.default_rng(5)
    names = ("vrc", "vtc", "vpc", "cvrc", "cvtc", "cvpc", "brc", "btc", "bpc", "cbrc", "cbtc", "cbpc", "sc")
    g = {k: rng.standard_normal((n, P, N)) for k in names}
    r = np.array([1.4, 1.0, 0.6])
    a = oracle.get_nl(g, 1.0 / r ** 2, N)
    b = oracle.get_nl_full(g, N, r)
    for k in ("Advr", "Advt", "Advp", "VSr", "VSt", "VSp", "VxBr", "VxBt", "VxBp"):
        assert np.allclose(a[k], b[k], rtol=1e-14, atol=1e-14), k
    assert np.isnan(b["VXir"]).all() and np.isnan(b["heatTerms"]).all()


def test_get_td_full_default_equals_single_configuration_restatement():
    """The get_td restatement with the reference's switches, at the default
    (single curl, Coriolis force, advection, induction, Boussinesq), equals the
    single-configuration restatement wherever both set an output, and leaves
    dpdt at l = 0 unset as get_dpdt does (get_td.f90:333-345)."""
    import numpy as np
    from oracle import oracle
    from magic_gb300.workload import spectra
    L, n = 20, 3
    names = ("w", "dw", "z", "AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "VxBrLM", "VxBtLM", "VxBpLM")
    spec = {k: spectra(L, 1, n, seed=3 + i) for i, k in enumerate(names)}
    r = np.array([1.4, 1.0, 0.6])
    lcut = np.array([20, 17, 20])
    a = oracle.get_td(spec, r, 900.0, L, 1, lcut=lcut, epsc=np.array([0.1, 0.2, 0.3]), nbc=np.array([0, 0, 2]))
    b = oracle.get_td_full(spec, r, 900.0, L, 1, lcut=lcut, epsc=np.array([0.1, 0.2, 0.3]), nbc=np.array([0, 0, 2]),
                           outputs=("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM"))
    for k in ("dwdt", "dzdt", "dsdt", "dbdt", "djdt", "dVxBhLM"):
        for i in range(n):
            if np.isnan(a[k][i]).all():
                continue
            assert np.allclose(a[k][i], b[k][i], rtol=1e-14, atol=1e-14), (k, i)
    assert np.isnan(b["dpdt"][0][0]) and np.allclose(a["dpdt"][0][1:], b["dpdt"][0][1:], rtol=1e-14, atol=1e-14)
