"""Pieces of the radial loop around the transforms: the Courant condition
(courant.f90: the GPU reduction and the host time-step rule) and the
boundary pieces of nonlinear_bcs.f90, against their numpy restatements in
the oracle."""
import numpy as np
import pytest

from test_gpu_parity import built, torch, make  # noqa: F401  (fixtures)


@pytest.mark.parametrize("case", [
    (np.array([0.3, 0.2, 0.5]), np.array([0.4, 0.9, 0.25]), 0.05, 0.1),   # 2 dt < dtMin: grow
    (np.array([0.3, 0.2, 0.5]), np.array([0.4, 0.9, 0.25]), 0.21, 1.0),   # dt > dtMin: shrink
    (np.array([0.3, 0.2, 0.5]), np.array([0.4, 0.9, 0.25]), 2.0, 1.0),    # dt > dtMax
    (np.array([0.3, 0.2, 0.5]), np.array([0.4, 0.9, 0.25]), 0.15, 1.0),   # keep
    (np.array([1e10] * 4), np.array([1e10] * 4), 1e-4, 1e-3),             # no flow: dt_2 = dtMax
    (np.array([]), np.array([]), 1e-3, 1e-3),                             # no levels
])
def test_dt_courant_matches_oracle(case):
    from oracle import oracle as orc
    from magic_gb300 import dt_courant
    dtr, dth, dt, dtmax = case
    assert dt_courant(dtr, dth, dt, dtmax) == orc.dt_courant(dtr, dth, dt, dtmax)


def _grids(torch, s, n, rng, zero_level=None):
    shape = (n, s.n_phi_max, s.nlat_padded)
    g = {k: torch.from_numpy(rng.standard_normal(shape)).cuda() for k in ("vrc", "vtc", "vpc", "brc", "btc", "bpc")}
    if zero_level is not None:
        for k in g:
            g[k][zero_level].zero_()
    return g


def _radial(n, rng):
    r = np.linspace(0.6, 1.5, n)
    return {"orho1": 1.0 + 0.1 * rng.random(n), "orho2": 1.0 + 0.2 * rng.random(n), "or2": 1.0 / r ** 2,
            "or4": 1.0 / r ** 4, "delxr2": 1e-3 * (1.0 + rng.random(n)), "delxh2": 1e-2 * (1.0 + rng.random(n))}


@pytest.mark.gpu
@pytest.mark.parametrize("grid", [(63, 1, 96, 192), (64, 4, 96, 48), (255, 1, 384, 768)])
@pytest.mark.parametrize("mag,damp", [(True, True), (True, False), (False, False)])
def test_courant_matches_oracle(built, torch, grid, mag, damp):
    """Per-level Courant steps on the GPU against the numpy restatement (FP64,
    products rounded in the reference's order: only the two 1/sin^2 tables
    differ, so the tolerance is 1e-13 relative).  Level 2 is all zero and must
    keep its start values."""
    from oracle import oracle as orc
    L, minc, N, P = grid
    s = make(L, minc, N, P)
    n = 5
    rng = np.random.default_rng(21)
    g = _grids(torch, s, n, rng, zero_level=2)
    if not mag:
        for k in ("brc", "btc", "bpc"):
            g[k] = None
    rad = _radial(n, rng)
    start_r = np.array([1e10, 1e10, 1e10, 1e-6, 1e10])  # level 3 starts below its Courant step
    start_h = np.full(n, 1e10)
    got_r, got_h = s.courant({k: v for k, v in g.items() if v is not None}, rad, courfac=2.5, alffac=1.0,
                             LFfac=1.3, opm=0.7, alf_damp=damp, dtrkc=start_r, dthkc=start_h)
    host = {k: (None if v is None else v.cpu().numpy()) for k, v in g.items()}
    exp_r, exp_h = orc.courant(host, rad, N, courfac=2.5, alffac=1.0, LFfac=1.3, opm=0.7, alf_damp=damp,
                               dtrkc=start_r, dthkc=start_h)
    np.testing.assert_allclose(got_r, exp_r, rtol=1e-13, atol=0)
    np.testing.assert_allclose(got_h, exp_h, rtol=1e-13, atol=0)
    assert got_r[2] == 1e10 and got_h[2] == 1e10      # zero level keeps its values
    assert got_r[3] == 1e-6                           # min with the start value
    s.device_status()  # raises if a device wait gave up


GRIDS = [(63, 1, 96, 192), (64, 4, 96, 48)]


@pytest.mark.gpu
@pytest.mark.parametrize("grid", GRIDS)
@pytest.mark.parametrize("keep_vr,deriv", [(False, True), (True, False)])
def test_v_rigid_boundary_matches_oracle(built, torch, grid, keep_vr, deriv):
    from oracle import oracle as orc
    L, minc, N, P = grid
    s = make(L, minc, N, P)
    rng = np.random.default_rng(4)
    names = ["vr", "vt", "vp"] + (["cvr", "dvrdt", "dvrdp", "dvtdp", "dvpdp"] if deriv else [])
    host = {k: rng.standard_normal((s.n_phi_max, s.nlat_padded)) for k in names}
    vr0 = host["vr"].copy()
    dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
    s.v_rigid_boundary(host, 1.7, 0.3, keep_vr)            # host arrays, in place
    s.v_rigid_boundary(dev, 1.7, 0.3, keep_vr)             # device arrays, in place
    exp = orc.v_rigid_boundary(N, P, 1.7, 0.3, keep_vr, vr0)
    for k in names:
        np.testing.assert_allclose(host[k][:, :N], exp[k], rtol=0, atol=1e-14, err_msg=k)
        np.testing.assert_allclose(dev[k].cpu().numpy()[:, :N], exp[k], rtol=0, atol=1e-14, err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("grid", GRIDS)
def test_v_center_sphere_matches_oracle(built, torch, grid):
    from oracle import oracle as orc
    L, minc, N, P = grid
    s = make(L, minc, N, P)
    rng = np.random.default_rng(5)
    ddw = rng.standard_normal(s.lm_max) + 1j * rng.standard_normal(s.lm_max)
    got = s.v_center_sphere(ddw)
    exp = orc.v_center_sphere(ddw, minc, N, P)
    for g, e, k in zip(got, exp, ("vr", "vt", "vp")):
        np.testing.assert_allclose(g[:, :N], e, rtol=0, atol=1e-14, err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("grid", GRIDS)
def test_br_v_bcs_and_b_nl_bcs_match_oracle(built, torch, grid):
    """get_br_v_bcs (grid products + spat_to_sphertor, FP64 form: 1e-12
    relative like the other FP64 transforms) and get_b_nl_bcs (exact)."""
    from oracle import oracle as orc
    from conftest import rel_l2
    L, minc, N, P = grid
    s = make(L, minc, N, P)
    o = orc.OracleSHT(L, minc, N, P)
    rng = np.random.default_rng(6)
    br, vt, vp = (rng.standard_normal((s.n_phi_max, s.nlat_padded)) for _ in range(3))
    got = s.get_br_v_bcs(br, vt, vp, omega=0.4, or2=1.3, orho1=0.9)
    exp = orc.get_br_v_bcs(o, br, vt, vp, 0.4, 1.3, 0.9)
    for g, e in zip(got, exp):
        assert rel_l2(g, e) < 1e-12
    b, aj = s.get_b_nl_bcs("CMB", 2.5, got[0], got[1])
    assert np.array_equal(b, orc.get_b_nl_bcs(2.5, got[0]))
    assert np.array_equal(aj, orc.get_b_nl_bcs(2.5, got[1]))
    b2, aj2 = s.get_b_nl_bcs("ICB", 0.7, got[0], got[1])
    assert b2 is None and np.array_equal(aj2, orc.get_b_nl_bcs(0.7, got[1]))
