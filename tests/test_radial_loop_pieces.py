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


@pytest.mark.gpu
def test_get_td_boundary_levels(built, torch):
    """get_td with boundary flags (nBc of rIter.f90): at flagged levels only
    dVxBhLM is written (get_td.f90:598-612), the other outputs keep the
    caller's values; interior levels match the oracle as before."""
    from oracle import oracle as orc
    from magic_gb300 import _lib
    from conftest import rel_l2
    L, minc, N, P = 63, 1, 96, 192
    s = make(L, minc, N, P)
    n = 4
    rng = np.random.default_rng(10)
    spec = {k: torch.from_numpy(rng.standard_normal((n, s.lm_max)) + 1j * rng.standard_normal((n, s.lm_max))).cuda()
            for k in _lib.TD_IN}
    r = np.array([1.5, 1.2, 0.9, 0.6])
    nbc = np.array([1, 0, 0, 2], dtype=np.int32)
    sentinel = 7.0 + 3.0j
    out = {k: torch.full((n, s.lm_max), sentinel, dtype=torch.complex128, device="cuda") for k in _lib.TD_OUT}
    s.get_td(spec, r, cor_fac=1.0e2, out=out, nbc=nbc)
    torch.cuda.synchronize()
    ref = orc.get_td({k: v.cpu().numpy() for k, v in spec.items()}, r, 1.0e2, L, minc, nbc=nbc)
    for k in _lib.TD_OUT:
        got = out[k].cpu().numpy()
        for i in range(n):
            if nbc[i] != 0 and k != "dVxBhLM":
                assert np.all(got[i] == sentinel), (k, i)
            else:
                assert rel_l2(got[i], ref[k][i]) < 1e-13, (k, i)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [
    dict(ktopv=2, kbotv=2, omega_ma=0.3, omega_ic=-0.2),                    # rigid, lMagNlBc off
    dict(ktopv=1, kbotv=1, l_cond_ma=True, omega_ma=0.25),                  # stress-free, conducting mantle
    dict(ktopv=2, kbotv=1, l_rot_ma=True, l_cond_ma=True, l_vr_cmb=True, omega_ma=0.3),  # rigid, vr kept, torque
])
def test_radial_loop_stage_matches_oracle(built, torch, oracle_mod, cfg):
    """One explicit stage of the radial loop (rIter.f90:94-464) over five
    levels with both boundaries, FP64 form, against the same stage composed
    from the oracle's transforms and restatements."""
    from test_gpu_parity import _radial_set_ref, close
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import grid_space_inputs
    from conftest import rel_l2
    orc = oracle_mod
    L, minc, N, P, n = 63, 1, 96, 192, 5
    s = make(L, minc, N, P)
    o = orc.OracleSHT(L, minc, N, P)
    r = np.linspace(1.538, 0.538, n)                         # outer boundary first
    lcut = np.array([L, L, L - 5, L, L], dtype=np.int32)
    epsc = np.array([0.0, 0.3, 0.1, -0.2, 0.0])
    spec_np = grid_space_inputs(L, minc, n, seed=8)
    loop = RadialLoop(s, r, cor_fac=50.0, courfac=2.5, alffac=1.0, lcut=lcut, epsc=epsc, **cfg)
    got = loop.step({k: torch.from_numpy(v).cuda() for k, v in spec_np.items()})
    torch.cuda.synchronize()
    # ---- the same stage from the oracle
    or2 = 1.0 / r ** 2
    g = _radial_set_ref(o, spec_np, or2, lcut)
    for i, kind, om, kv in ((0, cfg["ktopv"], cfg.get("omega_ma", 0.0), cfg.get("l_vr_cmb", False)),
                            (n - 1, cfg["kbotv"], cfg.get("omega_ic", 0.0), cfg.get("l_vr_icb", False))):
        if kind == 1:
            g["vrc"][i] = 0.0
        else:
            b = orc.v_rigid_boundary(N, P, r[i] ** 2, om, kv, g["vrc"][i])
            g["vrc"][i], g["vtc"][i], g["vpc"][i] = b["vr"], b["vt"], b["vp"]
    lo, hi = (0, n) if loop.lMagNlBc else (1, n - 1)
    nl = orc.get_nl({k: v[lo:hi] for k, v in g.items()}, or2[lo:hi], N)
    # a rigid boundary's V x B has vr = vt = 0 in the reference (get_nl.f90:391-395)
    for i, kind, kv in ((0, cfg["ktopv"], cfg.get("l_vr_cmb", False)), (n - 1, cfg["kbotv"], cfg.get("l_vr_icb", False))):
        if loop.lMagNlBc and kind == 2 and kv:
            gz = {k: np.array(v[i:i + 1]) for k, v in g.items()}
            gz["vrc"][:] = 0.0
            nz = orc.get_nl(gz, or2[i:i + 1], N)
            for k in nz:
                nl[k][i - lo] = nz[k][0]
    lm = {k: np.zeros((n, s.lm_max), dtype=np.complex128) for k in
          ("AdvrLM", "AdvtLM", "AdvpLM", "VSrLM", "VStLM", "VSpLM", "VxBrLM", "VxBtLM", "VxBpLM")}
    for j, i in enumerate(range(lo, hi)):
        for pre in ("Adv", "VS", "VxB"):
            q, ss, t = o.spat_to_qst(nl[pre + "r"][j], nl[pre + "t"][j], nl[pre + "p"][j], int(lcut[i]))
            lm[pre + "rLM"][i], lm[pre + "tLM"][i], lm[pre + "pLM"][i] = q, ss, t
    lm["VSrLM"][0] = 0.0
    lm["VSrLM"][n - 1] = 0.0
    td_in = {k: spec_np[k] for k in ("w", "dw", "z")}
    td_in.update({k: lm[k] for k in ("AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "VxBrLM", "VxBtLM", "VxBpLM")})
    td = orc.get_td(td_in, r, 50.0, L, minc, lcut, epsc, nbc=loop.nbc)
    for k in ("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM"):
        gk = got[k].cpu().numpy()
        for i in range(n):
            if loop.nbc[i] != 0 and k != "dVxBhLM":
                continue
            assert rel_l2(gk[i], td[k][i]) < 1e-10, (k, i, rel_l2(gk[i], td[k][i]))
    close(got["VSrLM"].cpu().numpy(), lm["VSrLM"], tol=1e-10)
    dtr, dth = orc.courant({k: g[k] for k in ("vrc", "vtc", "vpc", "brc", "btc", "bpc")}, loop.radial, N, 2.5, 1.0)
    np.testing.assert_allclose(got["dtrkc"], dtr, rtol=1e-10)
    np.testing.assert_allclose(got["dthkc"], dth, rtol=1e-10)
    if loop.torque_ma:  # the mantle's torque, negated by the radial loop (rIter.f90:462)
        exp_t = -orc.lorentz_torque(g["brc"][0], g["bpc"][0], N)
        scale = orc.lorentz_torque(np.abs(g["brc"][0]), np.abs(g["bpc"][0]), N)
        assert abs(got["lorentz_torque_ma"] - exp_t) <= 1e-12 * scale, (got["lorentz_torque_ma"], exp_t)
    if loop.l_b_nl_cmb:
        exp = orc.get_br_v_bcs(o, g["brc"][0], g["vtc"][0], g["vpc"][0], cfg["omega_ma"], or2[0], 1.0)
        close(got["br_vt_lm_cmb"].cpu().numpy(), exp[0], tol=1e-10)
        close(got["br_vp_lm_cmb"].cpu().numpy(), exp[1], tol=1e-10)


@pytest.mark.gpu
def test_radial_loop_kernels_have_phase_timers(built, torch):
    """The radial-loop kernels are timed like the transforms: with profiling
    on, one stage records CUDA-event time and launches under get_nl,
    courant, get_td and the boundary kernels."""
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import grid_space_inputs
    L, n = 31, 4
    s = make(L, 1, 48, 96)
    loop = RadialLoop(s, np.linspace(1.538, 0.538, n), cor_fac=10.0, ktopv=2, kbotv=2)
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, 1, n, seed=3).items()}
    s.set_profiling(True)
    s.phase_times(reset=True)
    loop.step(spec)
    ph = s.phase_times(reset=True)
    s.set_profiling(False)
    assert ph["nl"][1] == 1 and ph["td"][1] == 1 and ph["courant"][1] == 2 and ph["bcs"][1] == 2
    for k in ("nl", "courant", "td", "bcs", "fft_inv", "fft_fwd"):
        assert ph[k][0] > 0.0, k


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["wide", "ties", "tiny", "huge", "zeros_no_damp"])
@pytest.mark.parametrize("mag", [True, False])
def test_courant_filter_keeps_exact_maxima(built, torch, kind, mag):
    """The Courant kernel skips points whose FP32 estimate cannot hold the
    maximum; the maxima must still be the FP64 ones.  Inputs that stress the
    estimate: a dynamic range of 1e+-20 (lognormal), near-ties (every value
    1 + 1e-12 noise), fields of 1e-30 (below the estimate's absolute floor),
    values of 1e200 (beyond FP32), and exact zeros in B without damping (0/0
    terms left out of the maximum)."""
    from oracle import oracle as orc
    L, minc, N, P = 63, 1, 96, 192
    s = make(L, minc, N, P)
    n = 4
    rng = np.random.default_rng(77)
    shape = (n, s.n_phi_max, s.nlat_padded)
    keys = ("vrc", "vtc", "vpc", "brc", "btc", "bpc")
    if kind == "wide":
        h = {k: rng.standard_normal(shape) * np.exp(rng.standard_normal(shape) * 15.0) for k in keys}
    elif kind == "ties":
        h = {k: np.sign(rng.standard_normal(shape)) * (1.0 + 1e-12 * rng.standard_normal(shape)) for k in keys}
    elif kind == "tiny":
        h = {k: 1e-30 * rng.standard_normal(shape) for k in keys}
    elif kind == "huge":
        h = {k: rng.standard_normal(shape) for k in keys}
        for k in keys:
            h[k][:, 3, 5] = 1e200 * (1.0 + rng.random(n))
    else:
        h = {k: rng.standard_normal(shape) for k in keys}
        for k in ("brc", "btc", "bpc"):
            h[k][:, ::2, :] = 0.0
    damp = kind != "zeros_no_damp"
    g = {k: torch.from_numpy(v).cuda() for k, v in h.items()}
    if not mag:
        for k in ("brc", "btc", "bpc"):
            g.pop(k)
            h[k] = None
    rad = _radial(n, rng)
    got_r, got_h = s.courant(g, rad, courfac=2.5, alffac=1.0, LFfac=1.3, opm=0.7, alf_damp=damp)
    exp_r, exp_h = orc.courant(h, rad, N, courfac=2.5, alffac=1.0, LFfac=1.3, opm=0.7, alf_damp=damp)
    np.testing.assert_allclose(got_r, exp_r, rtol=1e-13, atol=0)
    np.testing.assert_allclose(got_h, exp_h, rtol=1e-13, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "bf16x3"])
def test_radial_loop_stage_graph_matches_eager(built, torch, form):
    """A stage captured as one CUDA graph (RadialLoop.capture) gives the eager
    stage's outputs bit for bit, and a replay after the spectra changed in
    place gives the eager outputs of the new spectra."""
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import grid_space_inputs
    L, n = 63, 5
    s = make(L, 1, 96, 192, prec=form)
    r = np.linspace(1.538, 0.538, n)
    loop = RadialLoop(s, r, cor_fac=50.0, ktopv=1, kbotv=2, l_cond_ma=True, omega_ma=0.25)
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, 1, n, seed=12).items()}
    keys = ("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM", "VSrLM", "br_vt_lm_cmb", "br_vp_lm_cmb")
    inner = slice(1, n - 1)  # get_td leaves all but dVxBhLM unwritten at the boundary levels

    def same(a, b, k):
        return torch.equal(a[inner], b[inner]) if k in ("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt") \
            else torch.equal(a, b)
    eager = loop.step(spec)
    eager = {k: (v.clone() if hasattr(v, "clone") else v) for k, v in eager.items() if k != "grids"}
    sg = loop.capture(spec)
    for _ in range(2):
        got = sg.replay()
        for k in keys:
            assert same(got[k], eager[k], k), k
        assert np.array_equal(got["dtrkc"], eager["dtrkc"]) and np.array_equal(got["dthkc"], eager["dthkc"])
    new = grid_space_inputs(L, 1, n, seed=13)
    for k, v in spec.items():
        v.copy_(torch.from_numpy(new[k]))
    torch.cuda.synchronize()
    ref = loop.step(spec)
    got = sg.replay()
    for k in keys:
        assert same(got[k], ref[k], k), k
    assert np.array_equal(got["dtrkc"], ref["dtrkc"])
    sg.close()
    s.device_status()


@pytest.mark.gpu
@pytest.mark.parametrize("grid", GRIDS + [(255, 1, 384, 768)])
def test_lorentz_torque_matches_oracle(built, torch, grid):
    """get_lorentz_torque (outRot.f90:423-483) of one boundary grid, host and
    device arrays, with and without the Grenoble b0 term, against the numpy
    restatement (summation order differs: tolerance relative to the sum of
    the absolute terms)."""
    from oracle import oracle as orc
    L, minc, N, P = grid
    s = make(L, minc, N, P)
    rng = np.random.default_rng(31)
    br = rng.standard_normal((s.n_phi_max, s.nlat_padded))
    bp = rng.standard_normal((s.n_phi_max, s.nlat_padded))
    scale = orc.lorentz_torque(np.abs(br), np.abs(bp) * 2.0, N, 1.7, 0.0)
    for b0 in (0.0, 0.45):
        exp = orc.lorentz_torque(br, bp, N, 1.7, b0)
        got_h = s.lorentz_torque(br, bp, 1.7, b0)
        out = torch.empty(1, dtype=torch.float64, device="cuda")
        s.lorentz_torque(torch.from_numpy(br).cuda(), torch.from_numpy(bp).cuda(), 1.7, b0, out=out)
        got_d = float(out.item())
        assert abs(got_h - exp) <= 1e-12 * scale, (got_h, exp)
        assert got_d == got_h
    s.device_status()


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [
    dict(ktopv=2, kbotv=2, omega_ma=0.3, omega_ic=-0.2),
    dict(ktopv=1, kbotv=2, l_cond_ma=True, omega_ma=0.25),
    dict(ktopv=2, kbotv=1, l_rot_ma=True, l_cond_ma=True, l_vr_cmb=True, omega_ma=0.3),
])
def test_radial_loop_general_physics_default_matches(built, torch, cfg):
    """The stage through the general get_nl / get_td (physics={}, the
    reference's defaults) equals the stage through the Boussinesq kernels to
    rounding, boundaries included (FP64 form)."""
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import grid_space_inputs
    from conftest import rel_l2
    L, minc, N, P, n = 63, 1, 96, 192, 5
    s = make(L, minc, N, P)
    r = np.linspace(1.538, 0.538, n)
    lcut = np.array([L, L, L - 5, L, L], dtype=np.int32)
    epsc = np.array([0.0, 0.3, 0.1, -0.2, 0.0])
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=8).items()}
    la = RadialLoop(s, r, cor_fac=50.0, lcut=lcut, epsc=epsc, **cfg)
    a = la.step(spec)
    b = RadialLoop(s, r, cor_fac=50.0, lcut=lcut, epsc=epsc, physics={}, **cfg).step(spec)
    torch.cuda.synchronize()
    for k in ("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM"):
        x, y = a[k].cpu().numpy(), b[k].cpu().numpy()
        for i in range(n):
            if la.nbc[i] != 0 and k != "dVxBhLM":  # outputs get_td leaves untouched at a boundary
                continue
            # get_dpdt leaves l = 0 (lm = 1, get_td.f90:311-379): zero on the general path
            xi, yi = (x[i][1:], y[i][1:]) if k == "dpdt" else (x[i], y[i])
            if k == "dpdt":
                assert y[i][0] == 0, (k, i)
            if np.linalg.norm(xi) == 0:
                assert np.linalg.norm(yi) == 0, (k, i)
                continue
            assert rel_l2(yi, xi) < 1e-12, (k, i, rel_l2(yi, xi))
    np.testing.assert_array_equal(a["dtrkc"], b["dtrkc"])
    np.testing.assert_array_equal(a["dthkc"], b["dthkc"])


@pytest.mark.gpu
def test_radial_loop_general_physics_composes_the_entry_points(built, torch):
    """A stage with density and temperature profiles, composition and
    double-curl dwdt: the loop's general path equals get_nl_opts -> the
    analysis set -> get_td_opts called directly with the same switches and
    profiles."""
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import grid_space_inputs
    L, minc, N, P, n = 63, 1, 96, 192, 6
    s = make(L, minc, N, P)
    r = np.linspace(1.538, 0.538, n)
    rng = np.random.default_rng(3)
    prof = {"orho1": 1.0 + 0.3 * rng.random(n), "beta": -0.5 * rng.random(n), "otemp1": 1.0 + 0.2 * rng.random(n),
            "visc": 1.0 + 0.1 * rng.random(n), "lam": 1.0 + 0.1 * rng.random(n), "temp0": 1.0 + 0.2 * rng.random(n)}
    physics = dict(prof, ViscHeatFac=0.7, OhmLossFac=0.4, l_chemical_conv=True, l_double_curl=True, epscXi=0.05)
    with pytest.raises(ValueError):
        RadialLoop(s, r, cor_fac=40.0, physics=dict(physics, l_anell=True))  # unknown key
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=21).items()}
    loop = RadialLoop(s, r, cor_fac=40.0, LFfac=0.8, ktopv=1, kbotv=1, physics=physics)
    got = loop.step(spec)
    torch.cuda.synchronize()
    # the same by hand (lMagNlBc holds with stress-free boundaries: every level)
    g = {k: v.clone() for k, v in got["grids"].items()}
    nbc = torch.from_numpy(loop.nbc).cuda()
    nl = s.get_nl_opts(g, r, LFfac=0.8, ViscHeatFac=0.7, OhmLossFac=0.4, nbc=nbc, l_chemical_conv=True,
                       **{k: prof[k] for k in ("orho1", "beta", "otemp1", "visc", "lam")})
    lm = s.transform_to_lm_space(nl)
    tdin = {k: spec[k] for k in ("w", "dw", "ddw", "z", "dz")}
    tdin.update({k: lm[k] for k in ("AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "heatTermsLM", "VXitLM", "VxBrLM",
                                    "VxBtLM", "VxBpLM")})
    outs = ["dwdt", "dzdt", "dVxVhLM", "dsdt", "dVSrLM", "dxidt", "dVXirLM", "dbdt", "djdt", "dVxBhLM"]
    td = s.get_td_opts(tdin, r, 40.0, outputs=outs, nbc=nbc, orho1=prof["orho1"], beta=prof["beta"],
                       temp0=prof["temp0"], epscXi=0.05, l_double_curl=True)
    torch.cuda.synchronize()
    for k in outs:
        assert torch.equal(got[k], td[k]), k
