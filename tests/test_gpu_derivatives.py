"""The velocity-derivative grids of the radial synthesis set
(rIter.f90:527-545): torpol_to_spat(dw, ddw, dz) -> dvrdrc, dvtdrc, dvpdrc;
pol_to_grad_spat(w) -> dvrdtc, dvrdpc; torpol_to_dphspat(dw, z) -> dvtdpc,
dvpdpc; and the u.grad u set's pol_to_curlr_spat(z) -> cvrc alone (:540).
Every grid of magic_sht_transform_to_grid_space with the derivative outputs
against the oracle's routines level by level (per-level lcut; device
arrays, and host arrays through the pipelined path), in the FP64,
FP64-accurate tensor-core and 3xBF16 forms; then the radial loop's u.grad u
and anelastic stage against the entry points it composes."""
import numpy as np
import pytest

from test_gpu_parity import close, make

pytestmark = pytest.mark.gpu

DV = ["dvrdrc", "dvtdrc", "dvpdrc", "dvrdtc", "dvrdpc", "dvtdpc", "dvpdpc"]
TOL = {"fp64": 1e-12, "fp64tc": 1e-11}


@pytest.fixture(scope="module")
def torch():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build()


def _derivative_ref(o, spec_in, lcut):
    out = {k: [] for k in DV + ["vrc", "vtc", "vpc", "cvrc"]}
    for r in range(spec_in["w"].shape[0]):
        lc = int(lcut[r])
        w, dw, ddw, z, dz = (spec_in[k][r] for k in ("w", "dw", "ddw", "z", "dz"))
        for k, v in zip(("vrc", "vtc", "vpc"), o.torpol_to_spat(w, dw, z, lc)):
            out[k].append(v)
        for k, v in zip(DV[:3], o.torpol_to_spat(dw, ddw, dz, lc)):
            out[k].append(v)
        for k, v in zip(DV[3:5], o.pol_to_grad_spat(w, lc)):
            out[k].append(v)
        for k, v in zip(DV[5:], o.torpol_to_dphspat(dw, z, lc)):
            out[k].append(v)
        out["cvrc"].append(o.pol_to_curlr_spat(z, lc))
    return {k: np.array(v) for k, v in out.items()}


def _check(got, ref, tol, l2_only=False):
    from conftest import rel_l2
    for k in ref:
        if l2_only:  # the split form's max error follows the row scale
            e = rel_l2(np.asarray(got[k]), ref[k])
            assert e <= tol, (k, e)
        else:
            close(got[k], ref[k], tol=tol)


@pytest.mark.parametrize("grid", [(31, 1, 48, 96), (64, 4, 96, 48), (63, 1, 96, 192), (128, 1, 192, 384)])
@pytest.mark.parametrize("prec", ["fp64", "fp64tc"])
def test_derivative_grids_match_oracle(built, oracle_mod, torch, grid, prec):
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P = grid
    n = 5
    s = make(*grid, prec=prec)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    spec_in = grid_space_inputs(L, minc, n, seed=61)
    lcut = np.array([L, 0, max(L - 9, 1), 1, L - 1], dtype=np.int32)  # lcut 0 and 1: the edge degrees
    ref = _derivative_ref(o, spec_in, lcut)
    din = {k: torch.from_numpy(v).cuda() for k, v in spec_in.items()}
    or2 = torch.from_numpy(or2_levels(n)).cuda()
    # the curl form: every grid of the set plus the derivatives
    got = s.transform_to_grid_space(din, or2=or2, lcut=lcut, derivatives=True)
    torch.cuda.synchronize()
    assert set(DV) <= set(got) and "cvtc" in got
    _check({k: got[k].cpu().numpy() for k in ref if k != "cvrc"}, {k: v for k, v in ref.items() if k != "cvrc"},
           TOL[prec])
    # the u.grad u form: cvrc alone (cvtc, cvpc left out)
    got2 = s.transform_to_grid_space(din, or2=or2, lcut=lcut, derivatives=True, out={"cvtc": None, "cvpc": None})
    torch.cuda.synchronize()
    assert "cvtc" not in got2 and "cvpc" not in got2
    _check({k: got2[k].cpu().numpy() for k in ref}, ref, TOL[prec])
    # the other grids are the same with and without the derivative outputs
    plain = s.transform_to_grid_space(din, or2=or2, lcut=lcut)
    torch.cuda.synchronize()
    assert not set(DV) & set(plain)
    for k in plain:
        assert torch.equal(plain[k], got[k]), k
    s.device_status()


def test_derivative_grids_host_arrays_pipelined(built, oracle_mod, torch):
    """Host arrays over more levels than one pipelined chunk (16): the
    derivative outputs travel with the rest."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 31, 1, 48, 96, 37
    s = make(L, minc, N, P)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    spec_in = grid_space_inputs(L, minc, n, seed=62)
    lcut = np.random.default_rng(4).integers(1, L + 1, size=n).astype(np.int32)
    ref = _derivative_ref(o, spec_in, lcut)
    got = s.transform_to_grid_space(spec_in, or2=or2_levels(n), lcut=lcut, derivatives=True,
                                    out={"cvtc": None, "cvpc": None})
    _check({k: got[k] for k in ref}, ref, TOL["fp64"])
    s.device_status()


def test_derivative_grids_bf16x3(built, oracle_mod, torch):
    """The 3xBF16 form: relative L2 within 2e-6 of the oracle."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 63, 1, 96, 192, 4
    s = make(L, minc, N, P, prec="bf16x3")
    o = oracle_mod.OracleSHT(L, minc, N, P)
    spec_in = grid_space_inputs(L, minc, n, seed=63)
    lcut = np.array([L, L - 3, L, L - 1], dtype=np.int32)
    ref = _derivative_ref(o, spec_in, lcut)
    din = {k: torch.from_numpy(v).cuda() for k, v in spec_in.items()}
    got = s.transform_to_grid_space(din, or2=torch.from_numpy(or2_levels(n)).cuda(), lcut=lcut,
                                    derivatives=True, out={"cvtc": None, "cvpc": None})
    torch.cuda.synchronize()
    _check({k: got[k].cpu().numpy() for k in ref}, ref, 2e-6, l2_only=True)
    s.device_status()


@pytest.mark.parametrize("physics", [
    dict(l_adv_curl=False),
    dict(l_anel=True, ViscHeatFac=0.6, OhmLossFac=1.3),
    dict(l_adv_curl=False, l_anel=True, l_chemical_conv=True, l_double_curl=True, ViscHeatFac=0.4, epscXi=0.02),
])
def test_radial_loop_derivative_physics_composes_the_entry_points(built, torch, physics):
    """The loop's u.grad u and anelastic stages (with density, temperature,
    viscosity and diffusivity profiles) equal the synthesis set with the
    derivative grids -> boundary grids -> get_nl_opts -> the analysis set ->
    get_td_opts called directly; the derivative grids are compared with the
    oracle above."""
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import grid_space_inputs
    L, minc, N, P, n = 63, 1, 96, 192, 6
    s = make(L, minc, N, P)
    r = np.linspace(1.538, 0.538, n)
    rng = np.random.default_rng(9)
    prof = {"orho1": 1.0 + 0.3 * rng.random(n), "beta": -0.5 * rng.random(n), "otemp1": 1.0 + 0.2 * rng.random(n),
            "visc": 1.0 + 0.1 * rng.random(n), "lam": 1.0 + 0.1 * rng.random(n), "temp0": 1.0 + 0.2 * rng.random(n)}
    ph = dict(prof, **physics)
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=23).items()}
    loop = RadialLoop(s, r, cor_fac=40.0, LFfac=0.8, ktopv=1, kbotv=1, physics=ph)
    got = loop.step(spec)
    torch.cuda.synchronize()
    curl = physics.get("l_adv_curl", True)
    g = got["grids"]
    assert set(DV) <= set(g)
    assert ("cvtc" in g) == curl
    # the synthesis set by hand (stress-free boundaries: vrc = 0 there)
    want = s.transform_to_grid_space(spec, or2=1.0 / r ** 2, derivatives=True,
                                     out=None if curl else {"cvtc": None, "cvpc": None})
    want["vrc"][0].zero_()
    want["vrc"][n - 1].zero_()
    torch.cuda.synchronize()
    assert set(want) == set(g)
    for k in want:
        assert torch.equal(g[k], want[k]), k
    nbc = torch.from_numpy(loop.nbc).cuda()
    flags = {k: physics[k] for k in ("l_adv_curl", "l_anel", "l_chemical_conv") if k in physics}
    consts = {k: physics[k] for k in ("ViscHeatFac", "OhmLossFac") if k in physics}
    nl = s.get_nl_opts({k: v.clone() for k, v in g.items()}, r, LFfac=0.8, nbc=nbc, **flags, **consts,
                       **{k: prof[k] for k in ("orho1", "beta", "otemp1", "visc", "lam")})
    lm = s.transform_to_lm_space(nl)
    tdin = {k: spec[k] for k in ("w", "dw", "ddw", "z", "dz")}
    tdin.update({k: lm[k] for k in ("AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "heatTermsLM", "VXitLM", "VxBrLM",
                                    "VxBtLM", "VxBpLM") if k in lm})
    outs = loop._td_outputs()
    td = s.get_td_opts(tdin, r, 40.0, outputs=outs, nbc=nbc, orho1=prof["orho1"], beta=prof["beta"],
                       temp0=prof["temp0"], epscXi=physics.get("epscXi", 0.0), l_anel=physics.get("l_anel", False),
                       l_double_curl=physics.get("l_double_curl", False))
    torch.cuda.synchronize()
    for k in outs:
        assert torch.equal(got[k], td[k]), k
    if physics.get("l_anel"):
        assert float(torch.linalg.vector_norm(lm["heatTermsLM"])) > 0
    s.device_status()


def test_radial_loop_rigid_boundaries_with_density_profile(built, oracle_mod, torch):
    """Rigid rotating boundaries under a density profile: v_rigid_boundary
    takes r^2 rho0 = r^2 / orho1 (nonlinear_bcs.f90:160-172), against the
    oracle's restatement; the anelastic stage runs to its end."""
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import grid_space_inputs
    L, minc, N, P, n = 31, 1, 48, 96, 5
    s = make(L, minc, N, P)
    r = np.linspace(1.538, 0.538, n)
    orho1 = 1.0 + 0.5 * np.linspace(0.0, 1.0, n)
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=29).items()}
    loop = RadialLoop(s, r, cor_fac=40.0, ktopv=2, kbotv=2, omega_ma=0.3, omega_ic=-0.2,
                      physics=dict(orho1=orho1, l_anel=True, l_adv_curl=False))
    got = loop.step(spec)
    torch.cuda.synchronize()
    g = got["grids"]
    for i, om in ((0, 0.3), (n - 1, -0.2)):
        b = oracle_mod.v_rigid_boundary(N, P, r[i] ** 2 / orho1[i], om, False, np.zeros((P, N)))
        for k, key in (("vr", "vrc"), ("vt", "vtc"), ("vp", "vpc")):
            np.testing.assert_allclose(g[key][i].cpu().numpy(), b[k], rtol=0, atol=1e-14 * max(1.0, np.abs(b[k]).max()))
    for k in loop._td_outputs():
        assert bool(torch.isfinite(got[k]).all()), k
    s.device_status()
