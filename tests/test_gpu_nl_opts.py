"""The general grid-space nonlinear products (magic_sht_get_nl_opts,
get_nl.f90:213-441 with the Lorentz-force combination of
rIter.f90:645-662) against the oracle's restatement (oracle.get_nl_full) on
seeded grids, for the reference's switch combinations: curl-form and
u.grad u advection, the Lorentz force with and without the advection,
entropy and composition advection, the induction in its bulk, stress-free
(nBc = 1, low-conductivity region) and rigid (nBc = 2) forms, anelastic
profiles, viscous heating and ohmic losses.  FP64 handle: <= 1e-13 relative
L2 per output and level; the FP64-accurate handle computes in double-float
arithmetic (2^-48 per operation): <= 1e-12; the 3xBF16 handle computes in
FP32: <= 1e-6.
Outputs a level does not produce must keep the values they had."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L, MINC, N, P, NLEV = 31, 1, 48, 96, 5

CASES = {
    "boussinesq": dict(),
    "ugradu_anel_chem": dict(l_adv_curl=False, l_chemical_conv=True, LFfac=0.7, orho1="prof", beta="prof"),
    "anel_heat": dict(l_anel=True, l_chemical_conv=True, ViscHeatFac=0.3, OhmLossFac=1.9, orho1="prof",
                      beta="prof", otemp1="prof", visc="prof", lam="prof"),
    "lorentz_only": dict(l_conv_nl=False, l_heat_nl=False, LFfac=2.5),
    "boundaries_lcr": dict(nbc=[1, 0, 0, 2, 0], lcr=[0, 0, 1, 0, 0]),
    "ugradu_boundaries": dict(l_adv_curl=False, l_anel=True, nbc=[2, 0, 0, 0, 1], lcr=[0, 1, 0, 0, 0]),
}


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


def _inputs():
    from magic_gb300 import _lib
    rng = np.random.default_rng(2024)
    grids = {k: rng.standard_normal((NLEV, P, N)) for k in _lib.NLF_IN}
    r = np.linspace(1.5, 0.55, NLEV)
    prof = {k: 0.5 + rng.random(NLEV) for k in ("orho1", "otemp1", "visc", "lam")}
    prof["beta"] = rng.standard_normal(NLEV)
    return grids, r, prof


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp64tc", 1e-12), ("bf16x3", 1e-6)])
def test_get_nl_opts_matches_oracle(built, oracle_mod, torch, case, prec, tol):
    from magic_gb300 import SHT, _lib
    grids, r, prof = _inputs()
    kw = dict(CASES[case])
    for k in ("orho1", "beta", "otemp1", "visc", "lam"):
        if kw.get(k) == "prof":
            kw[k] = prof[k]
    ref = oracle_mod.get_nl_full(grids, N, r, **kw)
    s = SHT(L, MINC, N, P, precision=prec, device=0)
    d = {k: torch.from_numpy(v).cuda() for k, v in grids.items()}
    fill = 123.25  # outputs a level does not produce keep this value
    out = {k: torch.full((NLEV, P, N), fill, dtype=torch.float64, device="cuda") for k in _lib.NLF_OUT}
    got = s.get_nl_opts(d, r, out=out, **kw)
    torch.cuda.synchronize()
    s.device_status()
    for k in _lib.NLF_OUT:
        g = got[k].cpu().numpy()
        for i in range(NLEV):
            if np.isnan(ref[k][i]).all():
                assert (g[i] == fill).all(), (case, k, i, "written")
                continue
            e = np.linalg.norm(g[i] - ref[k][i]) / max(np.linalg.norm(ref[k][i]), 1e-300)
            if np.linalg.norm(ref[k][i]) == 0:
                e = np.abs(g[i]).max()
            assert e <= tol, (case, prec, k, i, e)
    s.close()


def test_get_nl_opts_default_equals_get_nl(built, torch):
    """The Boussinesq default of the general entry point reproduces the
    single-configuration magic_sht_get_nl bit for bit on Adv, VS and VxB."""
    from magic_gb300 import SHT
    from magic_gb300.workload import radii
    grids, _, _ = _inputs()
    r = radii(NLEV)
    s = SHT(L, MINC, N, P, precision="fp64", device=0)
    d = {k: torch.from_numpy(v).cuda() for k, v in grids.items()}
    a = s.get_nl(d, or2=1.0 / r ** 2)
    b = s.get_nl_opts(d, r)
    torch.cuda.synchronize()
    for k in ("Advr", "Advt", "Advp", "VSr", "VSt", "VSp", "VxBr", "VxBt", "VxBp"):
        e = float(torch.linalg.vector_norm(a[k] - b[k]) / torch.linalg.vector_norm(a[k]))
        assert e <= 1e-15, (k, e)


def test_get_nl_opts_rejects_missing_grids(built, torch):
    from magic_gb300 import SHT, _lib
    grids, r, _ = _inputs()
    s = SHT(L, MINC, N, P, precision="fp64", device=0)
    d = {k: torch.from_numpy(v).cuda() for k, v in grids.items() if not k.startswith("dv")}
    with pytest.raises(_lib.ShtError) as e:
        s.get_nl_opts(d, r, l_adv_curl=False)  # u.grad u needs the derivative grids
    assert e.value.code == _lib.ERR_ARG


@pytest.mark.parametrize("prec", ["fp64", "fp64tc"])
def test_composition_flux_in_the_analysis_set(built, oracle_mod, torch, prec):
    """transform_to_lm_space with the composition flux V Xi (l_chemical_conv,
    rIter.f90:699-702): VXirLM, VXitLM, VXipLM are spat_to_qst of VXir, VXit,
    VXip, beside the other analysis outputs (device and host arrays)."""
    from magic_gb300 import SHT
    rng = np.random.default_rng(77)
    g = {k: rng.standard_normal((NLEV, P, N)) for k in ("VXir", "VXit", "VXip", "VSr", "VSt", "VSp")}
    s = SHT(L, MINC, N, P, precision=prec, device=0)
    o = oracle_mod.OracleSHT(L, MINC, N, P)
    for dev in (True, False):
        inp = {k: torch.from_numpy(v).cuda() for k, v in g.items()} if dev else g
        lm = s.transform_to_lm_space(inp)
        torch.cuda.synchronize()
        for i in range(NLEV):
            for pre in ("VXi", "VS"):
                ref = o.spat_to_qst(g[pre + "r"][i], g[pre + "t"][i], g[pre + "p"][i])
                for c, rv in zip("rtp", ref):
                    got = lm[pre + c + "LM"][i]
                    got = got.cpu().numpy() if dev else got
                    e = np.linalg.norm(got - rv) / np.linalg.norm(rv)
                    assert e <= 1e-12, (prec, dev, pre + c, i, e)
