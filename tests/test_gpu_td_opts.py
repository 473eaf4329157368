"""The general spectral assembly (magic_sht_get_td_opts: get_td.f90 as the
radial loop calls it, rIter.f90:410-428) against the oracle's restatement
(oracle.get_td_full) on seeded spectra: the single- and double-curl forms
of dwdt (with dVxVhLM), the anelastic profiles, heatTermsLM and temp0 in
dsdt, dxidt with epscXi, the switches off (advection, Coriolis force,
induction), l_single_matrix, a cut-off degree l_R, and boundary levels where
only dVxBhLM, dVxVhLM, dVSrLM and dVXirLM are written.  FP64 handle:
<= 1e-13 relative L2 per output and level; FP64-accurate handle (FP64
arithmetic as well): <= 1e-12; 3xBF16 handle (FP32 arithmetic): <= 1e-6.  Entries the reference leaves as they were must keep their values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NLEV = 5
CASES = {
    "default": dict(),
    "double_curl_anel": dict(l_double_curl=True, orho1="p", beta="p", lcut=[31, 28, 31, 20, 31],
                             l_single_matrix=True),
    "anel_liquid_chem": dict(l_anel=True, l_anelastic_liquid=True, temp0="p", epsc="p", epscXi=0.37),
    "switches_off": dict(l_conv_nl=False, l_mag_nl=False, l_corr=False),
    "boundaries": dict(nbc=[1, 0, 0, 0, 2], l_double_curl=True, orho1="p", beta="p"),
    "boundaries_no_mag": dict(nbc=[0, 2, 0, 1, 0], l_mag_nl=False),
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


@pytest.mark.parametrize("L,minc,N,P", [(31, 1, 48, 96), (32, 2, 64, 64)])
@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp64tc", 1e-12), ("bf16x3", 1e-6)])
def test_get_td_opts_matches_oracle(built, oracle_mod, torch, L, minc, N, P, case, prec, tol):
    from magic_gb300 import SHT, _lib
    from magic_gb300.workload import spectra
    rng = np.random.default_rng(99)
    spec = {k: spectra(L, minc, NLEV, seed=7 + i) for i, k in enumerate(_lib.TDF_IN)}
    r = np.linspace(1.5, 0.55, NLEV)
    kw = dict(CASES[case])
    for k in ("orho1", "beta", "temp0", "epsc"):
        if kw.get(k) == "p":
            kw[k] = 0.5 + rng.random(NLEV)
    if "lcut" in kw:
        kw["lcut"] = np.minimum(np.array(kw["lcut"]), L)
    ref = oracle_mod.get_td_full(spec, r, 1.7e3, L, minc, **kw)
    s = SHT(L, minc, N, P, precision=prec, device=0)
    d = {k: torch.from_numpy(v).cuda() for k, v in spec.items()}
    fill = complex(11.5, -3.25)
    out = {k: torch.full((NLEV, s.lm_max), fill, dtype=torch.complex128, device="cuda") for k in _lib.TDF_OUT}
    got = s.get_td_opts(d, r, 1.7e3, out=out, **kw)
    torch.cuda.synchronize()
    s.device_status()
    for k in _lib.TDF_OUT:
        g = got[k].cpu().numpy()
        for i in range(NLEV):
            nan = np.isnan(ref[k][i])
            assert (g[i][nan] == fill).all(), (case, k, i, "written where the reference leaves it")
            if nan.all():
                continue
            a, b = g[i][~nan], ref[k][i][~nan]
            nb = np.linalg.norm(b)
            e = np.linalg.norm(a - b) / nb if nb > 0 else np.abs(a).max()
            assert e <= tol, (case, prec, k, i, e)
    s.close()


def test_get_td_opts_default_equals_get_td(built, torch):
    """The default switches reproduce magic_sht_get_td_nbc on the outputs it
    writes (dpdt at l = 0 aside, which magic_sht_get_td sets to zero)."""
    from magic_gb300 import SHT
    from magic_gb300.workload import spectra
    L, minc, N, P = 31, 1, 48, 96
    names = ("w", "dw", "z", "AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "VxBrLM", "VxBtLM", "VxBpLM")
    spec = {k: torch.from_numpy(spectra(L, minc, NLEV, seed=30 + i)).cuda() for i, k in enumerate(names)}
    r = np.linspace(1.5, 0.55, NLEV)
    nbc = np.array([1, 0, 0, 0, 2], dtype=np.int32)
    s = SHT(L, minc, N, P, precision="fp64", device=0)
    a = s.get_td(spec, r, 2e3, nbc=nbc)
    b = s.get_td_opts(spec, r, 2e3, nbc=nbc, outputs=("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM"))
    torch.cuda.synchronize()
    for k in ("dwdt", "dzdt", "dsdt", "dbdt", "djdt", "dVxBhLM"):
        for i in (1, 2, 3):
            e = float(torch.linalg.vector_norm(a[k][i] - b[k][i]) / torch.linalg.vector_norm(a[k][i]))
            assert e <= 1e-15, (k, i, e)
    e = float(torch.linalg.vector_norm(a["dVxBhLM"] - b["dVxBhLM"]) / torch.linalg.vector_norm(a["dVxBhLM"]))
    assert e <= 1e-15
