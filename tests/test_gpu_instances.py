"""Every instance size of the sixteen-instance batching case (l_max in
{63, 127, 255} with n_theta = 3 (l_max + 1) / 2 and n_phi_tot = 2 n_theta,
minc in {1, 4}) against the oracle on one radial level of the radial-loop
transform set (rIter.f90:466-712: 15 grids from 13 spectra, then 10 spectra
from the grids):
  - FP64 form and FP64-accurate tensor-core form: every call normwise
    <= 1e-12 and every output <= 1e-11 relative L2.  An output much smaller
    than the other outputs of its call carries the call's rounding error
    times the ratio: the spheroidal part of the curl's spat_to_qst at
    l_max = 255 is ~600x smaller than its partners, and the FP64 form itself
    differs from the oracle there by 2.8e-12;
  - 3xBF16 form: every call normwise <= 1e-6 (a vector field's three grids,
    or the q, s, t of one spat_to_qst).
minc = 4 with l_max = 63 or 127 runs the general-size FFT (n_phi/2 = 24 or
48), the others the fast path."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

SIZES = [(L, minc) for L in (63, 127, 255) for minc in (1, 4)]


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


def _oracle_level(o, spec, or2, r):
    """The radial set of one level through the oracle's public routines."""
    out = {"sc": o.scal_to_spat(spec["s"][r]), "pc": o.scal_to_spat(spec["p"][r]),
           "xic": o.scal_to_spat(spec["xi"][r])}
    for ks, v in ((("vrc", "vtc", "vpc"), o.torpol_to_spat(spec["w"][r], spec["dw"][r], spec["z"][r])),
                  (("cvrc", "cvtc", "cvpc"),
                   o.torpol_to_curl_spat(or2[r], spec["w"][r], spec["ddw"][r], spec["z"][r], spec["dz"][r])),
                  (("brc", "btc", "bpc"), o.torpol_to_spat(spec["b"][r], spec["db"][r], spec["aj"][r])),
                  (("cbrc", "cbtc", "cbpc"),
                   o.torpol_to_curl_spat(or2[r], spec["b"][r], spec["ddb"][r], spec["aj"][r], spec["dj"][r]))):
        out.update(zip(ks, v))
    return out


@pytest.mark.parametrize("L,minc", SIZES)
def test_instance_size_matches_oracle(built, oracle_mod, torch, L, minc):
    from magic_gb300 import SHT
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    N = 3 * (L + 1) // 2
    P = 2 * N // minc
    n, r = 3, 1  # the middle level (the radial envelope vanishes at both boundaries)
    spec = grid_space_inputs(L, minc, n, seed=500 + L + minc)
    or2 = or2_levels(n)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    ref_g = _oracle_level(o, spec, or2, r)
    fwd_in = {k: ref_g[v] for k, v in FORWARD_FROM_INVERSE.items()}
    ref_l = {}
    for pre in ("Adv", "VS", "VxB"):
        q, s_, t = o.spat_to_qst(fwd_in[pre + "r"], fwd_in[pre + "t"], fwd_in[pre + "p"])
        ref_l.update({pre + "rLM": q, pre + "tLM": s_, pre + "pLM": t})
    ref_l["heatTermsLM"] = o.scal_to_SH(fwd_in["heatTerms"])
    d = {k: torch.from_numpy(v).cuda() for k, v in spec.items()}
    dfwd = {k: torch.from_numpy(np.stack([v] * n)).cuda() for k, v in fwd_in.items()}
    groups = [("vrc", "vtc", "vpc"), ("cvrc", "cvtc", "cvpc"), ("brc", "btc", "bpc"), ("cbrc", "cbtc", "cbpc"),
              ("AdvrLM", "AdvtLM", "AdvpLM"), ("VSrLM", "VStLM", "VSpLM"), ("VxBrLM", "VxBtLM", "VxBpLM"),
              ("sc",), ("pc",), ("xic",), ("heatTermsLM",)]
    for prec, tol in (("fp64", 1e-12), ("fp64tc", 1e-12), ("bf16x3", 1e-6)):
        s = SHT(L, minc, N, P, precision=prec, device=0)
        g = s.transform_to_grid_space(d, or2=torch.from_numpy(or2).cuda())
        lm = s.transform_to_lm_space(dfwd)
        torch.cuda.synchronize()
        s.device_status()
        got = {k: v[r].cpu().numpy() for k, v in g.items()}
        got.update({k: v[r].cpu().numpy() for k, v in lm.items()})
        ref = dict(ref_g, **ref_l)
        if prec != "bf16x3":
            for k in ref:
                e = rel_l2(got[k], ref[k])
                assert e <= 10 * tol, (prec, k, e)
        for ks in groups:
            num = sum(float(np.linalg.norm(got[k] - ref[k])) ** 2 for k in ks) ** 0.5
            den = sum(float(np.linalg.norm(ref[k])) ** 2 for k in ks) ** 0.5
            assert num / den <= tol, (prec, ks, num / den)
        s.close()
