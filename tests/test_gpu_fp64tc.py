"""The FP64-accurate tensor-core form (precision "fp64tc": seven fixed-point
BF16 digits per operand, 28 digit products accumulated exactly in FP32 on
tcgen05, double-float FFTs and half spectra) against the oracle.

Every public routine on the parity grids meets the FP64 form's own tolerance
(relative L2 <= 1e-12, relative max <= 1e-11), for both Legendre kernels of
the form: tc_kernel 0 (the tensor-core sums, the default) and 1 (the FP64
SIMT sums feeding the same double-float FFTs).  The double-float FFTs round
at 2^-48 (FP64: 2^-53), about 5e-15 normwise per call; an output much smaller
than the other outputs of its call carries that error times the ratio (the
spheroidal part of the curl's spat_to_qst is ~600x smaller than its partners
at l_max = 255: 3.8e-12), so the radial-set outputs are held to 1e-11 each
and to 1e-13 normwise per call."""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import GRIDS, close, make, spec, _radial_set_ref

pytestmark = pytest.mark.gpu
KERNELS = [0, 1]


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


def mk(grid, kernel):
    s = make(*grid, prec="fp64tc")
    s.set_tuning(tc_kernel=kernel)
    return s


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("grid", GRIDS)
def test_fp64tc_inverse_routines_match_oracle(built, oracle_mod, torch, grid, kernel):
    L, minc, N, P = grid
    s = mk(grid, kernel)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = spec(o, 4, seed=L + minc)
    for lcut in (L, max(L - 5, 1)):
        close(s.scal_to_spat(S[0], lcut), o.scal_to_spat(S[0], lcut))
        close(s.pol_to_curlr_spat(S[1], lcut), o.pol_to_curlr_spat(S[1], lcut))
        close(np.array(s.scal_to_grad_spat(S[0], lcut)), np.array(o.scal_to_grad_spat(S[0], lcut)))
        close(np.array(s.torpol_to_spat(S[0], S[1], S[2], lcut)),
              np.array(o.torpol_to_spat(S[0], S[1], S[2], lcut)))
        close(np.array(s.sphtor_to_spat(S[1], S[2], lcut)), np.array(o.sphtor_to_spat(S[1], S[2], lcut)))
        close(np.array(s.torpol_to_dphspat(S[1], S[2], lcut)),
              np.array(o.torpol_to_dphspat(S[1], S[2], lcut)))
        close(np.array(s.torpol_to_curl_spat(0.83, S[0], S[3], S[1], S[2], lcut)),
              np.array(o.torpol_to_curl_spat(0.83, S[0], S[3], S[1], S[2], lcut)))
    close(np.array(s.torpol_to_spat_IC(0.3, 0.35, S[0], S[1], S[2])),
          np.array(o.torpol_to_spat_IC(0.3, 0.35, S[0], S[1], S[2])))
    s.device_status()


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("grid", GRIDS)
def test_fp64tc_forward_routines_match_oracle(built, oracle_mod, torch, grid, kernel):
    L, minc, N, P = grid
    s = mk(grid, kernel)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    rng = np.random.default_rng(L)
    f, g, h = (rng.standard_normal((P, N)) for _ in range(3))
    for lcut in (L, max(L - 7, 1)):
        close(s.scal_to_SH(f, lcut), o.scal_to_SH(f, lcut))
        close(np.array(s.spat_to_qst(f, g, h, lcut)), np.array(o.spat_to_qst(f, g, h, lcut)))
        close(np.array(s.spat_to_sphertor(g, h, lcut)), np.array(o.spat_to_sphertor(g, h, lcut)))
    s.device_status()


@pytest.mark.parametrize("grid", [(31, 1, 48, 96), (64, 4, 96, 48), (63, 1, 96, 192)])
def test_fp64tc_radial_loop_set_matches_oracle(built, oracle_mod, torch, grid):
    """The batched radial-loop set (15 grids from 13 spectra, then 10 spectra
    from the grids) on device arrays, every output against the oracle."""
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P = grid
    n = 5
    s = mk(grid, 0)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    spec_in = grid_space_inputs(L, minc, n, seed=42)
    or2 = or2_levels(n)
    lcut = np.array([L, L - 1, L, max(L - 9, 1), L], dtype=np.int32)
    ref = _radial_set_ref(o, spec_in, or2, lcut)
    din = {k: torch.from_numpy(v).cuda() for k, v in spec_in.items()}
    got = s.transform_to_grid_space(din, or2=or2, lcut=lcut)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in got.items()}
    for k in ref:
        close(got[k], ref[k])  # the synthesis grids meet 1e-12
    fwd_in = {k: got[v] for k, v in FORWARD_FROM_INVERSE.items()}
    lm = s.transform_to_lm_space({k: torch.from_numpy(v).cuda() for k, v in fwd_in.items()}, lcut=lcut)
    torch.cuda.synchronize()
    lm = {k: v.cpu().numpy() for k, v in lm.items()}
    for r in range(n):
        lc = int(lcut[r])
        for pre in ("Adv", "VS", "VxB"):
            ref3 = o.spat_to_qst(fwd_in[pre + "r"][r], fwd_in[pre + "t"][r], fwd_in[pre + "p"][r], lc)
            got3 = [lm[pre + c + "LM"][r] for c in "rtp"]
            for a, b in zip(got3, ref3):
                close(a, b, tol=1e-11)
            num = sum(np.sum(np.abs(a - b) ** 2) for a, b in zip(got3, ref3)) ** 0.5
            assert num / sum(np.sum(np.abs(b) ** 2) for b in ref3) ** 0.5 <= 1e-13, pre
        close(lm["heatTermsLM"][r], o.scal_to_SH(fwd_in["heatTerms"][r], lc))
    s.device_status()


def test_fp64tc_full_size_levels_match_fp64_form(built, torch):
    """The bench workload's grid (l_max = 255, 384 x 768) on 8 levels of the
    radial set, against the FP64 form: every output field <= 1e-11, every
    call normwise <= 1e-13, and the synthesis grids <= 1e-13 each."""
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P, n = 255, 1, 384, 768, 8
    spec_np = grid_space_inputs(L, minc, n, seed=3)
    d = {k: torch.from_numpy(v).cuda() for k, v in spec_np.items()}
    or2 = torch.from_numpy(or2_levels(n)).cuda()
    s64 = make(L, minc, N, P, prec="fp64")
    stc = make(L, minc, N, P, prec="fp64tc")
    g64 = s64.transform_to_grid_space(d, or2=or2)
    gtc = stc.transform_to_grid_space(d, or2=or2)
    fwd = {k: g64[v] for k, v in FORWARD_FROM_INVERSE.items()}
    l64 = s64.transform_to_lm_space(fwd)
    ltc = stc.transform_to_lm_space(fwd)
    torch.cuda.synchronize()
    stc.device_status()
    for a, b, tol in ((gtc, g64, 1e-13), (ltc, l64, 1e-11)):
        for k in b:
            e = float(torch.linalg.vector_norm(a[k] - b[k]) / torch.linalg.vector_norm(b[k]))
            assert e <= tol, (k, e)
    for pre in ("Adv", "VS", "VxB"):
        ks = [pre + c + "LM" for c in "rtp"]
        num = sum(float(torch.linalg.vector_norm(ltc[k] - l64[k])) ** 2 for k in ks) ** 0.5
        den = sum(float(torch.linalg.vector_norm(l64[k])) ** 2 for k in ks) ** 0.5
        assert num / den <= 1e-13, (pre, num / den)


def test_fp64tc_round_trip_full_size(built, torch):
    """spectral -> grid -> spectral identity at l_max = 255 (Gauss quadrature
    is exact for band-limited input)."""
    from magic_gb300.workload import spectra
    s = make(255, 1, 384, 768, prec="fp64tc")
    S = spectra(255, 1, 3, seed=77)
    S[:, 0] = 0
    ell = s.lm2l
    d = [torch.from_numpy(x).cuda() for x in S]
    q, ss, t = s.spat_to_qst(*s.torpol_to_spat(d[0], d[1], d[2]))
    torch.cuda.synchronize()
    assert rel_l2(q.cpu().numpy(), ell * (ell + 1) * S[0]) < 1e-12
    assert rel_l2(ss.cpu().numpy(), S[1]) < 1e-12
    assert rel_l2(t.cpu().numpy(), S[2]) < 1e-12
    back = s.scal_to_SH(s.scal_to_spat(d[0]))
    torch.cuda.synchronize()
    assert rel_l2(back.cpu().numpy(), S[0]) < 1e-12
