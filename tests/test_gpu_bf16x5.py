"""The five-digit tensor-core form (precision "bf16x5": five fixed-point BF16
digits per operand, 15 digit products accumulated exactly in FP32 on tcgen05,
the double-float FFTs and half spectra of the seven-digit form) against the
oracle and the FP64 form.

The dropped digits and products leave an error near 2^-39 of each table
row's and data column's scale.  Measured on GB300: 1e-11 to 6e-11 relative
L2 per routine on the parity grids and up to 3.3e-10 on the spheroidal and
toroidal outputs of spat_to_qst at l_max = 255 (the spheroidal part of the
curl is ~600x smaller than its partners); on the bench workload every call
within 6e-11 normwise of the FP64 form.  The tests hold every routine to
1e-9 relative L2 (1e-8 relative max), every radial-set output at l_max = 255
to 1e-6 and every call there to 1e-9 normwise."""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import GRIDS, close, make, spec

pytestmark = pytest.mark.gpu
TOL5 = 1e-9


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


@pytest.mark.parametrize("grid", GRIDS)
def test_bf16x5_routines_match_oracle(built, oracle_mod, torch, grid):
    L, minc, N, P = grid
    s = make(*grid, prec="bf16x5")
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = spec(o, 4, seed=L + minc)
    for lcut in (L, max(L - 5, 1)):
        close(s.scal_to_spat(S[0], lcut), o.scal_to_spat(S[0], lcut), tol=TOL5)
        close(np.array(s.scal_to_grad_spat(S[0], lcut)), np.array(o.scal_to_grad_spat(S[0], lcut)), tol=TOL5)
        close(np.array(s.torpol_to_spat(S[0], S[1], S[2], lcut)),
              np.array(o.torpol_to_spat(S[0], S[1], S[2], lcut)), tol=TOL5)
        close(np.array(s.torpol_to_curl_spat(0.83, S[0], S[3], S[1], S[2], lcut)),
              np.array(o.torpol_to_curl_spat(0.83, S[0], S[3], S[1], S[2], lcut)), tol=TOL5)
    rng = np.random.default_rng(L)
    f, g, h = (rng.standard_normal((P, N)) for _ in range(3))
    for lcut in (L, max(L - 7, 1)):
        close(s.scal_to_SH(f, lcut), o.scal_to_SH(f, lcut), tol=TOL5)
        close(np.array(s.spat_to_qst(f, g, h, lcut)), np.array(o.spat_to_qst(f, g, h, lcut)), tol=TOL5)
        close(np.array(s.spat_to_sphertor(g, h, lcut)), np.array(o.spat_to_sphertor(g, h, lcut)), tol=TOL5)
    s.device_status()


def test_bf16x5_full_size_levels_match_fp64_form(built, torch):
    """The bench workload's grid (l_max = 255, 384 x 768) on 8 levels of the
    radial set against the FP64 form: every synthesis grid <= 1e-9, every
    analysis output <= 1e-6, every call normwise <= 1e-9."""
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P, n = 255, 1, 384, 768, 8
    d = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=3).items()}
    or2 = torch.from_numpy(or2_levels(n)).cuda()
    s64 = make(L, minc, N, P, prec="fp64")
    s5 = make(L, minc, N, P, prec="bf16x5")
    g64 = s64.transform_to_grid_space(d, or2=or2)
    g5 = s5.transform_to_grid_space(d, or2=or2)
    fwd = {k: g64[v] for k, v in FORWARD_FROM_INVERSE.items()}
    l64 = s64.transform_to_lm_space(fwd)
    l5 = s5.transform_to_lm_space(fwd)
    torch.cuda.synchronize()
    s5.device_status()
    for a, b, tol in ((g5, g64, TOL5), (l5, l64, 1e-6)):
        for k in b:
            e = float(torch.linalg.vector_norm(a[k] - b[k]) / torch.linalg.vector_norm(b[k]))
            assert e <= tol, (k, e)
    for pre in ("Adv", "VS", "VxB"):
        ks = [pre + c + "LM" for c in "rtp"]
        num = sum(float(torch.linalg.vector_norm(l5[k] - l64[k])) ** 2 for k in ks) ** 0.5
        den = sum(float(torch.linalg.vector_norm(l64[k])) ** 2 for k in ks) ** 0.5
        assert num / den <= TOL5, (pre, num / den)


def test_bf16x5_round_trip_full_size(built, torch):
    """spectral -> grid -> spectral identity at l_max = 255."""
    from magic_gb300.workload import spectra
    s = make(255, 1, 384, 768, prec="bf16x5")
    S = spectra(255, 1, 3, seed=77)
    S[:, 0] = 0
    ell = s.lm2l
    d = [torch.from_numpy(x).cuda() for x in S]
    q, ss, t = s.spat_to_qst(*s.torpol_to_spat(d[0], d[1], d[2]))
    torch.cuda.synchronize()
    assert rel_l2(q.cpu().numpy(), ell * (ell + 1) * S[0]) < TOL5
    assert rel_l2(ss.cpu().numpy(), S[1]) < TOL5
    assert rel_l2(t.cpu().numpy(), S[2]) < TOL5
