"""The runtime knobs of a handle (magic_sht_set_tuning) on the GPU: the FP32
azimuthal FFTs at 8 and at 16 theta rows per CTA give identical grids and
spectra equal to FP32 rounding (the forward FFT factors its twiddles at the
rows' stride), and both settings stay within the form's tolerance of the
oracle; the tile orders of the persistent tensor-core kernels give
identical results."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


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


def _pair(torch, s, spec, or2):
    from magic_gb300.workload import FORWARD_FROM_INVERSE
    gr = s.transform_to_grid_space(spec, or2=or2)
    lm = s.transform_to_lm_space({k: gr[v] for k, v in FORWARD_FROM_INVERSE.items()})
    torch.cuda.synchronize()
    return gr, lm


@pytest.mark.parametrize("prec", ["fp32", "bf16x3"])
def test_fft_rows_settings_agree(built, oracle_mod, torch, prec):
    from magic_gb300 import SHT
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P, n = 63, 1, 96, 192, 4
    s = SHT(L, minc, N, P, precision=prec, device=0)
    spec_np = grid_space_inputs(L, minc, n, seed=17)
    spec = {k: torch.from_numpy(v).cuda() for k, v in spec_np.items()}
    or2 = torch.from_numpy(or2_levels(n)).cuda()
    res = {}
    for rows in (16, 8):
        s.set_tuning(fft_rows=rows)
        res[rows] = _pair(torch, s, spec, or2)
    for k in res[16][0]:
        assert torch.equal(res[16][0][k], res[8][0][k]), k
    for k in res[16][1]:
        a, b = res[16][1][k], res[8][1][k]
        assert float((a - b).abs().max() / a.abs().max()) < 2e-6, k
    # both settings against the oracle (well-conditioned outputs)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    for rows in (16, 8):
        gr, lm = res[rows]
        for r in range(n):
            ref = o.scal_to_spat(spec_np["s"][r], L)
            assert rel_l2(gr["sc"][r].cpu().numpy(), ref) < 2e-6
            fin = gr[FORWARD_FROM_INVERSE["heatTerms"]][r].cpu().numpy()
            assert rel_l2(lm["heatTermsLM"][r].cpu().numpy(), o.scal_to_SH(fin, L)) < 2e-6
    s.device_status()
    s.close()


@pytest.mark.parametrize("prec", ["bf16x3", "fp64tc"])
def test_tile_orders_agree(built, torch, prec):
    from magic_gb300 import SHT
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 127, 1, 192, 384, 3
    s = SHT(L, minc, N, P, precision=prec, device=0)
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=18).items()}
    or2 = torch.from_numpy(or2_levels(n)).cuda()
    res = {}
    for order in (0, 1):
        s.set_tuning(tc_order=order)
        res[order] = _pair(torch, s, spec, or2)
    for i in (0, 1):
        for k in res[0][i]:
            assert torch.equal(res[0][i][k], res[1][i][k]), (i, k)
    s.device_status()
    s.close()
