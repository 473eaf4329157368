"""GPU parity: every public transform of the CUDA library (through the C ABI)
against the oracle on the same seeded inputs, and against the committed
golden vectors.  FP64 form: relative L2 and max error <= 1e-12.  FP32 form:
<= 2e-6 relative L2."""
import os

import numpy as np
import pytest

from conftest import rel_l2, rel_max

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12

GRIDS = [  # (l_max, minc, n_theta, n_phi_max)
    (15, 1, 24, 48),      # generic Stockham FFT path (n = 24)
    (31, 1, 48, 96),      # fast path S=1... (n = 48 -> generic), small
    (64, 4, 96, 48),      # minc = 4 like the reference sample boussBenchSat
    (63, 1, 96, 192),     # fast path S=3
    (64, 1, 96, 192),     # C0 grid
    (42, 2, 64, 128),     # fast path S=2 with minc=2
    (128, 1, 192, 384),   # C1 grid, fast path S=6
]


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


def make(L, minc, N, P, prec="fp64", nlat=0):
    from magic_gb300 import SHT
    return SHT(L, minc, N, P, precision=prec, nlat_padded=nlat, device=0)


def spec(o, n, seed):
    from magic_gb300.workload import spectra
    return spectra(o.l_max, o.minc, n, seed, m_max=o.m_max)


def close(a, b, tol=TOL64):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, (a.shape, b.shape)
    e2, em = rel_l2(a, b), rel_max(a, b)
    assert e2 <= tol and em <= 10 * tol, (e2, em)
    return e2


@pytest.mark.parametrize("grid", GRIDS)
def test_inverse_routines_match_oracle(built, oracle_mod, torch, grid):
    L, minc, N, P = grid
    s = make(*grid)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = spec(o, 4, seed=L + minc)
    for lcut in (L, max(L - 5, 1)):
        close(s.scal_to_spat(S[0], lcut), o.scal_to_spat(S[0], lcut))
        close(s.pol_to_curlr_spat(S[1], lcut), o.pol_to_curlr_spat(S[1], lcut))
        close(np.array(s.scal_to_grad_spat(S[0], lcut)), np.array(o.scal_to_grad_spat(S[0], lcut)))
        close(np.array(s.pol_to_grad_spat(S[2], lcut)), np.array(o.pol_to_grad_spat(S[2], lcut)))
        close(np.array(s.torpol_to_spat(S[0], S[1], S[2], lcut)),
              np.array(o.torpol_to_spat(S[0], S[1], S[2], lcut)))
        close(np.array(s.sphtor_to_spat(S[1], S[2], lcut)), np.array(o.sphtor_to_spat(S[1], S[2], lcut)))
        close(np.array(s.torpol_to_dphspat(S[1], S[2], lcut)),
              np.array(o.torpol_to_dphspat(S[1], S[2], lcut)))
        close(np.array(s.torpol_to_curl_spat(0.83, S[0], S[3], S[1], S[2], lcut)),
              np.array(o.torpol_to_curl_spat(0.83, S[0], S[3], S[1], S[2], lcut)))
    close(np.array(s.torpol_to_spat_IC(0.3, 0.35, S[0], S[1], S[2])),
          np.array(o.torpol_to_spat_IC(0.3, 0.35, S[0], S[1], S[2])))
    close(np.array(s.torpol_to_curl_spat_IC(0.2, 0.35, S[0], S[1], S[2], S[3])),
          np.array(o.torpol_to_curl_spat_IC(0.2, 0.35, S[0], S[1], S[2], S[3])))
    close(s.axi_to_spat(S[0][: L + 1]), o.axi_to_spat(S[0][: L + 1]))
    close(np.array(s.toraxi_to_spat(S[1][: L + 1], L - 2)), np.array(o.toraxi_to_spat(S[1][: L + 1], L - 2)))


@pytest.mark.parametrize("grid", GRIDS)
def test_forward_routines_match_oracle(built, oracle_mod, torch, grid):
    L, minc, N, P = grid
    s = make(*grid)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    rng = np.random.default_rng(L)
    f, g, h = (rng.standard_normal((P, N)) for _ in range(3))
    for lcut in (L, max(L - 7, 1)):
        close(s.scal_to_SH(f, lcut), o.scal_to_SH(f, lcut))
        close(np.array(s.spat_to_qst(f, g, h, lcut)), np.array(o.spat_to_qst(f, g, h, lcut)))
        close(np.array(s.spat_to_sphertor(g, h, lcut)), np.array(o.spat_to_sphertor(g, h, lcut)))


def test_golden_vectors_on_gpu(built, torch):
    g = np.load(os.path.join(GOLD, "oracle_small.npz"))
    s = make(15, 1, 24, 48)
    S = g["s15_in"]
    close(s.scal_to_spat(S[0]), g["s15_scal"])
    close(s.scal_to_spat(S[0], 11), g["s15_scal_lcut11"])
    close(np.array(s.torpol_to_spat(S[0], S[1], S[2])), g["s15_qst"])
    close(np.array(s.torpol_to_curl_spat(0.7, S[0], S[3], S[1], S[2])), g["s15_curl"])
    close(np.array(s.sphtor_to_spat(S[1], S[2])), g["s15_sphtor"])
    close(np.array(s.scal_to_grad_spat(S[0])), g["s15_grad"])
    close(np.array(s.torpol_to_dphspat(S[1], S[2])), g["s15_dph"])
    q = g["s15_qst"]
    close(np.array(s.spat_to_qst(q[0], q[1], q[2])), g["s15_fwd_qst"])
    close(s.scal_to_SH(q[0], 11), g["s15_fwd_sh_lcut11"])
    cp = np.load(os.path.join(GOLD, "checkpoint_spectra.npz"))
    L, minc, N, P = [int(x) for x in g["cp_dims"]]
    s = make(L, minc, N, P)
    w, z, sc = cp["wpol"][2], cp["ztor"][2], cp["entropy"][2]
    close(s.scal_to_spat(sc), g["cp_scal"])
    close(np.array(s.torpol_to_spat(w, w, z)), g["cp_qst"])
    qq = g["cp_qst"]
    close(np.array(s.spat_to_qst(qq[0], qq[1], qq[2])), g["cp_fwd_qst"])


def _radial_set_ref(o, spec_in, or2, lcut):
    n = spec_in["w"].shape[0]
    out = {k: [] for k in ("sc", "pc", "xic", "vrc", "vtc", "vpc", "cvrc", "cvtc", "cvpc",
                           "brc", "btc", "bpc", "cbrc", "cbtc", "cbpc")}
    for r in range(n):
        lc = int(lcut[r])
        out["sc"].append(o.scal_to_spat(spec_in["s"][r], lc))
        out["pc"].append(o.scal_to_spat(spec_in["p"][r], lc))
        out["xic"].append(o.scal_to_spat(spec_in["xi"][r], lc))
        for k, v in zip(("vrc", "vtc", "vpc"),
                        o.torpol_to_spat(spec_in["w"][r], spec_in["dw"][r], spec_in["z"][r], lc)):
            out[k].append(v)
        for k, v in zip(("cvrc", "cvtc", "cvpc"),
                        o.torpol_to_curl_spat(or2[r], spec_in["w"][r], spec_in["ddw"][r], spec_in["z"][r],
                                              spec_in["dz"][r], lc)):
            out[k].append(v)
        for k, v in zip(("brc", "btc", "bpc"),
                        o.torpol_to_spat(spec_in["b"][r], spec_in["db"][r], spec_in["aj"][r], lc)):
            out[k].append(v)
        for k, v in zip(("cbrc", "cbtc", "cbpc"),
                        o.torpol_to_curl_spat(or2[r], spec_in["b"][r], spec_in["ddb"][r], spec_in["aj"][r],
                                              spec_in["dj"][r], lc)):
            out[k].append(v)
    return {k: np.array(v) for k, v in out.items()}


@pytest.mark.parametrize("grid", [(31, 1, 48, 96), (64, 4, 96, 48), (63, 1, 96, 192)])
@pytest.mark.parametrize("device_ptrs", [False, True])
def test_radial_loop_set_matches_oracle(built, oracle_mod, torch, grid, device_ptrs):
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P = grid
    n = 5
    s = make(*grid)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    spec_in = grid_space_inputs(L, minc, n, seed=42)
    or2 = or2_levels(n)
    lcut = np.array([L, L - 1, L, max(L - 9, 1), L], dtype=np.int32)
    ref = _radial_set_ref(o, spec_in, or2, lcut)
    if device_ptrs:
        din = {k: torch.from_numpy(v).cuda() for k, v in spec_in.items()}
        got = s.transform_to_grid_space(din, or2=or2, lcut=lcut)
        torch.cuda.synchronize()
        got = {k: v.cpu().numpy() for k, v in got.items()}
    else:
        got = s.transform_to_grid_space(spec_in, or2=or2, lcut=lcut)
    for k in ref:
        close(got[k], ref[k])
    # grid -> spectral on the same levels
    fwd_in = {k: got[v] for k, v in FORWARD_FROM_INVERSE.items()}
    if device_ptrs:
        lm = s.transform_to_lm_space({k: torch.from_numpy(v).cuda() for k, v in fwd_in.items()}, lcut=lcut)
        torch.cuda.synchronize()
        lm = {k: v.cpu().numpy() for k, v in lm.items()}
    else:
        lm = s.transform_to_lm_space(fwd_in, lcut=lcut)
    for r in range(n):
        lc = int(lcut[r])
        for pre in ("Adv", "VS", "VxB"):
            q, ss, t = o.spat_to_qst(fwd_in[pre + "r"][r], fwd_in[pre + "t"][r], fwd_in[pre + "p"][r], lc)
            close(lm[pre + "rLM"][r], q)
            close(lm[pre + "tLM"][r], ss)
            close(lm[pre + "pLM"][r], t)
        close(lm["heatTermsLM"][r], o.scal_to_SH(fwd_in["heatTerms"][r], lc))


def test_padded_grids(built, oracle_mod, torch):
    L, minc, N, P = 31, 1, 48, 96
    s = make(L, minc, N, P, nlat=52)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = spec(o, 3, 1)
    vr, vt, vp = s.torpol_to_spat(S[0], S[1], S[2])
    assert vr.shape == (P, 52)
    rr = o.torpol_to_spat(S[0], S[1], S[2])
    close(np.array([vr[:, :N], vt[:, :N], vp[:, :N]]), np.array(rr))
    g = np.zeros((P, 52))
    g[:, :N] = rr[0]
    close(s.scal_to_SH(g), o.scal_to_SH(rr[0]))


def test_round_trip_identity_full_size(built, torch):
    """Size-independent property at the precision-form grid (l_max=255)."""
    from magic_gb300.workload import spectra
    s = make(255, 1, 384, 768)
    S = spectra(255, 1, 3, seed=77)
    S[:, 0] = 0
    ell = s.lm2l
    d = [torch.from_numpy(x).cuda() for x in S]
    q, ss, t = s.spat_to_qst(*s.torpol_to_spat(d[0], d[1], d[2]))
    torch.cuda.synchronize()
    assert rel_l2(q.cpu().numpy(), ell * (ell + 1) * S[0]) < 1e-12
    assert rel_l2(ss.cpu().numpy(), S[1]) < 1e-12
    assert rel_l2(t.cpu().numpy(), S[2]) < 1e-12
    f = s.scal_to_spat(d[0])
    back = s.scal_to_SH(f)
    torch.cuda.synchronize()
    assert rel_l2(back.cpu().numpy(), S[0]) < 1e-12


def test_fp32_form(built, oracle_mod, torch):
    L, minc, N, P = 63, 1, 96, 192
    s = make(L, minc, N, P, prec="fp32")
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = spec(o, 3, 5)
    for a, b in zip(s.torpol_to_spat(S[0], S[1], S[2]), o.torpol_to_spat(S[0], S[1], S[2])):
        assert rel_l2(a, b) < 2e-6
    g = o.torpol_to_spat(S[0], S[1], S[2])
    for a, b in zip(s.spat_to_qst(*g), o.spat_to_qst(*g)):
        assert rel_l2(a, b) < 2e-6


def test_graph_replay_matches_direct(built, torch):
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 63, 1, 96, 192, 6
    s = make(L, minc, N, P)
    spec_in = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=3).items()}
    or2 = torch.from_numpy(or2_levels(n)).cuda()
    ref = s.transform_to_grid_space(spec_in, or2=or2)
    torch.cuda.synchronize()
    out = {k: torch.zeros_like(v) for k, v in ref.items()}
    s.reserve(n)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):  # capture needs a non-default stream
        s.graph_begin()
        s.transform_to_grid_space(spec_in, or2=or2, out=out)
        gr = s.graph_end()
        s.graph_launch(gr)
        s.synchronize()
    for k in ref:
        assert torch.equal(out[k], ref[k]), k
    s.graph_destroy(gr)


def test_zero_levels_are_no_ops(built, torch):
    """n_levels = 0 on every batched entry point: status OK, nothing written
    (host and device arrays)."""
    from magic_gb300.workload import grid_space_inputs, FORWARD_FROM_INVERSE
    s = make(31, 1, 48, 96)
    for dev in (False, True):
        spec_in = {k: v[:0] for k, v in grid_space_inputs(31, 1, 2, seed=1).items()}
        if dev:
            spec_in = {k: torch.from_numpy(v).cuda() for k, v in spec_in.items()}
        g = s.transform_to_grid_space(spec_in, derivatives=True)
        assert all(v.shape[0] == 0 for v in g.values()) and "dvrdrc" in g
        lm = s.transform_to_lm_space({k: g[v] for k, v in FORWARD_FROM_INVERSE.items()})
        assert all(v.shape[0] == 0 for v in lm.values())
    s.device_status()


def test_error_codes(built, torch):
    from magic_gb300._lib import ShtError
    s = make(31, 1, 48, 96)
    S = np.zeros(s.lm_max, complex)
    with pytest.raises(ShtError) as e:
        s.scal_to_spat(S, 40)
    assert e.value.code == 3
    with pytest.raises(ShtError) as e:
        s.scal_to_spat(S, -1)
    assert e.value.code == 3


@pytest.mark.parametrize("grid", [(63, 1, 96, 192), (64, 4, 96, 48), (128, 1, 192, 384)])
def test_bf16x3_form_matches_oracle(built, oracle_mod, torch, grid):
    """Tensor-core form (3xBF16 split products, FP32 accumulation, FP32 FFT):
    relative L2 against the FP64 oracle within 2e-6 on well-conditioned outputs."""
    L, minc, N, P = grid
    s = make(L, minc, N, P, prec="bf16x3")
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = spec(o, 4, 17)
    for a, b in zip(s.torpol_to_spat(S[0], S[1], S[2]), o.torpol_to_spat(S[0], S[1], S[2])):
        assert rel_l2(a, b) < 2e-6
    assert rel_l2(s.scal_to_spat(S[3], L - 3), o.scal_to_spat(S[3], L - 3)) < 2e-6
    for a, b in zip(s.sphtor_to_spat(S[1], S[2]), o.sphtor_to_spat(S[1], S[2])):
        assert rel_l2(a, b) < 2e-6
    g = o.torpol_to_spat(S[0], S[1], S[2])
    for a, b in zip(s.spat_to_qst(*g), o.spat_to_qst(*g)):
        assert rel_l2(a, b) < 2e-6
    assert rel_l2(s.scal_to_SH(g[0], L - 2), o.scal_to_SH(g[0], L - 2)) < 2e-6
    s.device_status()


def test_bf16x3_full_size_levels(built, torch):
    """Precision-form grid (l_max=255, 384 x 768): the tensor-core form against
    the FP64 form on 3 radial levels of the full transform set; every output
    finite and within 2e-6 relative L2 except the ill-conditioned spheroidal
    part of the vorticity-derived pair."""
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    n = 3
    s64 = make(255, 1, 384, 768)
    sbf = make(255, 1, 384, 768, prec="bf16x3")
    spec_in = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(255, 1, n, seed=5).items()}
    or2 = torch.from_numpy(or2_levels(n)).cuda()
    g64 = s64.transform_to_grid_space(spec_in, or2=or2)
    gbf = sbf.transform_to_grid_space(spec_in, or2=or2)
    l64 = s64.transform_to_lm_space({k: g64[v] for k, v in FORWARD_FROM_INVERSE.items()})
    lbf = sbf.transform_to_lm_space({k: g64[v] for k, v in FORWARD_FROM_INVERSE.items()})
    torch.cuda.synchronize()
    sbf.device_status()
    for k in g64:
        assert torch.isfinite(gbf[k]).all(), k
        e = float(torch.linalg.vector_norm(gbf[k] - g64[k]) / torch.linalg.vector_norm(g64[k]))
        assert e < 2e-6, (k, e)
    for k in l64:
        assert torch.isfinite(lbf[k]).all(), k
        e = float(torch.linalg.vector_norm(lbf[k] - l64[k]) / torch.linalg.vector_norm(l64[k]))
        assert e < (1e-3 if k == "VStLM" else 2e-6), (k, e)


@pytest.mark.parametrize("prec", ["fp64", "bf16x3"])
def test_pipelined_host_levels_match_device_call(built, torch, prec):
    """Host arrays with more levels than one pipeline chunk go through the
    chunked copy/compute pipeline; results equal the device-pointer call."""
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P, n = 63, 1, 96, 192, 19
    s = make(L, minc, N, P, prec=prec)
    spec_np = grid_space_inputs(L, minc, n, seed=8)
    or2 = or2_levels(n)
    lcut = np.full(n, L, dtype=np.int32)
    lcut[3] = L - 11
    pin = {k: torch.from_numpy(v).pin_memory() for k, v in spec_np.items()}
    host = s.transform_to_grid_space(pin, or2=or2, lcut=lcut)
    dev = s.transform_to_grid_space({k: v.cuda() for k, v in pin.items()}, or2=or2, lcut=lcut)
    torch.cuda.synchronize()
    for k in dev:
        assert torch.equal(host[k], dev[k].cpu()), k
    fin = {k: host[v] for k, v in FORWARD_FROM_INVERSE.items()}
    lh = s.transform_to_lm_space(fin, lcut=lcut)
    ld = s.transform_to_lm_space({k: v.cuda() for k, v in fin.items()}, lcut=lcut)
    torch.cuda.synchronize()
    for k in ld:
        assert torch.equal(lh[k], ld[k].cpu()), k
    # pageable numpy arrays take the same path
    hn = s.transform_to_grid_space(spec_np, or2=or2, lcut=lcut)
    for k in dev:
        assert np.array_equal(hn[k], dev[k].cpu().numpy()), k


@pytest.mark.gpu
@pytest.mark.parametrize("grid", [(63, 1, 96, 192), (64, 4, 96, 48), (255, 1, 384, 768)])
def test_persistent_tensor_core_kernels_match_tiled(built, torch, grid, monkeypatch):
    """The persistent tensor-core kernels (stacked split products) and the
    one-tile-per-CTA kernels both stay within the 3xBF16 tolerance of the FP64
    form on the radial-loop set (ragged lcut and the odd-parity m = l_max
    tile included), and agree with each other."""
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P = grid
    n = 5 if L > 200 else 11
    spec_np = grid_space_inputs(L, minc, n, seed=21)
    or2 = or2_levels(n)
    lcut = np.full(n, L, dtype=np.int32)
    lcut[1] = L - 7
    spec_d = {k: torch.from_numpy(v).cuda() for k, v in spec_np.items()}
    out = {}
    for kern, prec in (("tiled", "fp64"), ("tiled", "bf16x3"), ("persistent", "bf16x3")):
        monkeypatch.setenv("MAGIC_SHT_TC_KERNEL", kern)
        s = make(L, minc, N, P, prec=prec)
        g = s.transform_to_grid_space(spec_d, or2=or2, lcut=lcut)
        if prec == "fp64":
            fin = {k: g[v] for k, v in FORWARD_FROM_INVERSE.items()}
        lm = s.transform_to_lm_space(fin, lcut=lcut)  # same grid inputs for every form
        torch.cuda.synchronize()
        s.device_status()
        out[(kern, prec)] = {**{k: v.cpu() for k, v in g.items()}, **{k: v.cpu() for k, v in lm.items()}}
    ref = out[("tiled", "fp64")]
    flat = lambda t: (torch.view_as_real(t) if t.is_complex() else t).numpy().ravel()
    for k in ref:
        tol = 1e-3 if k == "VStLM" else 2e-6  # VStLM: small output of a near-cancelling pair
        a = flat(out[("tiled", "bf16x3")][k])
        b = flat(out[("persistent", "bf16x3")][k])
        r = flat(ref[k])
        assert rel_l2(a, r) < tol, (k, rel_l2(a, r))
        assert rel_l2(b, r) < tol, (k, rel_l2(b, r))
        assert rel_l2(b, a) < 2 * tol, (k, rel_l2(b, a))


@pytest.mark.gpu
@pytest.mark.parametrize("grid", [(63, 1, 96, 192), (255, 1, 384, 768)])
def test_get_nl_matches_oracle(built, oracle_mod, torch, grid):
    """Grid-space nonlinear products on the GPU against the numpy restatement
    of get_nl.f90 (FP64, every output, two radial levels with different r)."""
    from oracle import oracle as orc
    from magic_gb300 import _lib
    L, minc, N, P = grid
    n = 3
    s = make(L, minc, N, P)
    rng = np.random.default_rng(5)
    grids = {k: torch.from_numpy(rng.standard_normal((n, P, N))).cuda() for k in _lib.NL_IN}
    or2 = np.array([1.0, 0.37, 2.5])
    out = s.get_nl(grids, or2=or2)
    torch.cuda.synchronize()
    ref = orc.get_nl({k: v.cpu().numpy() for k, v in grids.items()}, or2, N)
    for k in _lib.LM_SPACE_IN:
        assert rel_l2(out[k].cpu().numpy(), ref[k]) < 1e-13, k


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["bf16x3", "tf32x2", "fp32"])
def test_get_nl_reduced_forms_compute_in_fp32(built, oracle_mod, torch, form):
    """On a reduced-precision handle get_nl computes in FP32 (FP64 grids in
    and out): every product within 1e-6 relative L2 of the FP64 restatement,
    and not bit-identical to it (the FP32 kernel ran)."""
    from oracle import oracle as orc
    from magic_gb300 import _lib
    L, minc, N, P = 63, 1, 96, 192
    n = 3
    s = make(L, minc, N, P, prec=form)
    rng = np.random.default_rng(5)
    grids = {k: torch.from_numpy(rng.standard_normal((n, P, N))).cuda() for k in _lib.NL_IN}
    or2 = np.array([1.0, 0.37, 2.5])
    out = s.get_nl(grids, or2=or2)
    torch.cuda.synchronize()
    ref = orc.get_nl({k: v.cpu().numpy() for k, v in grids.items()}, or2, N)
    for k in _lib.LM_SPACE_IN:
        e = rel_l2(out[k].cpu().numpy(), ref[k])
        assert 0.0 < e < 1e-6, (k, e)
    s.close()


@pytest.mark.gpu
def test_get_nl_fp64_accurate_form_computes_in_double_float(built, oracle_mod, torch):
    """On an FP64-accurate handle get_nl computes in double-float arithmetic
    on the FP32 pipe (FP64 grids in and out, about 2^-48 per operation):
    every product within 1e-12 relative L2 of the FP64 restatement."""
    from oracle import oracle as orc
    from magic_gb300 import _lib
    L, minc, N, P = 63, 1, 96, 192
    n = 3
    s = make(L, minc, N, P, prec="fp64tc")
    rng = np.random.default_rng(5)
    grids = {k: torch.from_numpy(rng.standard_normal((n, P, N))).cuda() for k in _lib.NL_IN}
    or2 = np.array([1.0, 0.37, 2.5])
    out = s.get_nl(grids, or2=or2)
    torch.cuda.synchronize()
    ref = orc.get_nl({k: v.cpu().numpy() for k, v in grids.items()}, or2, N)
    for k in _lib.LM_SPACE_IN:
        e = rel_l2(out[k].cpu().numpy(), ref[k])
        assert e < 1e-12, (k, e)
    s.close()


@pytest.mark.gpu
def test_radial_step_with_nonlinear_products(built, torch):
    """The radial-loop step of rIter.f90:94-464 on the GPU: synthesis set,
    get_nl on the FP64 grids, analysis set.  Each vector analysis
    (spat_to_qst) of the 3xBF16 form is within 2e-6 of the FP64 form
    normwise over its three outputs, and every output field within 2e-6
    except AdvpLM: the toroidal part of the advection of these synthetic
    (mutually inconsistent) spectra is ~1e-3 of the field's other parts, so
    its own relative error is that much larger."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 127, 1, 192, 384, 6
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=17).items()}
    or2 = or2_levels(n)
    s64 = make(L, minc, N, P, prec="fp64")
    nl = s64.get_nl(s64.transform_to_grid_space(spec, or2=or2), or2=or2)
    res = {}
    for prec in ("fp64", "bf16x3"):
        s = s64 if prec == "fp64" else make(L, minc, N, P, prec=prec)
        lm = s.transform_to_lm_space(nl)
        torch.cuda.synchronize()
        res[prec] = {k: torch.view_as_real(v).cpu().numpy() for k, v in lm.items()}
    a, r = res["bf16x3"], res["fp64"]
    for pre in ("Adv", "VS", "VxB"):
        ks = [pre + c + "LM" for c in "rtp"]
        num = np.sqrt(sum(np.sum((a[k] - r[k]) ** 2) for k in ks))
        den = np.sqrt(sum(np.sum(r[k] ** 2) for k in ks))
        assert num / den < 2e-6, (pre, num / den)
    for k in r:
        tol = 2e-3 if k == "AdvpLM" else 2e-6
        assert rel_l2(a[k], r[k]) < tol, (k, rel_l2(a[k], r[k]))


@pytest.mark.gpu
def test_large_config_l511(built, oracle_mod, torch):
    """The large configuration (l_max=511, 768 x 1536 grid): the FP64 form
    against the oracle on one level of the radial set, the 3xBF16 form
    against the FP64 form on three levels (normwise per call <= 1e-6), and
    the FP64-accurate tensor-core form (its double-float FFTs at 24 points
    per lane) against the FP64 form: every call normwise <= 1e-12, every
    output <= 1e-9 (AdvpLM, the small toroidal part of the advection, sits
    near 3e-10 as at l_max = 255)."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 511, 1, 768, 1536, 3
    spec_np = grid_space_inputs(L, minc, n, seed=29)
    or2 = or2_levels(n)
    spec = {k: torch.from_numpy(v).cuda() for k, v in spec_np.items()}
    s64 = make(L, minc, N, P, prec="fp64")
    g64 = s64.transform_to_grid_space(spec, or2=or2)
    torch.cuda.synchronize()
    o = oracle_mod.OracleSHT(L, minc, N, P)
    vr, vt, vp = o.torpol_to_spat(spec_np["w"][1], spec_np["dw"][1], spec_np["z"][1])
    assert rel_l2(g64["vtc"][1].cpu().numpy(), vt) < 1e-12
    assert rel_l2(g64["vpc"][1].cpu().numpy(), vp) < 1e-12
    sc = o.scal_to_spat(spec_np["s"][1])
    assert rel_l2(g64["sc"][1].cpu().numpy(), sc) < 1e-12
    s16 = make(L, minc, N, P, prec="bf16x3")
    g16 = s16.transform_to_grid_space(spec, or2=or2)
    nl = s64.get_nl(g64, or2=or2)
    l64 = s64.transform_to_lm_space(nl)
    l16 = s16.transform_to_lm_space(nl)
    torch.cuda.synchronize()
    for name, ks, a, b in (("v", ("vrc", "vtc", "vpc"), g16, g64), ("b", ("brc", "btc", "bpc"), g16, g64),
                           ("VxB", ("VxBrLM", "VxBtLM", "VxBpLM"), l16, l64),
                           ("VS", ("VSrLM", "VStLM", "VSpLM"), l16, l64)):
        num = sum(float(torch.linalg.vector_norm(a[k] - b[k])) ** 2 for k in ks) ** 0.5
        den = sum(float(torch.linalg.vector_norm(b[k])) ** 2 for k in ks) ** 0.5
        assert num / den < 1e-6, (name, num / den)
    del s16, g16, l16
    stc = make(L, minc, N, P, prec="fp64tc")
    gtc = stc.transform_to_grid_space(spec, or2=or2)
    ltc = stc.transform_to_lm_space(nl)
    torch.cuda.synchronize()
    stc.device_status()
    for a, b in ((gtc, g64), (ltc, l64)):
        for k in b:
            e = float(torch.linalg.vector_norm(a[k] - b[k]) / torch.linalg.vector_norm(b[k]))
            assert e < 1e-9, (k, e)
    for a, b, ks in ((gtc, g64, ("vrc", "vtc", "vpc")), (gtc, g64, ("cvrc", "cvtc", "cvpc")),
                     (ltc, l64, ("AdvrLM", "AdvtLM", "AdvpLM")), (ltc, l64, ("VSrLM", "VStLM", "VSpLM")),
                     (ltc, l64, ("VxBrLM", "VxBtLM", "VxBpLM"))):
        num = sum(float(torch.linalg.vector_norm(a[k] - b[k])) ** 2 for k in ks) ** 0.5
        den = sum(float(torch.linalg.vector_norm(b[k])) ** 2 for k in ks) ** 0.5
        assert num / den < 1e-12, (ks, num / den)
    # the same handle with the FP64 SIMT Legendre sums (tc_kernel 1): FP64 half
    # spectra into and out of the same double-float FFTs, whose rounding alone
    # sets AdvpLM's 3e-10 (the same as with the tensor-core sums)
    stc.set_tuning(tc_kernel=1)
    g1 = stc.transform_to_grid_space(spec, or2=or2)
    l1 = stc.transform_to_lm_space(nl)
    torch.cuda.synchronize()
    for a, b in ((g1, g64), (l1, l64)):
        for k in b:
            e = float(torch.linalg.vector_norm(a[k] - b[k]) / torch.linalg.vector_norm(b[k]))
            assert e < (1e-9 if k == "AdvpLM" else 1e-12), ("tc_kernel 1", k, e)


@pytest.mark.gpu
def test_sixteen_instances_in_one_graph(built, torch):
    """Sixteen independent transform instances of mixed sizes (l_max in
    {63, 127, 255}, minc in {1, 4}, a fixed seeded list) captured together in
    one CUDA graph on one stream and replayed: every instance's grids equal
    its direct call."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    rng = np.random.default_rng(1234)
    insts = []
    for i in range(16):
        L = int(rng.choice([63, 127, 255]))
        minc = int(rng.choice([1, 4]))
        N = 3 * (L + 1) // 2
        P = 2 * N // minc
        n = int(rng.choice([3, 5, 9]))
        s = make(L, minc, N, P, prec="bf16x3")
        spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, n, seed=100 + i).items()}
        or2 = torch.from_numpy(or2_levels(n)).cuda()
        ref = s.transform_to_grid_space(spec, or2=or2)
        insts.append((s, spec, or2, ref, {k: torch.zeros_like(v) for k, v in ref.items()}, n))
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        for s, _, _, _, _, n in insts:
            s.reserve(n)
            s.set_stream(side.cuda_stream)  # bind before the capture (binding synchronizes)
        side.synchronize()
        insts[0][0].graph_begin()  # every handle is bound to this stream: one capture
        try:
            for s, spec, or2, _, out, _ in insts:
                s.transform_to_grid_space(spec, or2=or2, out=out)
        finally:
            gr = insts[0][0].graph_end()
        insts[0][0].graph_launch(gr)
        side.synchronize()
    for s, _, _, ref, out, _ in insts:
        s.device_status()
        for k in ref:
            assert torch.equal(out[k], ref[k]), k
    insts[0][0].graph_destroy(gr)


@pytest.mark.gpu
def test_async_host_batches_match_sync(built, torch):
    """With asynchronous host batches two consecutive pipelined calls overlap
    and, after synchronize(), give the same host results as synchronous calls."""
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    L, minc, N, P, n = 63, 1, 96, 192, 21
    s = make(L, minc, N, P, prec="bf16x3")
    spec = {k: torch.from_numpy(v).pin_memory() for k, v in grid_space_inputs(L, minc, n, seed=44).items()}
    or2 = or2_levels(n)
    ref_g = s.transform_to_grid_space(spec, or2=or2)
    fin = {k: ref_g[v].clone().pin_memory() for k, v in FORWARD_FROM_INVERSE.items()}
    ref_l = s.transform_to_lm_space(fin)
    out_g = {k: torch.zeros_like(v).pin_memory() for k, v in ref_g.items()}
    out_l = {k: torch.zeros_like(v).pin_memory() for k, v in ref_l.items()}
    s.set_host_async(True)
    for _ in range(2):
        s.transform_to_grid_space(spec, or2=or2, out=out_g)
        s.transform_to_lm_space(fin, out=out_l)
    s.synchronize()
    s.set_host_async(False)
    for k in ref_g:
        assert torch.equal(out_g[k], ref_g[k]), k
    for k in ref_l:
        assert torch.equal(out_l[k], ref_l[k]), k


@pytest.mark.gpu
@pytest.mark.parametrize("grid", [(63, 1, 96, 192), (64, 4, 96, 48), (128, 1, 192, 384)])
def test_tf32x2_form_matches_oracle(built, oracle_mod, torch, grid):
    """TF32 variant (2xTF32 split products hi*hi, hi*lo, lo*hi; FP32
    accumulation, FP32 FFT) against the FP64 oracle: relative L2 within 4e-6."""
    L, minc, N, P = grid
    s = make(L, minc, N, P, prec="tf32x2")
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = spec(o, 4, 17)
    for a, b in zip(s.torpol_to_spat(S[0], S[1], S[2]), o.torpol_to_spat(S[0], S[1], S[2])):
        assert rel_l2(a, b) < 4e-6
    assert rel_l2(s.scal_to_spat(S[3], L - 3), o.scal_to_spat(S[3], L - 3)) < 4e-6
    g = o.torpol_to_spat(S[0], S[1], S[2])
    for a, b in zip(s.spat_to_qst(*g), o.spat_to_qst(*g)):
        assert rel_l2(a, b) < 4e-6
    assert rel_l2(s.scal_to_SH(g[0], L - 2), o.scal_to_SH(g[0], L - 2)) < 4e-6
    s.device_status()


@pytest.mark.gpu
def test_tf32x2_full_size_radial_set(built, torch):
    """TF32 variant at l_max=255 (384 x 768), 3 levels of the radial set with
    get_nl analysis inputs: normwise per call within 1e-6 of the FP64 form."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    n = 3
    s64 = make(255, 1, 384, 768)
    s32 = make(255, 1, 384, 768, prec="tf32x2")
    spec_in = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(255, 1, n, seed=5).items()}
    or2 = or2_levels(n)
    g64 = s64.transform_to_grid_space(spec_in, or2=or2)
    g32 = s32.transform_to_grid_space(spec_in, or2=or2)
    nl = s64.get_nl(g64, or2=or2)
    l64 = s64.transform_to_lm_space(nl)
    l32 = s32.transform_to_lm_space(nl)
    torch.cuda.synchronize()
    s32.device_status()
    groups = [("vrc", "vtc", "vpc"), ("cvrc", "cvtc", "cvpc"), ("brc", "btc", "bpc"), ("cbrc", "cbtc", "cbpc"),
              ("sc",), ("pc",), ("xic",), ("AdvrLM", "AdvtLM", "AdvpLM"), ("VSrLM", "VStLM", "VSpLM"),
              ("VxBrLM", "VxBtLM", "VxBpLM"), ("heatTermsLM",)]
    a, b = {**g32, **l32}, {**g64, **l64}
    for ks in groups:
        num = sum(float(torch.linalg.vector_norm(a[k] - b[k])) ** 2 for k in ks) ** 0.5
        den = sum(float(torch.linalg.vector_norm(b[k])) ** 2 for k in ks) ** 0.5
        assert num / den < 1e-6, (ks, num / den)


@pytest.mark.gpu
@pytest.mark.parametrize("grid", [(63, 1, 96, 192), (64, 4, 96, 48), (255, 1, 384, 768)])
def test_get_td_matches_oracle(built, torch, grid):
    """Spectral assembly of the time derivatives on the GPU against the numpy
    restatement of get_td.f90 (FP64; ragged l_R, internal heating)."""
    from oracle import oracle as orc
    from magic_gb300 import _lib
    L, minc, N, P = grid
    s = make(L, minc, N, P)
    n = 4
    rng = np.random.default_rng(9)
    spec = {k: torch.from_numpy(rng.standard_normal((n, s.lm_max)) + 1j * rng.standard_normal((n, s.lm_max))).cuda()
            for k in _lib.TD_IN}
    r = np.array([0.6, 0.9, 1.2, 1.5])
    lcut = np.array([L, L - 3, L, 1], dtype=np.int32)
    epsc = np.array([0.0, 0.5, -1.0, 2.0])
    out = s.get_td(spec, r, cor_fac=2.0e3, lcut=lcut, epsc=epsc)
    torch.cuda.synchronize()
    ref = orc.get_td({k: v.cpu().numpy() for k, v in spec.items()}, r, 2.0e3, L, minc, lcut, epsc)
    for k in _lib.TD_OUT:
        got = out[k].cpu().numpy()
        assert rel_l2(got, ref[k]) < 1e-13, (k, rel_l2(got, ref[k]))


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["bf16x3", "fp32"])
def test_get_td_reduced_forms_compute_in_fp32(built, torch, form):
    """On a reduced-precision handle get_td computes in FP32 (FP64 spectra in
    and out): every output within 1e-6 relative L2 of the FP64 restatement,
    not bit-identical to it; device per-level arrays (r, lcut, epsc, nbc)
    give the same results as host ones."""
    from oracle import oracle as orc
    from magic_gb300 import _lib
    L, minc, N, P = 63, 1, 96, 192
    s = make(L, minc, N, P, prec=form)
    n = 4
    rng = np.random.default_rng(9)
    spec = {k: torch.from_numpy(rng.standard_normal((n, s.lm_max)) + 1j * rng.standard_normal((n, s.lm_max))).cuda()
            for k in _lib.TD_IN}
    r = np.array([0.6, 0.9, 1.2, 1.5])
    lcut = np.array([L, L - 3, L, 1], dtype=np.int32)
    epsc = np.array([0.0, 0.5, -1.0, 2.0])
    nbc = np.array([1, 0, 0, 2], dtype=np.int32)
    out = s.get_td(spec, r, cor_fac=2.0e3, lcut=lcut, epsc=epsc, nbc=nbc)
    dev = s.get_td(spec, torch.from_numpy(r).cuda(), cor_fac=2.0e3, lcut=torch.from_numpy(lcut).cuda(),
                   epsc=torch.from_numpy(epsc).cuda(), nbc=torch.from_numpy(nbc).cuda())
    torch.cuda.synchronize()
    ref = orc.get_td({k: v.cpu().numpy() for k, v in spec.items()}, r, 2.0e3, L, minc, lcut, epsc, nbc=nbc)
    for k in _lib.TD_OUT:
        got = out[k].cpu().numpy()
        rows = [i for i in range(n) if nbc[i] == 0 or k == "dVxBhLM"]
        e = rel_l2(got[rows], ref[k][rows])
        assert 0.0 < e < 1e-6, (k, e)
        assert np.array_equal(got[rows], dev[k].cpu().numpy()[rows]), k
    s.close()
