"""Batched facade jobs (magic_sht_inv_batch / magic_sht_fwd_batch,
SHT.inv_batch / SHT.fwd_batch): every synthesis routine of module sht
(sht_native.f90:40-336) and every analysis routine (:338-379) over many
levels in one call, inputs shared between jobs, per-level lcut and or2,
against the oracle's single-level routines level by level; device arrays in
the FP64 and FP64-accurate tensor-core forms, host arrays through the
pipelined path; and the argument checks."""
import numpy as np
import pytest

from test_gpu_parity import close, make

pytestmark = pytest.mark.gpu
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


def _inv_jobs(S):
    a, b, c, d = S["w"], S["dw"], S["z"], S["dz"]
    return [("scal_to_spat", a), ("scal_to_grad_spat", b), ("pol_to_grad_spat", c), ("torpol_to_spat", a, b, c),
            ("sphtor_to_spat", b, d), ("torpol_to_curl_spat", a, S["ddw"], c, d), ("pol_to_curlr_spat", d),
            ("torpol_to_dphspat", b, c)]


def _inv_ref(o, job, r, lc, or2):
    name, ins = job[0], [x[r] for x in job[1:]]
    if name == "torpol_to_curl_spat":
        out = o.torpol_to_curl_spat(or2[r], *ins, lc)
    else:
        out = getattr(o, name)(*ins, lc)
    return out if isinstance(out, tuple) else (out,)


def _check_inv(o, jobs, got, lcut, or2, tol, host=False):
    n = len(lcut)
    for job, outs in zip(jobs, got):
        refs = [_inv_ref(o, job, r, int(lcut[r]), or2) for r in range(n)]
        for k, out in enumerate(outs):
            a = out if host else out.cpu().numpy()
            close(a, np.array([ref[k] for ref in refs]), tol=tol)


@pytest.mark.parametrize("grid", [(31, 1, 48, 96), (64, 4, 96, 48), (63, 1, 96, 192)])
@pytest.mark.parametrize("prec", ["fp64", "fp64tc"])
def test_inv_and_fwd_batch_match_oracle(built, oracle_mod, torch, grid, prec):
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P = grid
    n = 5
    s = make(*grid, prec=prec)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = grid_space_inputs(L, minc, n, seed=71)
    lcut = np.array([L, 1, max(L - 9, 1), 0, L - 1], dtype=np.int32)
    or2 = or2_levels(n)
    jobs = [tuple([j[0]] + [torch.from_numpy(x).cuda() for x in j[1:]]) for j in _inv_jobs(S)]
    got = s.inv_batch(jobs, or2=torch.from_numpy(or2).cuda(), lcut=lcut)
    torch.cuda.synchronize()
    _check_inv(o, _inv_jobs(S), got, lcut, or2, TOL[prec])
    # analysis of three of the grids just made
    f, g2, h2 = got[3]  # torpol_to_spat: vr, vt, vp
    fj = [("scal_to_SH", f), ("spat_to_qst", f, g2, h2), ("spat_to_sphertor", g2, h2)]
    lf = np.array([L, L - 3, 2, 0, 1], dtype=np.int32)
    res = s.fwd_batch(fj, lcut=lf)
    torch.cuda.synchronize()
    _check_fwd(o, fj, res, lf, TOL[prec])
    s.device_status()


def _check_fwd(o, jobs, got, lcut, tol, host=False):
    """Every output over all levels at once (a level whose true output is
    only rounding noise, e.g. the l = 0 mode of vr, does not dominate)."""
    for job, outs in zip(jobs, got):
        ins = [x if host else x.cpu().numpy() for x in job[1:]]
        refs = []
        for r in range(len(lcut)):
            out = getattr(o, job[0])(*[x[r] for x in ins], int(lcut[r]))
            refs.append(out if isinstance(out, tuple) else (out,))
        for k, out in enumerate(outs):
            close(out if host else out.cpu().numpy(), np.array([ref[k] for ref in refs]), tol=tol)


def test_batch_host_arrays_pipelined(built, oracle_mod, torch):
    """Host arrays over more levels than one pipelined chunk (16)."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 31, 1, 48, 96, 35
    s = make(L, minc, N, P)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = grid_space_inputs(L, minc, n, seed=72)
    lcut = np.random.default_rng(8).integers(0, L + 1, size=n).astype(np.int32)
    or2 = or2_levels(n)
    jobs = _inv_jobs(S)
    got = s.inv_batch(jobs, or2=or2, lcut=lcut)
    _check_inv(o, jobs, got, lcut, or2, TOL["fp64"], host=True)
    f, g2, h2 = got[3]
    fj = [("spat_to_qst", f, g2, h2), ("scal_to_SH", got[0][0])]
    res = s.fwd_batch(fj, lcut=lcut)
    _check_fwd(o, fj, res, lcut, TOL["fp64"], host=True)
    s.device_status()


def test_batch_argument_checks(built, torch):
    from magic_gb300 import _lib
    from magic_gb300.workload import grid_space_inputs
    s = make(31, 1, 48, 96)
    S = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(31, 1, 2, seed=3).items()}
    lib, h = s._lib, s._h

    def call(jobs, inverse=True, or2=None):
        arr = (_lib.Job * len(jobs))()
        for j, (code, ins, outs) in enumerate(jobs):
            arr[j].routine = code
            for k, p in enumerate(ins):
                getattr(arr[j], "in")[k] = p
            for k, p in enumerate(outs):
                arr[j].out[k] = p
        gl = s.n_phi_max * s.nlat_padded
        if inverse:
            return lib.magic_sht_inv_batch(h, 2, or2, None, s.lm_max, gl, arr, len(jobs))
        return lib.magic_sht_fwd_batch(h, 2, None, gl, s.lm_max, arr, len(jobs))

    g = [torch.zeros((2, s.n_phi_max, s.nlat_padded), dtype=torch.float64, device="cuda") for _ in range(3)]
    w, z = S["w"].data_ptr(), S["z"].data_ptr()
    o0, o1, o2 = (x.data_ptr() for x in g)
    assert call([(1, [w], [o0])]) == _lib.OK
    assert call([(99, [w], [o0])]) == _lib.ERR_ARG                     # unknown routine
    assert call([(101, [o0], [w])]) == _lib.ERR_ARG                    # analysis job in a synthesis call
    assert call([(1, [w], [o0])], inverse=False) == _lib.ERR_ARG       # and the other way round
    assert call([(4, [w, z], [o0, o1, o2])]) == _lib.ERR_ARG           # missing input
    assert call([(1, [w, z], [o0])]) == _lib.ERR_ARG                   # unused slot set
    assert call([(1, [w], [o0]), (7, [z], [o0])]) == _lib.ERR_ARG      # repeated output
    assert call([(6, [w, w, z, z], [o0, o1, o2])]) == _lib.ERR_ARG     # curl job without or2
    assert call([(1, [o1], [o1])]) == _lib.ERR_ARG                     # output aliases an input
    torch.cuda.synchronize()
    s.device_status()


def test_batch_small_host_call_and_graph_replay(built, oracle_mod, torch):
    """Host arrays within one chunk (staged without the pipeline), and a
    CUDA-graph capture of device-array batch calls replayed on new inputs."""
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, minc, N, P, n = 31, 1, 48, 96, 3
    s = make(L, minc, N, P)
    o = oracle_mod.OracleSHT(L, minc, N, P)
    S = grid_space_inputs(L, minc, n, seed=73)
    lcut = np.array([L, 5, L - 1], dtype=np.int32)
    or2 = or2_levels(n)
    jobs = _inv_jobs(S)
    got = s.inv_batch(jobs, or2=or2, lcut=lcut)
    _check_inv(o, jobs, got, lcut, or2, TOL["fp64"], host=True)
    # capture: the same jobs on device arrays, replayed after the inputs change
    dS = {k: torch.from_numpy(v).cuda() for k, v in S.items()}
    djobs = [tuple([j[0]] + [dS[k] for k in names]) for j, names in zip(
        jobs, [("w",), ("dw",), ("z",), ("w", "dw", "z"), ("dw", "dz"), ("w", "ddw", "z", "dz"), ("dz",), ("dw", "z")])]
    dor2 = torch.from_numpy(or2).cuda()
    s.reserve(n)
    ref = s.inv_batch(djobs, or2=dor2, lcut=lcut)  # eager outputs, reused as the captured call's outputs
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        n_jobs = len(djobs)
        dlc = torch.from_numpy(lcut).cuda()  # inside a capture every array is a device array
        nlev, arr, outs, keep, plc, por2 = s._batch(djobs, True, dlc, dor2)
        for j in range(n_jobs):  # write into the eager call's output arrays
            for k, t in enumerate(ref[j]):
                arr[j].out[k] = t.data_ptr()
        s.graph_begin()
        try:
            rc = s._lib.magic_sht_inv_batch(s._h, nlev, por2, plc, s.lm_max, s.n_phi_max * s.nlat_padded, arr, n_jobs)
        finally:
            gr = s.graph_end()
        assert rc == 0
        S2 = grid_space_inputs(L, minc, n, seed=74)
        for k, v in dS.items():
            v.copy_(torch.from_numpy(S2[k]))
        s.graph_launch(gr)
        side.synchronize()
    _check_inv(o, _inv_jobs(S2), ref, lcut, or2, TOL["fp64"])
    s.graph_destroy(gr)
    s.device_status()
