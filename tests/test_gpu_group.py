"""Several independent instances of uneven size in one launch per kind
(magic_sht_group_*, SHTGroup; the seven- and five-digit and the 3xBF16
tensor-core forms):
the synthesis and analysis sets of every
instance (rIter.f90:466-712 per instance) with the Legendre sums of all
instances in one pack + one persistent tensor-core launch per direction and
field kind.  Each tile is computed by the same arithmetic as in the
instance's own call, so the group's outputs must equal the instances' own
calls bit for bit; those calls are compared with the oracle for every
instance size in test_gpu_instances.py.  Also: per-level lcut, the
velocity-derivative grids, a CUDA-graph
capture of both group calls replayed, and the argument checks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (l_max, minc, levels): the l_max / minc values of the sixteen-instance case
INSTANCES = [(127, 1, 5), (63, 4, 3), (255, 4, 4), (63, 1, 7), (127, 4, 2), (255, 1, 3)]


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


def _make(torch, precision="fp64tc"):
    from magic_gb300 import SHT
    from magic_gb300.workload import grid_space_inputs, or2_levels
    shts, specs, or2s = [], [], []
    for i, (L, minc, R) in enumerate(INSTANCES):
        N = 3 * (L + 1) // 2
        shts.append(SHT(L, minc, N, 2 * N // minc, precision=precision, device=0))
        specs.append({k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, R, seed=900 + i).items()})
        or2s.append(torch.from_numpy(or2_levels(R)).cuda())
    return shts, specs, or2s


def _assert_equal(torch, got, ref, what):
    assert set(got) == set(ref), what
    for k in ref:
        assert torch.equal(got[k], ref[k]), (what, k, float((got[k] - ref[k]).abs().max()))


@pytest.mark.parametrize("precision", ["fp64tc", "bf16x5", "bf16x3"])
def test_group_equals_separate_calls(built, torch, precision):
    from magic_gb300 import SHTGroup
    from magic_gb300.workload import FORWARD_FROM_INVERSE
    shts, specs, or2s = _make(torch, precision)
    rng = np.random.default_rng(5)
    lcuts = [rng.integers(L // 2, L + 1, size=R).astype(np.int32) for (L, _, R) in INSTANCES]
    ref_g = [s.transform_to_grid_space(sp, or2=o2, lcut=lc) for s, sp, o2, lc in zip(shts, specs, or2s, lcuts)]
    fins = [{k: g[v] for k, v in FORWARD_FROM_INVERSE.items()} for g in ref_g]
    ref_l = [s.transform_to_lm_space(fi, lcut=lc) for s, fi, lc in zip(shts, fins, lcuts)]
    torch.cuda.synchronize()
    G = SHTGroup(shts)
    for rep in range(2):  # the second call reuses the uploaded instance tables
        got_g = G.transform_to_grid_space(specs, or2s=or2s, lcuts=lcuts)
        got_l = G.transform_to_lm_space(fins, lcuts=lcuts)
        torch.cuda.synchronize()
        for i in range(len(shts)):
            _assert_equal(torch, got_g[i], ref_g[i], ("grid", rep, INSTANCES[i]))
            _assert_equal(torch, got_l[i], ref_l[i], ("lm", rep, INSTANCES[i]))
    # with the velocity-derivative grids (and cvrc alone, the u.grad u set)
    skip = {"cvtc": None, "cvpc": None}
    ref_d = [s.transform_to_grid_space(sp, or2=o2, lcut=lc, derivatives=True, out=skip)
             for s, sp, o2, lc in zip(shts, specs, or2s, lcuts)]
    got_d = G.transform_to_grid_space(specs, or2s=or2s, lcuts=lcuts, outs=[dict(skip) for _ in shts],
                                      derivatives=True)
    torch.cuda.synchronize()
    for i in range(len(shts)):
        assert "dvrdrc" in got_d[i] and "cvtc" not in got_d[i]
        _assert_equal(torch, got_d[i], ref_d[i], ("derivatives", INSTANCES[i]))
    for s in shts:
        s.device_status()
    G.close()
    for s in shts:
        s.close()


def test_group_many_calls_reuse_the_ring(built, torch):
    """Uncaptured group calls with new output arrays each time take their
    instance tables from a fixed device ring (wrapping more than once here):
    every call stays equal to the instances' own calls."""
    from magic_gb300 import SHTGroup
    shts, specs, or2s = _make(torch)
    ref_g = [s.transform_to_grid_space(sp, or2=o2) for s, sp, o2 in zip(shts, specs, or2s)]
    torch.cuda.synchronize()
    G = SHTGroup(shts)
    for rep in range(160):
        got_g = G.transform_to_grid_space(specs, or2s=or2s)  # fresh outputs every call
        if rep % 40 == 39:
            torch.cuda.synchronize()
            for i in range(len(shts)):
                _assert_equal(torch, got_g[i], ref_g[i], ("ring", rep, INSTANCES[i]))
    G.close()
    for s in shts:
        s.close()


def test_group_graph_replay(built, torch):
    from magic_gb300 import SHTGroup
    from magic_gb300.workload import FORWARD_FROM_INVERSE
    shts, specs, or2s = _make(torch)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        ref_g = [s.transform_to_grid_space(sp, or2=o2) for s, sp, o2 in zip(shts, specs, or2s)]
        fins = [{k: g[v] for k, v in FORWARD_FROM_INVERSE.items()} for g in ref_g]
        ref_l = [s.transform_to_lm_space(fi) for s, fi in zip(shts, fins)]
        out_g = [{k: torch.zeros_like(v) for k, v in g.items()} for g in ref_g]
        out_l = [{k: torch.zeros_like(v) for k, v in l.items()} for l in ref_l]
        G = SHTGroup(shts)
        G.transform_to_grid_space(specs, or2s=or2s, outs=out_g)
        G.transform_to_lm_space(fins, outs=out_l)
        side.synchronize()
        for d in out_g + out_l:
            for v in d.values():
                v.zero_()
        shts[0].graph_begin()
        try:
            G.transform_to_grid_space(specs, or2s=or2s, outs=out_g)
            G.transform_to_lm_space(fins, outs=out_l)
        finally:
            gr = shts[0].graph_end()
        # the same calls outside the graph before its first replay (the
        # captured instance tables exist only when the graph runs)
        G.transform_to_grid_space(specs, or2s=or2s, outs=out_g)
        G.transform_to_lm_space(fins, outs=out_l)
        side.synchronize()
        for i in range(len(shts)):
            _assert_equal(torch, out_g[i], ref_g[i], ("eager after capture", INSTANCES[i]))
            _assert_equal(torch, out_l[i], ref_l[i], ("eager after capture", INSTANCES[i]))
        for d in out_g + out_l:
            for v in d.values():
                v.zero_()
        shts[0].graph_launch(gr)
        side.synchronize()
    for i in range(len(shts)):
        _assert_equal(torch, out_g[i], ref_g[i], ("graph grid", INSTANCES[i]))
        _assert_equal(torch, out_l[i], ref_l[i], ("graph lm", INSTANCES[i]))
    shts[0].graph_destroy(gr)
    G.close()
    for s in shts:
        s.close()


def test_group_argument_checks(built, torch):
    from magic_gb300 import SHT, SHTGroup
    from magic_gb300 import _lib
    from magic_gb300.workload import grid_space_inputs
    a = SHT(63, 1, 96, 192, precision="fp64tc", device=0)
    b = SHT(63, 1, 96, 192, precision="fp64", device=0)
    with pytest.raises(_lib.ShtError) as e:
        SHTGroup([a, b])
    assert e.value.code == _lib.ERR_UNSUPPORTED
    with pytest.raises(_lib.ShtError) as e:
        SHTGroup([a, a])
    assert e.value.code == _lib.ERR_ARG
    c = SHT(63, 1, 96, 192, precision="bf16x3", device=0)
    with pytest.raises(_lib.ShtError) as e:  # one arithmetic form per group
        SHTGroup([a, c])
    assert e.value.code == _lib.ERR_ARG
    c.close()
    G = SHTGroup([a])
    host = grid_space_inputs(63, 1, 2, seed=3)  # numpy arrays: host memory
    with pytest.raises(_lib.ShtError) as e:
        G.transform_to_grid_space([host])
    assert e.value.code == _lib.ERR_ARG
    G.close()
    a.close()
    b.close()
