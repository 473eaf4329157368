"""Autotuner of the runtime knobs (magic_gb300/autotune.py): the search and
the JSON cache on the CPU with a stand-in handle and timer, and one real
tuning run of a small geometry on the GPU."""
import numpy as np
import pytest

from magic_gb300 import autotune as at


class FakeSHT:
    l_max, minc, n_theta_max, n_phi_max = 63, 1, 96, 192

    def __init__(self, precision):
        self.precision = precision
        self.t = {"tc_kernel": 0, "tc_order": 0, "pipe_chunk": 16, "fft_rows": 0}
        self.calls = []

    def tuning(self):
        return dict(self.t)

    def set_tuning(self, **kw):
        old = dict(self.t)
        self.t.update(kw)
        self.calls.append(dict(self.t))
        return old


def _cost(s):
    t = s.t  # a made-up landscape with one best point
    return 10.0 - 2 * t["tc_kernel"] + 3 * t["tc_order"] + (0 if t["fft_rows"] == 16 else 1) + abs(t["pipe_chunk"] - 16) / 8


@pytest.mark.parametrize("form,host,n", [("bf16x3", False, 6), ("bf16x3", True, 18), ("tf32x2", False, 4),
                                         ("fp32", True, 6), ("fp64", False, 1)])
def test_candidates(form, host, n):
    c = at.candidates(FakeSHT(form), host)
    assert len(c) == n
    assert all(not (x["tc_kernel"] == 1 and x["tc_order"] == 1) for x in c)
    assert len({tuple(sorted(x.items())) for x in c}) == n


def test_search_picks_the_fastest_and_caches_it(tmp_path):
    path = str(tmp_path / "tuning.json")
    s = FakeSHT("bf16x3")
    r = at.autotune(s, 12, host=True, cache=path, timer=lambda: _cost(s))
    assert not r["cached"]
    assert r["tuning"] == {"tc_kernel": 1, "tc_order": 0, "fft_rows": 16, "pipe_chunk": 16}
    assert s.t == r["tuning"] and r["ms"] == min(t for _, t in r["trials"])
    s2 = FakeSHT("bf16x3")
    r2 = at.autotune(s2, 12, host=True, cache=path, timer=lambda: pytest.fail("cached: no timing"))
    assert r2["cached"] and s2.t == r["tuning"]
    s3 = FakeSHT("bf16x3")   # another level count is another key
    r3 = at.autotune(s3, 13, host=True, cache=path, timer=lambda: _cost(s3))
    assert not r3["cached"]


def test_failed_trial_restores_the_start_setting(tmp_path):
    s = FakeSHT("bf16x3")
    s.t["tc_order"] = 1

    def boom():
        raise RuntimeError("timing failed")
    with pytest.raises(RuntimeError):
        at.autotune(s, 4, cache=str(tmp_path / "t.json"), timer=boom)
    assert s.t["tc_order"] == 1


@pytest.mark.gpu
def test_autotune_on_gpu_keeps_results(tmp_path):
    """Tune a small geometry for real; the chosen setting gives the same
    transforms as the default one (3xBF16 vs FP64 within 1e-6)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import __graft_entry__ as g
    g.build()
    from magic_gb300 import SHT
    from magic_gb300.workload import grid_space_inputs, or2_levels
    L, N, P, n = 63, 96, 192, 8
    s = SHT(L, 1, N, P, precision="bf16x3", device=0)
    r = at.autotune(s, n, cache=str(tmp_path / "t.json"), repeats=2)
    assert s.tuning() == dict(r["tuning"], pipe_chunk=s.tuning()["pipe_chunk"])
    s64 = SHT(L, 1, N, P, precision="fp64", device=0)
    spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, 1, n, seed=5).items()}
    a = s.transform_to_grid_space(spec, or2=or2_levels(n))
    b = s64.transform_to_grid_space(spec, or2=or2_levels(n))
    for k in ("vrc", "vtc", "vpc", "sc"):
        x, y = a[k].cpu().numpy(), b[k].cpu().numpy()
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 1e-6, k
    s.device_status()
