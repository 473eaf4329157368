"""Autotuner of a handle's runtime knobs (magic_sht_set_tuning).

For one geometry (l_max, minc, n_theta, n_phi, precision form, number of
radial levels, device or host arrays) it times the radial loop's transform
pair -- transform_to_grid_space then transform_to_lm_space on the grids it
produced -- for every candidate setting of

  tc_kernel   persistent tensor-core kernels or one tile per CTA (3xBF16),
  tc_order    tile order of the persistent kernels (table or data reuse),
  fft_rows    theta rows per CTA of the FP32 azimuthal FFTs (8 or 16; the
              double-float FFTs of the fixed-point forms keep their own),
  pipe_chunk  levels per chunk of the host-buffer pipeline (host arrays only),

keeps the fastest, applies it to the handle and caches it in a JSON file keyed
by device name and geometry, so later handles of the same geometry pick it up
without timing.  tc_kernel changes arithmetic (two kernels of the same
3xBF16 form), fft_rows the factorisation of the forward FFT's twiddles
(spectra differ at FP32 rounding); the other knobs change scheduling only.
"""
from __future__ import annotations

import itertools
import json
import os
import statistics
import tempfile
import time
from typing import Callable, Dict, List, Optional

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "magic_gb300", "tuning.json")


def cache_path(path: Optional[str] = None) -> str:
    return path or os.environ.get("MAGIC_SHT_TUNE_CACHE") or DEFAULT_CACHE


def device_name(device: int = 0) -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(device)
    except Exception:
        pass
    return "cpu"


def key(sht, n_levels: int, host: bool, device: str) -> str:
    return "%s|L%d|minc%d|N%d|P%d|%s|R%d|%s" % (device, sht.l_max, sht.minc, sht.n_theta_max, sht.n_phi_max,
                                               sht.precision, n_levels, "host" if host else "device")


def candidates(sht, host: bool) -> List[Dict[str, int]]:
    """Settings to try for this handle's precision form."""
    form = sht.precision
    tc = form in ("bf16x3", "tf32x2", "fp64tc", "bf16x5")  # persistent tensor-core kernels: tile order
    kernels = [0, 1] if form == "bf16x3" else [0]
    orders = [0, 1] if tc else [0]
    rows = [8, 16] if form in ("fp32", "bf16x3", "tf32x2") else [0]  # FP32 FFTs only
    chunks = [8, 16, 32] if host else [sht.tuning()["pipe_chunk"]]
    out = []
    for kern, order, row, chunk in itertools.product(kernels if tc else [0], orders, rows, chunks):
        if kern == 1 and order == 1:  # the one-tile-per-CTA kernels have no tile order
            continue
        out.append({"tc_kernel": kern, "tc_order": order, "fft_rows": row, "pipe_chunk": chunk})
    return out


def _load(path: str) -> Dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, data: Dict) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=os.path.dirname(os.path.abspath(path)), suffix=".tmp")
    with os.fdopen(fd, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _timer(sht, n_levels: int, host: bool, repeats: int) -> Callable[[], float]:
    """A function that times one transform pair (median of `repeats`, ms)."""
    import torch
    from .workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    spec = {k: torch.from_numpy(v) for k, v in grid_space_inputs(sht.l_max, sht.minc, n_levels, seed=99).items()}
    or2 = or2_levels(n_levels)
    dev = {k: v.cuda() for k, v in spec.items()}
    g = sht.transform_to_grid_space(dev, or2=or2)
    fin = {k: g[v] for k, v in FORWARD_FROM_INVERSE.items()}
    if host:
        spec = {k: v.pin_memory() for k, v in spec.items()}
        fin = {k: v.cpu().pin_memory() for k, v in fin.items()}
        g_out = {k: torch.empty(tuple(v.shape), dtype=v.dtype, pin_memory=True) for k, v in g.items()}
        lm = sht.transform_to_lm_space({k: v.cuda() for k, v in fin.items()})
        l_out = {k: torch.empty(tuple(v.shape), dtype=v.dtype, pin_memory=True) for k, v in lm.items()}
    else:
        spec, g_out, l_out = dev, None, None

    def one():
        sht.transform_to_grid_space(spec, or2=or2, out=g_out)
        sht.transform_to_lm_space(fin, out=l_out)

    def run() -> float:
        one()  # warm-up with this setting
        torch.cuda.synchronize()
        ts = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            one()
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
        return statistics.median(ts)
    return run


def autotune(sht, n_levels: int, host: bool = False, cache: Optional[str] = None, repeats: int = 3,
             force: bool = False, timer: Optional[Callable[[], float]] = None) -> Dict:
    """Tune `sht` for batches of `n_levels` levels (device arrays, or host
    arrays with `host`), apply the fastest setting and return
    {"tuning": {...}, "ms": best time or None when taken from the cache,
    "cached": bool, "trials": [(setting, ms), ...]}."""
    path = cache_path(cache)
    k = key(sht, n_levels, host, device_name(getattr(sht, "device", 0) or 0))
    data = _load(path)
    if not force and k in data:
        sht.set_tuning(**data[k]["tuning"])
        return {"tuning": data[k]["tuning"], "ms": None, "cached": True, "trials": []}
    run = timer or _timer(sht, n_levels, host, repeats)
    start = sht.tuning()
    trials = []
    try:
        for c in candidates(sht, host):
            sht.set_tuning(**c)
            trials.append((c, run()))
    except Exception:
        sht.set_tuning(**start)
        raise
    best, ms = min(trials, key=lambda t: t[1])
    sht.set_tuning(**best)
    data = _load(path)  # another process may have written meanwhile
    data[k] = {"tuning": best, "ms": ms, "trials": [[c, t] for c, t in trials]}
    _store(path, data)
    return {"tuning": best, "ms": ms, "cached": False, "trials": trials}
