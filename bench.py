#!/usr/bin/env python
"""Benchmark of the radial loop's spherical-harmonic transform set on GB300.

Workload (the precision-form configuration): l_max=255, n_theta=384 Gauss
points, n_phi=768, minc=1, 129 radial levels; per level 13 spectral fields ->
15 grids (transform_to_grid_space, src/rIter.f90:466-622) and 10 grids -> 10
spectral fields (transform_to_lm_space, src/rIter.f90:624-712).  Synthetic
seeded spectra with std (l+1)^-2 and a radial envelope; the forward inputs
are the grids produced by the inverse transforms.

One step = both transform sets over all 129 levels.  The headline `value` is
radial levels/s of the FP64-accurate tensor-core form (fp64tc: every output
within 1e-6 relative L2 of the FP64 form, reported per output); the FP64 form
is timed in the same run, and the 3xBF16 / 2xTF32 forms, the other
configurations (l_max 63 and 511, the sixteen-instance case), one explicit
stage of the radial loop and the CPU oracle are reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SHT radial levels/s at lmax=255: mixed-prec vs FP64 GPU at <=1e-6 rel L2"
L_MAX, N_THETA, N_PHI, MINC, N_LEVELS = 255, 384, 768, 1, 129
WORKLOAD = ("precision form: l_max=255, n_theta=384, n_phi=768, minc=1, 129 radial levels, "
            "15 inverse + 10 forward grids per level")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="auto", choices=["auto", "fp32", "bf16x3", "tf32x2", "fp64tc", "bf16x5", "fp64"])
    ap.add_argument("--cpu-levels", type=int, default=2)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-stage", action="store_true", help="skip the radial-loop stage measurement")
    ap.add_argument("--no-variant", action="store_true", help="skip the other precision forms (3xBF16, 2xTF32)")
    ap.add_argument("--levels", type=int, default=N_LEVELS,
                    help="radial levels (profiling cases; with --instances: the cap of every instance)")
    ap.add_argument("--instances", action="store_true",
                    help="instead of the bench line: sixteen mixed-size instances in one graph (one JSON line)")
    ap.add_argument("--group", action="store_true",
                    help="with --instances: the sixteen instances as one group (magic_sht_group_*)")
    ap.add_argument("--only-reduced", action="store_true", help="skip the FP64 form (profiling)")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations (C0, C1, C3, C4)")
    ap.add_argument("--stage-only", action="store_true",
                    help="profiling case: two radial-loop stages of --form over --levels levels, then exit")
    ap.add_argument("--clock-seconds", type=float, default=1.5,
                    help="back-to-back steps sampled for clocks before the timed steps")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


# ---------------------------------------------------------------- clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ algorithmic
def algorithmic_per_level(L, N, P, minc, t2):
    """Bytes and flops per radial level of each launch phase (FP64 outputs,
    half spectra of t2 bytes per complex).  Tables are counted per launch."""
    n_m = L // minc + 1
    K = sum(L - m + 1 for m in range(0, L + 1, minc))
    hs = n_m * N * t2
    grid = N * P * 8
    spec = K * 16
    return {
        "inv_leg_scalar": dict(bytes=7 * spec + 7 * hs, flops=7 * 2 * K * N),
        "inv_leg_vector": dict(bytes=11 * spec + 8 * hs, flops=4 * 8 * K * N),
        "fft_inv": dict(bytes=15 * hs + 15 * grid, flops=15 * N * 2.5 * P * __import__("math").log2(P)),
        "fft_fwd": dict(bytes=10 * grid + 10 * hs, flops=10 * N * 2.5 * P * __import__("math").log2(P)),
        "fwd_leg_scalar": dict(bytes=4 * hs + 4 * spec, flops=4 * 2 * K * N),
        "fwd_leg_vector": dict(bytes=6 * hs + 6 * spec, flops=3 * 8 * K * N),
    }, K


def stage_measure(sm, s64, spec, n_levels, steps, hbm):
    """One explicit stage of the radial loop (RadialLoop.step: the synthesis
    set, rigid-boundary overrides, get_nl on the interior levels, the
    analysis set, the Courant steps and get_td with the boundary flags) over
    every level, eager, as a caller runs it: the Courant steps return to the
    host once per stage.  Wall time and CUDA events per stage, and the
    radial-loop kernels (get_nl, courant, get_td, boundary kernels) against
    the HBM roofline with their algorithmic bytes."""
    import numpy as np
    import torch
    from magic_gb300.radial_loop import RadialLoop
    from magic_gb300.workload import radii
    loop = RadialLoop(sm, radii(n_levels), cor_fac=1e3, ktopv=2, kbotv=2)
    # accuracy of the stage against the same stage on the FP64 handle
    ref = RadialLoop(s64, radii(n_levels), cor_fac=1e3, ktopv=2, kbotv=2).step(spec)
    got = loop.step(spec)
    acc = {}
    for k in ("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM"):
        acc[k] = float(torch.linalg.vector_norm(got[k] - ref[k]) / torch.linalg.vector_norm(ref[k]))
    acc["dtrkc"] = float(np.max(np.abs(got["dtrkc"] / ref["dtrkc"] - 1.0)))
    acc["dthkc"] = float(np.max(np.abs(got["dthkc"] / ref["dthkc"] - 1.0)))
    del ref, got
    for _ in range(2):
        loop.step(spec)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    t0 = time.perf_counter()
    ev[0].record(st)
    for k in range(steps):
        loop.step(spec)
        ev[k + 1].record(st)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / steps * 1e3
    per = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
    sm.set_profiling(True)
    sm.phase_times(reset=True)
    loop.step(spec)
    ph = sm.phase_times(reset=True)
    sm.set_profiling(False)
    torch.cuda.synchronize()
    # the same stage captured once as a CUDA graph and replayed (one launch and
    # the Courant steps' synchronisation per stage)
    sg = loop.capture(spec)
    sg.replay()
    t0 = time.perf_counter()
    for _ in range(steps):
        sg.replay()
    graph_ms = (time.perf_counter() - t0) / steps * 1e3
    sg.close()
    torch.cuda.synchronize()
    sm.device_status()
    N, P, K = sm.nlat_padded, sm.n_phi_max, sm.lm_max
    grid = 8 * N * P
    interior = n_levels - 2  # rigid boundaries: get_nl on the interior levels only
    alg = {"nl": (13 + 10) * grid * interior,          # 13 synthesis grids in, 10 analysis grids out
           "courant": 6 * grid * n_levels,             # v and B grids in, two numbers per level out
           "td": (10 + 7) * 16 * K * n_levels}         # 10 spectra in, 7 out
    kern = {}
    for k, (ms, n) in ph.items():
        if not n:
            continue
        kern[k] = {"ms": ms, "launches": n}
        if k in alg and ms > 0:
            gbs = alg[k] / (ms * 1e-3) / 1e9
            kern[k].update({"algorithmic_gb": alg[k] / 1e9, "achieved_gbs": gbs, "hbm_frac": gbs / hbm})
    return {"what": "RadialLoop.step: transform_to_grid_space, rigid boundaries, get_nl (interior), "
                    "transform_to_lm_space, courant (host dt arrays), get_td with nBc",
            "levels": n_levels, "steps": steps, "ms_per_stage_wall": wall,
            "ms_per_stage_events": statistics.median(per), "levels_per_s": n_levels / (wall * 1e-3),
            "graph": {"ms_per_stage": graph_ms, "levels_per_s": n_levels / (graph_ms * 1e-3),
                      "what": "RadialLoop.capture: the stage as one CUDA graph, replayed; wall time per "
                              "replay including the Courant steps' copy to the host"},
            "kernels": kern,
            "rel_l2_vs_fp64_stage": acc}


def table_bytes(L, N, minc, elem):
    K = sum(L - m + 1 for m in range(0, L + 1, minc))
    return 2 * K * (N // 2) * elem


# ------------------------------------------------------------------ arms
def reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle
    from magic_gb300.workload import grid_space_inputs, or2_levels
    oracle.build_oracle()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    n = max(1, args.cpu_levels)
    o = oracle.OracleSHT(L_MAX, MINC, N_THETA, N_PHI)
    spec = grid_space_inputs(L_MAX, MINC, N_LEVELS, seed=1234)
    or2 = or2_levels(N_LEVELS)

    def one_level(r):
        """Both transform sets of level r; returns the seconds spent in them
        (the nonlinear products between the sets are not timed, as on the GPU)."""
        t0 = time.perf_counter()
        g = {}
        g["sc"] = o.scal_to_spat(spec["s"][r])
        g["pc"] = o.scal_to_spat(spec["p"][r])
        g["xic"] = o.scal_to_spat(spec["xi"][r])
        g["vrc"], g["vtc"], g["vpc"] = o.torpol_to_spat(spec["w"][r], spec["dw"][r], spec["z"][r])
        g["cvrc"], g["cvtc"], g["cvpc"] = o.torpol_to_curl_spat(or2[r], spec["w"][r], spec["ddw"][r],
                                                                spec["z"][r], spec["dz"][r])
        g["brc"], g["btc"], g["bpc"] = o.torpol_to_spat(spec["b"][r], spec["db"][r], spec["aj"][r])
        g["cbrc"], g["cbtc"], g["cbpc"] = o.torpol_to_curl_spat(or2[r], spec["b"][r], spec["ddb"][r],
                                                                spec["aj"][r], spec["dj"][r])
        t1 = time.perf_counter()
        f = {k: v[0] for k, v in oracle.get_nl({k: v[None] for k, v in g.items()}, or2[r:r + 1], N_THETA).items()}
        t2 = time.perf_counter()
        for pre in ("Adv", "VS", "VxB"):
            o.spat_to_qst(f[pre + "r"], f[pre + "t"], f[pre + "p"])
        o.scal_to_SH(f["heatTerms"])
        return (t1 - t0) + (time.perf_counter() - t2)

    for w in range(args.warmup):
        one_level(w % N_LEVELS)
    times = []
    for k in range(args.steps):
        times.append(sum(one_level((k * n + i) % N_LEVELS) for i in range(n)))
    total = sum(times)
    v = n * args.steps / total
    line = {
        "metric": METRIC, "impl": "reference", "value": v, "unit": "levels/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "l_max": L_MAX, "n_theta": N_THETA, "n_phi": N_PHI,
                   "minc": MINC, "n_levels": N_LEVELS, "parallelism": "openmp over theta"},
        "cpu_baseline": {"value": v, "unit": "levels/s", "cores": threads, "kind": "port",
                         "sample": "%d of %d levels per step, full 15+10 transform set" % (n, N_LEVELS)},
        "e2e": {"value": v, "unit": "levels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Fortran and no Fortran compiler exists here; the timed CPU code "
                "is the C++ restatement of its native transforms (oracle/sht_oracle.cpp)",
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(levels: int, threads: int = 0):
    """The oracle's rate on `levels` levels of the set, with `threads` host
    threads (0: every core)."""
    from oracle import oracle
    from magic_gb300.workload import spectra
    oracle.build_oracle()
    threads = threads or os.cpu_count() or 1
    oracle.set_threads(threads)
    o = oracle.OracleSHT(L_MAX, MINC, N_THETA, N_PHI)
    S = spectra(L_MAX, MINC, 13, seed=99)
    t0 = time.perf_counter()
    for _ in range(levels):
        for i in range(3):
            o.scal_to_spat(S[i])
        g = o.torpol_to_spat(S[3], S[4], S[5])
        o.torpol_to_curl_spat(0.7, S[3], S[6], S[5], S[7])
        o.torpol_to_spat(S[8], S[9], S[10])
        o.torpol_to_curl_spat(0.7, S[8], S[11], S[10], S[12])
        for _ in range(3):
            o.spat_to_qst(g[0], g[1], g[2])
        o.scal_to_SH(g[0])
    dt = time.perf_counter() - t0
    return {"value": levels / dt, "unit": "levels/s", "cores": threads, "kind": "port",
            "sample": "%d levels of the full 15+10 transform set at l_max=255 (oracle, OpenMP)" % levels}


def tc_available(local) -> bool:
    from magic_gb300 import SHT
    try:
        SHT(15, 1, 24, 48, precision="fp64tc", device=local).close()
        return True
    except Exception:
        return False


def field_errors(a_g, a_l, b_g, b_l):
    """Relative L2 of every output field of a against b, the normwise error
    of every call (a vector field's three grids, the q, s, t of one
    spat_to_qst) and the fields above 1e-6."""
    import torch
    errs = {}
    for a, b in ((a_g, b_g), (a_l, b_l)):
        for k in b:
            errs[k] = float(torch.linalg.vector_norm(a[k] - b[k]) / torch.linalg.vector_norm(b[k]))
    groups = {"v": ("vrc", "vtc", "vpc"), "curl v": ("cvrc", "cvtc", "cvpc"), "b": ("brc", "btc", "bpc"),
              "curl b": ("cbrc", "cbtc", "cbpc"), "Adv": ("AdvrLM", "AdvtLM", "AdvpLM"),
              "VS": ("VSrLM", "VStLM", "VSpLM"), "VxB": ("VxBrLM", "VxBtLM", "VxBpLM")}
    allm = dict({k: (a_g[k], b_g[k]) for k in b_g}, **{k: (a_l[k], b_l[k]) for k in b_l})
    normwise = {}
    for name, ks in groups.items():
        if not all(k in allm for k in ks):
            continue
        num = sum(float(torch.linalg.vector_norm(allm[k][0] - allm[k][1])) ** 2 for k in ks)
        den = sum(float(torch.linalg.vector_norm(allm[k][1])) ** 2 for k in ks)
        normwise[name] = (num / den) ** 0.5
    for k in ("sc", "pc", "xic", "heatTermsLM"):
        if k in errs:
            normwise[k] = errs[k]
    over = sorted(k for k, v in errs.items() if not v <= 1e-6)
    return {"max": max(errs.values()), "per_field": errs, "max_normwise_per_call": max(normwise.values()),
            "normwise_per_call": normwise, "over_1e-6": over, "every_output_within_1e-6": not over}


def checkpoint_accuracy(form, local):
    """The report of field_errors on the reference's own sample spectra
    (samples/boussBenchSat/checkpoint_end.start: l_max = 64, minc = 4, five
    radial levels of w, z, s, b, j, committed as tests/golden/
    checkpoint_spectra.npz): the radial-loop synthesis set with every spectral
    slot filled from the checkpoint field of its kind (radial derivatives are
    not in the checkpoint), the nonlinear products of the FP64 grids, then
    the analysis set; `form` against the FP64 form."""
    import numpy as np
    import torch
    from magic_gb300 import SHT
    d = np.load(os.path.join(ROOT, "tests", "golden", "checkpoint_spectra.npz"))
    L, minc, N = int(d["l_max"]), int(d["minc"]), int(d["n_theta_max"])
    P = int(d["n_phi_tot"]) // minc
    w, z, s, b, j = (d[k] for k in ("wpol", "ztor", "entropy", "bpol", "btor"))
    spec = {"s": s, "p": s, "xi": s, "w": w, "dw": w, "ddw": w, "z": z, "dz": z,
            "b": b, "db": b, "ddb": b, "aj": j, "dj": j}
    spec = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in spec.items()}
    or2 = 1.0 / np.asarray(d["radius"], dtype=np.float64) ** 2
    s64 = SHT(L, minc, N, P, precision="fp64", device=local)
    sm = SHT(L, minc, N, P, precision=form, device=local)
    g64 = s64.transform_to_grid_space(spec, or2=or2)
    nl = s64.get_nl(g64, or2=or2)
    l64 = s64.transform_to_lm_space(nl)
    gm = sm.transform_to_grid_space(spec, or2=or2)
    lm = sm.transform_to_lm_space(nl)
    torch.cuda.synchronize()
    sm.device_status()
    out = field_errors(gm, lm, g64, l64)
    out["what"] = ("reference sample spectra (boussBenchSat checkpoint, l_max=%d, minc=%d, %d levels); "
                   "analysis inputs = get_nl of the FP64 grids" % (L, minc, w.shape[0]))
    s64.close()
    sm.close()
    return out


def batched_set_ms(s, spec, fin, or2, batch, steps, warmup):
    """Both transform sets over every level in batches of `batch` levels (the
    large configuration does not keep all levels' grids resident); `fin`
    holds the analysis inputs of one batch, reused by every batch.  Returns
    the ms of one pass (CUDA events, mean of `steps`)."""
    import torch
    n = next(iter(spec.values())).shape[0]
    st = torch.cuda.current_stream()
    out_g, out_l = {}, {}

    def one():
        for r0 in range(0, n, batch):
            r1 = min(n, r0 + batch)
            full = r1 - r0 == batch
            g = s.transform_to_grid_space({k: v[r0:r1] for k, v in spec.items()}, or2=or2[r0:r1],
                                          out=out_g if (full and out_g) else None)
            lm = s.transform_to_lm_space({k: v[:r1 - r0] for k, v in fin.items()},
                                         out=out_l if (full and out_l) else None)
            if full and not out_g:
                out_g.update(g)
                out_l.update(lm)
    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        one()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def config_measure(name, L, minc, N, P, R, forms, local, hbm, full_set=True, batch=None, steps=3,
                   cpu_levels=0, what=""):
    """One configuration: every form's levels/s over R levels of the radial
    set (or of the scalar + QST round trip when full_set is False), its
    per-output error against the FP64 form, the dominant kernel's HBM
    fraction, and the oracle's CPU rate on a bounded sample."""
    import torch
    from magic_gb300 import SHT
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    fields = None if full_set else ("s", "w", "dw", "z")
    spec_np = grid_space_inputs(L, minc, R, seed=4321 + L)
    if fields:
        spec_np = {k: v for k, v in spec_np.items() if k in fields}
    spec = {k: torch.from_numpy(v).cuda() for k, v in spec_np.items()}
    or2 = torch.from_numpy(or2_levels(R)).cuda()
    fwd_map = FORWARD_FROM_INVERSE if full_set else {"Advr": "vrc", "Advt": "vtc", "Advp": "vpc",
                                                      "heatTerms": "sc"}
    batch = batch or R
    res = {"workload": what, "l_max": L, "minc": minc, "n_theta": N, "n_phi": P, "levels": R, "forms": {}}
    ref = None
    t2_of = {"fp64": 16, "fp64tc": 16, "bf16x5": 16}
    for form in forms:
        s = SHT(L, minc, N, P, precision=form, device=local)
        s.reserve(batch)
        g = s.transform_to_grid_space({k: v[:batch] for k, v in spec.items()}, or2=or2[:batch])
        fin_b = {k: g[v] for k, v in fwd_map.items()}
        lm = s.transform_to_lm_space(fin_b)
        if form == "fp64":
            ref = (g, fin_b, lm)
        # analysis inputs of every form and batch: the FP64 form's synthesis grids of the first batch
        fin = ref[1] if ref else fin_b
        ms = batched_set_ms(s, spec, fin, or2, batch, 1 if form == "fp64" else steps, 1)
        entry = {"value": R / (ms * 1e-3), "unit": "levels/s", "ms_per_step": ms}
        if ref is not None and form != "fp64":
            gm = s.transform_to_grid_space({k: v[:batch] for k, v in spec.items()}, or2=or2[:batch])
            lmm = s.transform_to_lm_space(ref[1])
            torch.cuda.synchronize()
            acc = field_errors(gm, lmm, ref[0], ref[2])
            entry["rel_l2_vs_fp64_max"] = acc["max"]
            entry["max_normwise_per_call"] = acc["max_normwise_per_call"]
            entry["over_1e-6"] = acc["over_1e-6"]
            del gm, lmm
        s.set_profiling(True)
        s.phase_times(reset=True)
        s.transform_to_grid_space({k: v[:batch] for k, v in spec.items()}, or2=or2[:batch])
        s.transform_to_lm_space(fin)
        ph = s.phase_times(reset=True)
        s.set_profiling(False)
        s.device_status()
        alg, _ = algorithmic_per_level(L, N, P, minc, t2_of.get(form, 8))
        dom = max(ph, key=lambda k: ph[k][0])
        if dom in alg and ph[dom][0] > 0:
            gbs = alg[dom]["bytes"] * batch / (ph[dom][0] * 1e-3) / 1e9
            entry["dominant_kernel"] = {"phase": dom, "ms_per_batch": ph[dom][0], "achieved_gbs": gbs,
                                        "hbm_frac": gbs / hbm}
        entry["phases_ms_per_batch"] = {k: v[0] for k, v in ph.items() if v[1]}
        res["forms"][form] = entry
        s.close()
        del g, lm, fin_b, fin
        torch.cuda.synchronize()
    if "fp64" in res["forms"]:
        for f, e in res["forms"].items():
            e["speedup_vs_fp64_gpu"] = e["value"] / res["forms"]["fp64"]["value"]
    del ref
    torch.cuda.synchronize()
    if cpu_levels > 0:
        from oracle import oracle
        oracle.build_oracle()
        threads = os.cpu_count() or 1
        oracle.set_threads(threads)
        o = oracle.OracleSHT(L, minc, N, P)
        t0 = time.perf_counter()
        for r in range(cpu_levels):
            if full_set:
                sc = o.scal_to_spat(spec_np["s"][r])
                o.scal_to_spat(spec_np["p"][r])
                o.scal_to_spat(spec_np["xi"][r])
                v = o.torpol_to_spat(spec_np["w"][r], spec_np["dw"][r], spec_np["z"][r])
                o.torpol_to_curl_spat(0.7, spec_np["w"][r], spec_np["ddw"][r], spec_np["z"][r], spec_np["dz"][r])
                o.torpol_to_spat(spec_np["b"][r], spec_np["db"][r], spec_np["aj"][r])
                o.torpol_to_curl_spat(0.7, spec_np["b"][r], spec_np["ddb"][r], spec_np["aj"][r], spec_np["dj"][r])
                for _ in range(3):
                    o.spat_to_qst(*v)
                o.scal_to_SH(sc)
            else:
                f = o.scal_to_spat(spec_np["s"][r])
                v = o.torpol_to_spat(spec_np["w"][r], spec_np["dw"][r], spec_np["z"][r])
                o.spat_to_qst(*v)
                o.scal_to_SH(f)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": cpu_levels / dt, "unit": "levels/s", "cores": threads, "kind": "port",
                               "sample": "%d of %d levels (oracle, OpenMP)" % (cpu_levels, R)}
    return res


def our_arm(args):
    global N_LEVELS
    N_LEVELS = args.levels
    import numpy as np
    import torch
    import torch.distributed as dist
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from magic_gb300 import build as b
    b.build()
    from magic_gb300 import SHT, measure_gflops, _lib
    from magic_gb300.workload import grid_space_inputs, or2_levels

    dev = torch.device("cuda", local)
    hbm, bf16, peak_kind = peaks()
    form = args.form
    if form == "auto":
        form = "fp64tc" if tc_available(local) else "fp32"

    spec_np = grid_space_inputs(L_MAX, MINC, N_LEVELS, seed=1234 + 7919 * rank)
    spec = {k: torch.from_numpy(v).to(dev) for k, v in spec_np.items()}
    if args.stage_only:
        from magic_gb300.radial_loop import RadialLoop
        from magic_gb300.workload import radii
        sp = SHT(L_MAX, MINC, N_THETA, N_PHI, precision=form, device=local)
        loop = RadialLoop(sp, radii(N_LEVELS), cor_fac=1e3, ktopv=2, kbotv=2)
        for _ in range(2):
            loop.step(spec)
        torch.cuda.synchronize()
        sp.device_status()
        print(json.dumps({"form": form, "levels": N_LEVELS, "stage_only": True}), flush=True)
        return
    or2_np = or2_levels(N_LEVELS)
    or2 = torch.from_numpy(or2_np).to(dev)
    fin = {}  # analysis inputs: nonlinear products of the FP64 synthesis grids (set below)

    def run_set(s, out_g, out_s):
        g = s.transform_to_grid_space(spec, or2=or2, out=out_g)
        return g, s.transform_to_lm_space(fin, out=out_s)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    def time_steps(s, out_g, out_s, steps, fn=None):
        """One step (both transform sets over all levels) captured in a CUDA
        graph and replayed `steps` times; CUDA events on the replay stream
        around every replay.  Returns (total ms, kernel launches, per-step ms)."""
        fn = fn or run_set
        s.reserve(N_LEVELS)
        side = torch.cuda.Stream()
        barrier()
        with torch.cuda.stream(side):
            n0 = s.launch_count()
            s.graph_begin()
            fn(s, out_g, out_s)
            gr = s.graph_end()
            per_step_launches = s.launch_count() - n0
            s.graph_launch(gr)  # warm replay
            side.synchronize()
            barrier()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
            ev[0].record(side)
            for k in range(steps):
                s.graph_launch(gr)
                ev[k + 1].record(side)
            side.synchronize()
        barrier()
        per = [ev[k].elapsed_time(ev[k + 1]) for k in range(steps)]
        ms = ev[0].elapsed_time(ev[steps])
        s.graph_destroy(gr)
        if world > 1:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, per_step_launches * steps, per

    # ---- FP64 form; its synthesis grids give the analysis inputs of every form
    # (the grid-space nonlinear products of get_nl, outside the timed steps)
    s64 = SHT(L_MAX, MINC, N_THETA, N_PHI, precision="fp64", device=local)
    fin.update(s64.get_nl(s64.transform_to_grid_space(spec, or2=or2), or2=or2_np))
    torch.cuda.synchronize()
    k64 = max(1, min(args.steps, 3))
    if not args.only_reduced:
        g64, l64 = run_set(s64, None, None)
        for _ in range(max(0, args.warmup - 1)):
            run_set(s64, g64, l64)
        ms64, _, _ = time_steps(s64, g64, l64, k64)
        lev64 = world * N_LEVELS * k64 / (ms64 * 1e-3)

    # ---- headline form
    sm = SHT(L_MAX, MINC, N_THETA, N_PHI, precision=form, device=local)
    gm, lmx = run_set(sm, None, None)
    for _ in range(max(0, args.warmup - 1)):
        run_set(sm, gm, lmx)
    # clocks: sampled while the same steps run back to back, then the timed K steps
    clk = ClockSampler(local)
    clk.start()
    t_end = time.time() + args.clock_seconds
    while time.time() < t_end:
        run_set(sm, gm, lmx)
        torch.cuda.synchronize()
    ms, launches, per_step = time_steps(sm, gm, lmx, args.steps)
    clocks = clk.stop()
    value = world * N_LEVELS * args.steps / (ms * 1e-3)

    if args.only_reduced:
        sm.set_profiling(True)
        sm.phase_times(reset=True)
        run_set(sm, gm, lmx)
        ph = sm.phase_times(reset=True)
        sm.set_profiling(False)
        sm.device_status()
        print(json.dumps({"form": form, "value": value, "ms_per_step": ms / args.steps, "levels": N_LEVELS,
                          "phases_ms": {k: v[0] for k, v in ph.items() if v[1]}}), flush=True)
        return
    # ---- accuracy of the headline form against the FP64 form (same inputs): every output
    run_set(sm, gm, lmx)
    run_set(s64, g64, l64)
    torch.cuda.synchronize()
    sm.device_status()
    acc = field_errors(gm, lmx, g64, l64)
    acc["max_abs_over_max"] = max(float((gm[k] - g64[k]).abs().max() / g64[k].abs().max()) for k in g64)
    # the whole chain in the headline form: its synthesis grids -> get_nl on its
    # handle -> its analysis, against the same chain on the FP64 handle
    gA = sm.transform_to_grid_space(spec, or2=or2)
    lA = sm.transform_to_lm_space(sm.get_nl(gA, or2=or2_np))
    torch.cuda.synchronize()
    chain = field_errors(gA, lA, g64, l64)
    chain["what"] = ("synthesis -> get_nl -> analysis, all on the %s handle, against the same chain "
                     "on the FP64 handle" % form)
    del gA, lA
    checkpoint = checkpoint_accuracy(form, local)

    # ---- the other precision forms: same step, timing and accuracy, beside the headline
    others = {}
    if not args.no_variant:
        for f in ("fp64tc", "bf16x5", "bf16x3", "tf32x2"):
            if f == form:
                continue
            sv = SHT(L_MAX, MINC, N_THETA, N_PHI, precision=f, device=local)
            gv, lv = run_set(sv, None, None)
            for _ in range(max(0, args.warmup - 1)):
                run_set(sv, gv, lv)
            msv, _, perv = time_steps(sv, gv, lv, args.steps)
            run_set(sv, gv, lv)
            torch.cuda.synchronize()
            sv.device_status()
            av = field_errors(gv, lv, g64, l64)
            vv = world * N_LEVELS * args.steps / (msv * 1e-3)
            others[f] = {"value": vv, "unit": "levels/s", "ms_per_step": msv / args.steps,
                         "median_ms_per_step": statistics.median(perv), "speedup_vs_fp64_gpu": vv / lev64,
                         "rel_l2_vs_fp64_max": av["max"], "over_1e-6": av["over_1e-6"],
                         "max_normwise_per_call": av["max_normwise_per_call"],
                         "rel_l2_vs_fp64": av}
            sv.close()
            del gv, lv
            torch.cuda.synchronize()

    # ---- the reference's Boussinesq default analysis set (rIter.f90:682-702): the
    # composition flux V Xi (spat_to_qst, 3 grids) in place of heatTerms, 12 forward grids
    bouss = None
    if not args.no_variant:
        finx = {k: v for k, v in fin.items() if k != "heatTerms"}
        finx.update({"VXir": fin["VSr"], "VXit": fin["VSt"], "VXip": fin["VSp"]})

        def run_bouss(s, out_g, out_s):
            g = s.transform_to_grid_space(spec, or2=or2, out=out_g)
            return g, s.transform_to_lm_space(finx, out=out_s)
        gb, lb = run_bouss(sm, gm, None)
        for _ in range(max(0, args.warmup - 1)):
            run_bouss(sm, gm, lb)
        msb, _, perb = time_steps(sm, gm, lb, args.steps, fn=run_bouss)
        sm.device_status()
        bouss = {"what": "15 synthesis grids + 12 analysis grids per level (V Xi in place of heatTerms), "
                         "headline form", "value": world * N_LEVELS * args.steps / (msb * 1e-3),
                 "unit": "levels/s", "ms_per_step": msb / args.steps, "median_ms_per_step": statistics.median(perb)}
        del lb, finx
        torch.cuda.synchronize()

    # ---- per-phase kernel timing (CUDA events on the launching stream)
    sm.set_profiling(True)
    sm.phase_times(reset=True)
    for _ in range(2):
        run_set(sm, gm, lmx)
    ph = sm.phase_times(reset=True)
    sm.set_profiling(False)
    s64.set_profiling(True)
    s64.phase_times(reset=True)
    run_set(s64, g64, l64)
    ph64 = s64.phase_times(reset=True)
    s64.set_profiling(False)

    t2 = 16 if form in ("fp64", "fp64tc", "bf16x5") else 8
    alg, K = algorithmic_per_level(L_MAX, N_THETA, N_PHI, MINC, t2)
    # table bytes per Legendre launch: the split images (7 bf16 digits for
    # fp64tc, 5 for bf16x5, 3 bf16 for bf16x3, 2 tf32 for tf32x2) of P and dP
    tab_elem = {"fp64tc": 14, "bf16x5": 10, "bf16x3": 6, "tf32x2": 8, "fp32": 4, "fp64": 8}[form]
    dom = max(ph, key=lambda k: ph[k][0])
    dom_ms, dom_n = ph[dom]
    per_launch_ms = dom_ms / max(dom_n, 1)
    levels_per_launch = N_LEVELS  # every launch covers all levels of its field group
    nbytes = alg[dom]["bytes"] * levels_per_launch
    if "leg" in dom:
        nbytes += table_bytes(L_MAX, N_THETA, MINC, tab_elem)
    achieved_gbs = nbytes / (per_launch_ms * 1e-3) / 1e9
    fp32_peak = measure_gflops("fp32", local)
    fp64_peak = measure_gflops("fp64", local)
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_per_level.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            if form in tj and dom in tj[form]:
                traffic = tj[form][dom] * levels_per_launch
        except Exception:
            traffic = None
    if "leg" in dom and form in ("fp32", "fp64"):
        achieved_gf = alg[dom]["flops"] * levels_per_launch / (per_launch_ms * 1e-3) / 1e9
        pk = fp32_peak if form == "fp32" else fp64_peak
        roof = {"bound": form, "achieved": achieved_gf / 1e3, "peak": pk / 1e3, "unit": "TFLOP/s",
                "frac": achieved_gf / pk, "traffic": traffic, "kernel": dom,
                "hbm_achieved_gbs": achieved_gbs, "hbm_frac": achieved_gbs / hbm,
                "peak_source": "measured in this run (FMA-chain probe)"}
    else:
        roof = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s",
                "frac": achieved_gbs / hbm, "traffic": traffic, "kernel": dom,
                "peak_source": peak_kind}
        if form in ("fp64tc", "bf16x5") and "fft" in dom:
            # the double-float FFTs execute ~10 FP32 operations per FP32-FFT operation:
            # their binding pipe is FP32 issue; the FP32 probe beside the HBM figure
            roof["note"] = ("double-float FFT: FP32-pipe bound (HBM fraction reported as the contract's "
                            "roofline; FP32 FMA probe %.1f TFLOP/s in this run)" % (fp32_peak / 1e3))
    phases = {k: {"ms_per_step": v[0] / 2, "launches_per_step": v[1] // 2} for k, v in ph.items() if v[1]}
    # every phase against its own roofline: algorithmic bytes (tables once per
    # launch for the Legendre phases, whose time includes their pack kernels)
    # over HBM, and for the Legendre phases algorithmic flops (the 2KN / 8KN
    # per transform counts, not the split-product count) over the bf16 dense peak
    for k, v in phases.items():
        if k not in alg or v["ms_per_step"] <= 0:
            continue
        sec = v["ms_per_step"] * 1e-3
        nb = alg[k]["bytes"] * N_LEVELS + (table_bytes(L_MAX, N_THETA, MINC, tab_elem) if "leg" in k else 0)
        v["algorithmic_gb"] = nb / 1e9
        v["achieved_gbs"] = nb / sec / 1e9
        v["hbm_frac"] = v["achieved_gbs"] / hbm
        if "leg" in k:
            fl = alg[k]["flops"] * N_LEVELS
            v["achieved_tflops"] = fl / sec / 1e12
            v["tensor_frac_of_bf16_peak"] = v["achieved_tflops"] / bf16 if bf16 else None
            if form in ("fp64tc", "bf16x5"):
                # 28 (seven digits) or 15 (five digits) digit products per algorithmic multiply-add
                nprod = 28 if form == "fp64tc" else 15
                v["digit_product_tflops"] = nprod * v["achieved_tflops"]
                v["digit_product_frac_of_bf16_peak"] = nprod * v["achieved_tflops"] / bf16 if bf16 else None
    phases64 = {k: {"ms_per_step": v[0], "launches_per_step": v[1]} for k, v in ph64.items() if v[1]}
    # FP64 form's Legendre against the FP64 pipe
    leg64_ms = sum(v[0] for k, v in ph64.items() if "leg" in k)
    leg_flops = sum(alg[k]["flops"] for k in alg if "leg" in k) * N_LEVELS
    fp64_leg_frac = (leg_flops / (leg64_ms * 1e-3) / 1e9) / fp64_peak

    # ---- end to end through the public API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hspec = {k: torch.from_numpy(v).pin_memory() for k, v in spec_np.items()}
        hor2 = or2_levels(N_LEVELS)
        hg = {k: torch.empty(tuple(v.shape), dtype=torch.float64, pin_memory=True) for k, v in gm.items()}
        hl = {k: torch.empty(tuple(v.shape), dtype=torch.complex128, pin_memory=True) for k, v in lmx.items()}

        hfin = {k: v.cpu().pin_memory() for k, v in fin.items()}

        # both batched calls queued back to back (magic_sht_set_host_async), so the
        # synthesis outputs' device->host copies overlap the analysis inputs'
        # host->device copies; every step ends with its host outputs written
        sm.set_host_async(True)

        def host_set():
            sm.transform_to_grid_space(hspec, or2=hor2, out=hg)
            sm.transform_to_lm_space(hfin, out=hl)
            sm.synchronize()

        host_set()  # two untimed steps: the first one allocates the staging slots
        host_set()
        barrier()
        ke = max(1, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(ke):
            host_set()
        barrier()
        dt = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([dt], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
        h2d = sum(v.numel() * v.element_size() for v in hspec.values()) + \
            sum(v.numel() * 8 for v in hfin.values())
        d2h = sum(v.numel() * 8 for v in hg.values()) + sum(v.numel() * 16 for v in hl.values())
        sm.set_host_async(False)
        e2e = {"value": world * N_LEVELS * ke / dt, "unit": "levels/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": ke,
               "path": "transform_to_grid_space + transform_to_lm_space on pinned host arrays, "
                       "asynchronous host batches, synchronized every step"}
        del hspec, hg, hl, hfin

    # ---- one explicit stage of the radial loop (headline form)
    stage = None
    if not args.no_stage:
        stage = stage_measure(sm, s64, spec, N_LEVELS, max(3, min(args.steps, 10)), hbm)

    # ---- the other configurations of the benchmark set (each with every form's
    # levels/s, accuracy against the FP64 form and dominant kernel)
    configs = None
    if not args.no_configs and world == 1:
        sm.close()
        s64.close()
        del gm, lmx, g64, l64
        torch.cuda.synchronize()
        configs = {
            "C0": config_measure("C0", 64, 1, 96, 192, 33, ("fp64", form), local, hbm, full_set=False,
                                 steps=5, cpu_levels=33,
                                 what="scalar + toroidal/poloidal round trip, l_max=64, 96x192, 33 levels"),
            "C1": config_measure("C1", 128, 1, 192, 384, 65, ("fp64", form), local, hbm, steps=5, cpu_levels=2,
                                 what="full 15+10 set, l_max=128, 192x384, 65 levels"),
            "C4": config_measure("C4", 511, 1, 768, 1536, 193, ("fp64", form, "bf16x3"), local, hbm,
                                 batch=65, steps=1, cpu_levels=1,
                                 what="full 15+10 set, l_max=511, 768x1536, 193 levels in batches of 65 "
                                      "(the grids of one batch resident)"),
        }
        configs["C3"] = instances_measure(form, local, max(3, args.warmup), 5)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args.cpu_levels)
        # the same on one core (one level), beside the all-core figure
        one = cpu_baseline(1, threads=1)
        cpu["one_core"] = {k: one[k] for k in ("value", "unit", "cores", "sample")}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "levels/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "median_ms_per_step": statistics.median(per_step), "timing": "graph replay of one step, CUDA events per step",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "bf16x3": "bf16x3+f32", "tf32x2": "tf32x2+f32", "fp64": "f64",
                      "fp64tc": "bf16 digits x7 + exact f32 accumulate; f32x2 FFT",
                      "bf16x5": "bf16 digits x5 + exact f32 accumulate; f32x2 FFT"}[form],
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "form": form, "l_max": L_MAX, "n_theta": N_THETA,
                       "n_phi": N_PHI, "minc": MINC, "n_levels": N_LEVELS,
                       "l2": "inputs larger than L2 (882 MB spectra, 4.6 GB grids per step)",
                       "parallelism": "radial-level replicas" if world > 1 else "single GPU"},
            "fp64_gpu": {"value": lev64, "unit": "levels/s", "ms_per_step": ms64 / k64,
                         "steps": k64, "legendre_frac_of_fp64_peak": fp64_leg_frac,
                         "phases": phases64},
            "rel_l2_vs_fp64_max": acc["max"],
            "every_output_within_1e-6": acc["every_output_within_1e-6"],
            "speedup_vs_fp64_gpu": value / lev64,
            "rel_l2_vs_fp64": acc,
            "accuracy_chain": chain,
            "accuracy_checkpoint_spectra": checkpoint,
            "other_forms": others,
            "boussinesq_default_set": bouss,
            "roofline": roof,
            "phases": phases,
            "peaks": {"fp64_gflops": fp64_peak, "fp32_gflops": fp32_peak, "hbm_gbs": hbm,
                      "bf16_tflops": bf16, "source": peak_kind},
            "gpu_launches": launches,
            "clocks": clocks,
            "e2e": e2e,
            "stage": stage,
            "configs": configs,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def instances_measure(form, local, warmup, steps):
    """The sixteen-instance batching case (see instances_arm) in `form` and in
    3xBF16, as a nested entry of the headline line: each as one group (one
    pack + one persistent launch per direction and field kind over all sixteen
    instances) and as the instances' own launches."""
    out = {}
    r = None
    runs = [(form, True), (form, False), ("bf16x3", True), ("bf16x3", False)]
    for f, grp in runs:
        r = instances_run(f, local, warmup, steps, group=grp)
        out[f + ("_group" if grp else "")] = {k: r[k] for k in ("value", "unit", "ms_per_step", "levels_per_step",
                                                                  "gpu_launches_per_step")}
    out["instances"] = r["instances"]
    out["what"] = ("sixteen mixed-size instances, both transform sets, captured in one CUDA graph: "
                   "<form>_group = one pack + one persistent tensor-core launch per direction and field kind "
                   "over every instance (magic_sht_group_*), <form> = each instance's own launches")
    return out


def instances_run(form, local, warmup, steps, group=False, max_levels=None):
    """Sixteen independent instances of mixed size (l_max in {63, 127, 255},
    minc in {1, 4}, {33, 65, 129} radial levels, n_theta = 3(l_max+1)/2,
    n_phi = 2 n_theta / minc; a fixed seeded list), both transform sets of every
    instance captured into one CUDA graph on one stream and replayed.  The
    analysis inputs are the instance's synthesis grids.  group: the instances'
    Legendre sums as one launch per direction and field kind (SHTGroup)."""
    import numpy as np
    import torch
    from magic_gb300 import SHT, SHTGroup
    from magic_gb300.workload import grid_space_inputs, or2_levels, FORWARD_FROM_INVERSE
    rng = np.random.default_rng(1234)
    insts, desc = [], []
    for i in range(16):
        L = int(rng.choice([63, 127, 255]))
        minc = int(rng.choice([1, 4]))
        R = int(rng.choice([33, 65, 129]))
        if max_levels:  # profiling cases: every instance capped at max_levels levels
            R = min(R, max_levels)
        N = 3 * (L + 1) // 2
        P = 2 * N // minc
        s = SHT(L, minc, N, P, precision=form, device=local)
        spec = {k: torch.from_numpy(v).cuda() for k, v in grid_space_inputs(L, minc, R, seed=500 + i).items()}
        or2 = torch.from_numpy(or2_levels(R)).cuda()
        g = s.transform_to_grid_space(spec, or2=or2)
        fin = {k: g[v] for k, v in FORWARD_FROM_INVERSE.items()}
        lm = s.transform_to_lm_space(fin)
        insts.append((s, spec, or2, g, fin, lm, R))
        desc.append({"l_max": L, "minc": minc, "n_theta": N, "n_phi": P, "levels": R})
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    grp = None
    with torch.cuda.stream(side):
        for s, *_ in insts:
            s.set_stream(side.cuda_stream)
        if group:
            grp = SHTGroup([i[0] for i in insts])
            args = ([i[1] for i in insts], [i[2] for i in insts], [i[3] for i in insts],
                    [i[4] for i in insts], [i[5] for i in insts])

            def step():
                grp.transform_to_grid_space(args[0], or2s=args[1], outs=args[2])
                grp.transform_to_lm_space(args[3], outs=args[4])
        else:
            def step():
                for s, spec, or2, g, fin, lm, _ in insts:
                    s.transform_to_grid_space(spec, or2=or2, out=g)
                    s.transform_to_lm_space(fin, out=lm)
        step()  # sizes the workspaces (and uploads the group's instance tables)
        side.synchronize()
        n0 = sum(i[0].launch_count() for i in insts)
        insts[0][0].graph_begin()
        try:
            step()
        finally:
            gr = insts[0][0].graph_end()
        launches = sum(i[0].launch_count() for i in insts) - n0
        for _ in range(max(warmup, 3)):
            insts[0][0].graph_launch(gr)
        side.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(side)
        for _ in range(steps):
            insts[0][0].graph_launch(gr)
        e1.record(side)
        side.synchronize()
    ms = e0.elapsed_time(e1)
    for s, *_ in insts:
        s.device_status()
    insts[0][0].graph_destroy(gr)
    levels = sum(d["levels"] for d in desc)
    if grp is not None:
        grp.close()
    for s, *_ in insts:
        s.close()
    del insts
    torch.cuda.synchronize()
    return {"metric": "SHT radial levels/s, sixteen mixed instances in one graph",
            "value": levels * steps / (ms * 1e-3), "unit": "levels/s", "n_gpus": 1,
            "steps": steps, "warmup": max(warmup, 3), "ms_per_step": ms / steps,
            "higher_is_better": True, "form": form, "group": group, "levels_per_step": levels,
            "gpu_launches_per_step": launches,
            "timing": "graph replay, CUDA events on the replay stream", "instances": desc}


def instances_arm(args):
    """Sixteen independent instances of mixed size (l_max in {63, 127, 255},
    minc in {1, 4}, {33, 65, 129} radial levels, n_theta = 3(l_max+1)/2,
    n_phi = 2 n_theta / minc; a fixed seeded list), both transform sets of every
    instance captured into one CUDA graph on one stream and replayed.  The
    analysis inputs are the instance's synthesis grids."""
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    form = "bf16x3" if args.form == "auto" else args.form
    r = instances_run(form, local, args.warmup, args.steps, group=args.group,
                      max_levels=args.levels if args.levels != N_LEVELS else None)
    if rank == 0:
        print(json.dumps(r), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.instances:
        instances_arm(args)
        return
    our_arm(args)


if __name__ == "__main__":
    main()
