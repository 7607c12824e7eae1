#!/usr/bin/env python
"""ARMA(1,1) REML voxelwise GLM throughput on GB300 (voxels/s).

One step = one complete ``fit_glm_arma11`` of the 200,000-voxel workload
(N = 400 as 2 runs x 200, p = 20, the 33 x 33 grid on [-0.8, 0.8] -> 561 valid
(a, b) pairs, default hierarchical selector): FP64 grid factors, per-voxel
scaling and residualisation, the criterion at every pair, selection and the GLS
refit with t, F, R^2, sigma2 and lambda. ``value`` keeps the data resident in
HBM; ``e2e`` calls the same public API with pinned host buffers (host->device
copy of the data and device->host copy of the results inside the timed region).

Usage: python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Multi-GPU (torchrun): every rank fits its own 200,000 voxels (weak scaling, no
data-path collective); the step time is the max over ranks.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ARMA REML voxels/s: learned-seeded vs full-grid on GB300 at beta rel err ≤1e-4"
GRID = 33
L2_BYTES = 129 * 2**20


def workload_config(V: int, selector: str) -> dict:
    return {
        "workload": f"synthetic fMRI, N=400 (2 runs x 200), V={V:,} voxels, p=20, "
                    f"(a,b) grid 33x33 on [-0.8,0.8] -> 561 valid pairs, {selector} selector",
        "voxels": V, "timepoints": 400, "regressors": 20, "pairs": 561, "selector": selector,
        "l2": "inputs larger than L2 (Y is 320 MB fp32 > 129 MB L2); no flush needed",
    }


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return dist, dist.get_rank(), ws, int(os.environ.get("LOCAL_RANK", "0"))
    return None, 0, 1, 0


def cpu_baseline(w, n_voxels: int) -> dict:
    """The reference's default CPU fit (torch CPU port) on a bounded voxel sample."""
    from oracle import cpu_port

    cores = len(os.sched_getaffinity(0))
    torch.set_num_threads(cores)
    g = torch.linspace(-0.8, 0.8, GRID).numpy()
    sub = w.Y[:n_voxels]
    cpu_port.fit(sub[:64], w.X, g, g, w.run_starts)  # warm the kernels
    t0 = time.perf_counter()
    cpu_port.fit(sub, w.X, g, g, w.run_starts)
    dt = time.perf_counter() - t0
    return {"value": n_voxels / dt, "unit": "voxels/s", "cores": cores, "kind": "port",
            "sample": f"{n_voxels} voxels of the same workload, float32, default hierarchical selector, "
                      f"{dt:.1f} s"}


def run_reference(args) -> None:
    dist, rank, ws, _ = dist_init()
    if rank != 0:
        return
    from fastfuncstuff_gb300 import synth
    from oracle import cpu_port

    w = synth.workload(1, V=args.ref_voxels * (args.steps + args.warmup))
    cores = len(os.sched_getaffinity(0))
    torch.set_num_threads(cores)
    g = torch.linspace(-0.8, 0.8, GRID).numpy()
    n = args.ref_voxels
    for s in range(args.warmup):
        cpu_port.fit(w.Y[s * n:(s + 1) * n], w.X, g, g, w.run_starts)
    t0 = time.perf_counter()
    for s in range(args.warmup, args.warmup + args.steps):
        cpu_port.fit(w.Y[s * n:(s + 1) * n], w.X, g, g, w.run_starts)
    dt = (time.perf_counter() - t0) / args.steps
    value = n / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded workload)",
        "config": workload_config(args.voxels, "hierarchical"),
        "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": cores, "kind": "port",
                         "sample": f"{n} voxels per step of the same workload on {cores} host threads"},
        "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args) -> None:
    from fastfuncstuff_gb300 import fit_glm_arma11, synth
    from fastfuncstuff_gb300.glm import engine

    dist, rank, ws, local = dist_init()
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    w = synth.workload(1, V=args.voxels, seed=1001 + 7919 * rank)
    g = torch.linspace(-0.8, 0.8, GRID)
    Xd = torch.from_numpy(w.X).to(dev)
    Yd = torch.from_numpy(w.Y).to(dev)
    kw = dict(tr=2.0, a_grid=g, b_grid=g, run_starts=w.run_starts, device=dev, verbose=False,
              force_exhaustive_search=args.selector == "exhaustive", projector=args.projector)

    def step():
        return fit_glm_arma11(Yd, Xd, return_device=True, **kw)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    timer = engine.StageTimer()
    engine.set_stage_timer(timer)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        barrier()
    engine.set_stage_timer(None)
    ms = e0.elapsed_time(e1) / args.steps
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * args.voxels / (ms / 1e3)
    stages = timer.summary()

    # roofline of the dominant kernel (device time measured above, per launch)
    pk = peaks()
    V, T, K, P = args.voxels, 400, 20, 561
    dom = max(stages.items(), key=lambda kv: kv[1]["mean_ms"] * kv[1]["calls"])[0]
    roof = None
    if dom == "ffs_reml_project_tc":
        flops = 3 * 2.0 * V * P * K * 448  # three fp16 products over the padded k extent
        ach = flops / (stages[dom]["mean_ms"] / 1e3) / 1e12
        roof = {"kernel": dom, "bound": "tensor", "achieved": ach, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": ach / pk["bf16_tflops"], "traffic": None,
                "work": "issued fp16 tensor flops = 3 x 2 x V x P x K x 448 (k padded to 64)",
                "peak_src": pk["src"]}
    elif dom in ("ffs_reml_surface", "ffs_reml_project_simt"):
        if dom == "ffs_reml_surface":
            flops = 2.0 * 3 * V * P * T  # 3 FMA per (voxel, pair, time point)
        else:
            flops = 2.0 * V * P * K * T
        ach = flops / (stages[dom]["mean_ms"] / 1e3) / 1e12
        sm = (clk.summary()["sm_mhz"] or 1900.0) * 1e6
        fp32_peak = 152 * 128 * 2 * sm / 1e12
        roof = {"kernel": dom, "bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": ach / fp32_peak, "traffic": None,
                "work": "fp32 FMA flops of the O(T) recurrences", "peak_src": "152 SMs x 128 FMA/clk at the sampled clock"}

    line = {
        "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded workload, see fastfuncstuff_gb300/synth.py)",
        "config": workload_config(args.voxels, args.selector),
        "roofline": roof,
        "stages_ms": {k: round(v["mean_ms"], 4) for k, v in stages.items()},
        "gpu_launches": timer.launches,
        "clocks": clk.summary(),
    }

    if rank == 0 and not args.no_e2e:
        # end to end through the public API from pinned host buffers
        Yh = torch.from_numpy(w.Y).pin_memory()
        Xh = torch.from_numpy(w.X)
        kwh = dict(kw)
        for _ in range(2):
            r = fit_glm_arma11(Yh, Xh, **kwh)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            r = fit_glm_arma11(Yh, Xh, **kwh)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / args.e2e_steps
        d2h = sum(t.numel() * t.element_size() for t in (r.betas, r.tstats, r.r2, r.arma_params, r.arma_lambda,
                                                         r.reml_likelihood, r.sigma2, r.fstats))
        line["e2e"] = {"value": args.voxels / dt, "unit": "voxels/s", "h2d_bytes_per_step": Yh.numel() * 4 + Xh.numel() * 4,
                       "d2h_bytes_per_step": d2h, "ms_per_step": dt * 1e3}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_voxels)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--voxels", type=int, default=200_000)
    ap.add_argument("--selector", default="hierarchical", choices=["hierarchical", "exhaustive"])
    ap.add_argument("--projector", default="tc", choices=["tc", "simt"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-voxels", type=int, default=4000)
    ap.add_argument("--ref-voxels", type=int, default=4000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
