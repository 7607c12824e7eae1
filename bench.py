#!/usr/bin/env python
"""ARMA(1,1) REML voxelwise GLM throughput on GB300 (voxels/s): learned-seeded
refine vs the full-grid solve.

One step = one complete ``fit_glm_arma11`` of the 200,000-voxel workload
(N = 400 as 2 runs x 200, p = 20, the 33 x 33 grid on [-0.8, 0.8] -> 561 valid
(a, b) pairs): FP64 grid factors, per-voxel scaling and residualisation, the
(a, b) search, and the GLS refit with t, F, R^2, sigma2 and lambda.
``value`` is the learned-seeded step (each voxel's 5 x 5 window around the
proposal of the MLP, one re-centred round, the strip next to the identity line
for voxels near it, the full grid for the voxels still on a window edge or
beaten by a strip pair); ``full_grid`` is the same fit evaluating all 561 pairs
(the reference's default hierarchical selector). The proposal is trained on
the GPU before timing (6M voxels simulated with this design, full-grid
labels, 40 epochs). ``value`` keeps the data resident in HBM; ``e2e`` calls the same
public API with pinned host buffers (host->device copy of the data and
device->host copy of the results inside the timed region).

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


WORKLOADS = {
    1: "N=400 (2 runs x 200), p=20",
    2: "N=855 (4 runs of 180/220/240/260, 5% censored), p=18, 20 HRF-group designs (Zipf)",
    3: "N=600 (3 runs x 200), p=130 single-trial design",
    4: "N=400 (2 runs x 200), p=20, learned-proposal inference size",
}


def workload_config(V: int, cid: int = 1, T: int = 400, K: int = 20) -> dict:
    mb = V * T * 4 / 1e6
    return {
        "workload": f"synthetic fMRI, {WORKLOADS[cid]}, V={V:,} voxels, (a,b) grid 33x33 on [-0.8,0.8] -> 561 "
                    f"valid pairs",
        "voxels": V, "timepoints": T, "regressors": K, "pairs": 561,
        "l2": f"inputs larger than L2 (Y is {mb:.0f} MB fp32 > 129 MB L2); no flush needed",
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


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith(("model name", "cpu model")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_baseline(w, n_voxels: int, n_exhaustive: int) -> dict:
    """The reference's CPU fit (torch CPU port) on bounded voxel samples: the
    default hierarchical selector (``value``) and force_exhaustive_search."""
    from oracle import cpu_port

    cores = len(os.sched_getaffinity(0))
    torch.set_num_threads(cores)
    g = torch.linspace(-0.8, 0.8, GRID).numpy()
    cpu_port.fit(w.Y[:64], w.X, g, g, w.run_starts)  # warm the kernels
    t0 = time.perf_counter()
    cpu_port.fit(w.Y[:n_voxels], w.X, g, g, w.run_starts)
    dt = time.perf_counter() - t0
    out = {"value": n_voxels / dt, "unit": "voxels/s", "cores": cores, "cpu": cpu_model(), "kind": "port",
           "sample": f"{n_voxels} voxels of the same workload, float32, default hierarchical selector, "
                     f"{dt:.1f} s on {cores} threads"}
    if n_exhaustive > 0:
        t0 = time.perf_counter()
        cpu_port.fit(w.Y[:n_exhaustive], w.X, g, g, w.run_starts, exhaustive=True)
        de = time.perf_counter() - t0
        out["exhaustive"] = {"value": n_exhaustive / de, "unit": "voxels/s",
                             "sample": f"{n_exhaustive} voxels, float32, force_exhaustive_search, {de:.1f} s"}
    return out


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
        "config": workload_config(args.voxels or 200_000),
        "method": "the reference's default CPU fit (full grid, hierarchical selector)",
        "cpu_baseline": {"value": value, "unit": "voxels/s", "cores": cores, "cpu": cpu_model(), "kind": "port",
                         "sample": f"{n} voxels per step of the same workload on {cores} host threads"},
        "e2e": {"value": value, "unit": "voxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# DRAM bytes per voxel of one launch (dram__bytes_read.sum + dram__bytes_write.sum)
# from ncu --set full captures of the N=400, p=20, 561-pair workload at
# 100k-217k voxels; traffic grows with the voxels, so a launch's traffic is this
# times the voxels it processes. None for other shapes.
NCU_DRAM_BYTES_PER_VOXEL = {
    (400, 20, "ffs_reml_gls_grouped"): 1866.0,
    (400, 20, "ffs_reml_surface"): 5524.0,
}


def roofline(dom: str, ms_step: float, launches: float, T: int, K: int, P: int, pk: dict, sm_mhz,
             work: dict) -> dict:
    """The dominant kernel against its bound: the algorithmic work of ALL its
    launches in one step (``work``: "voxels" it processed, "pair_evals" for the
    window kernels, "designs" for the grid build) over their summed device time
    ``ms_step`` (per-call CUDA events of an eager pass), i.e. the launches'
    average rate; ``launches`` is how many there were per step."""
    r = _roofline(dom, ms_step, T, K, P, pk, sm_mhz, work)
    r["ms_per_step"] = ms_step
    r["launches_per_step"] = launches
    per_voxel = NCU_DRAM_BYTES_PER_VOXEL.get((T, K, dom)) if P == 561 else None
    if per_voxel is not None:
        r["traffic"] = per_voxel * work["voxels"] / max(launches, 1)
        r["traffic_unit"] = ("bytes per launch: ncu DRAM read + write per voxel (from a 100k-217k voxel capture) x "
                             "the voxels of the step's launches / launches")
    return r


def _roofline(dom: str, ms_step: float, T: int, K: int, P: int, pk: dict, sm_mhz, work: dict) -> dict:
    sec = ms_step / 1e3
    V = work["voxels"]
    fp32_peak = 152 * 128 * 2 * (sm_mhz or 1900.0) * 1e6 / 1e12
    if dom in ("ffs_reml_project_tc", "ffs_reml_project_tc_list"):
        k_eff = (T + 15) // 16 * 16
        cols = work.get("pair_evals", V * P) if dom == "ffs_reml_project_tc_list" else V * P
        flops = 3 * 2.0 * cols * K * k_eff
        ach = flops / sec / 1e12
        return {"kernel": dom, "bound": "tensor", "achieved": ach, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                "frac": ach / pk["bf16_tflops"], "traffic": None, "peak_src": pk["src"] + " (bf16 burst)",
                "work": "3 fp16 products x 2 x (voxel, pair) x K x T (k rounded to 16)"}
    if dom in ("ffs_reml_surface", "ffs_reml_window"):
        n = work.get("pair_evals", V * P) if dom == "ffs_reml_window" else V * P
        flops = 4.0 * n * T  # v_t = z_t - m_t v_t-1 and s += v_t^2 / D_t: 2 FMA
        ach = flops / sec / 1e12
        return {"kernel": dom, "bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": ach / fp32_peak, "traffic": None, "peak_src": "152 SMs x 128 FMA/clk at the sampled clock",
                "work": "2 FMA per (voxel, pair, time point) of the O(T) recurrences"}
    if dom == "ffs_reml_gls_grouped":
        flops = V * (3 * 2.0 * K * T + 6.0 * T)
        ach = flops / sec / 1e12
        return {"kernel": dom, "bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": ach / fp32_peak, "traffic": None, "peak_src": "152 SMs x 128 FMA/clk at the sampled clock",
                "work": "G'y, X b0 and G'r (3 K x T products) and the whitening recurrence per voxel"}
    if dom in ("ffs_grid_build", "ffs_grid_build_designs"):
        # FP64: the whitened design (2 T K) and its Gram matrix (T K (K + 1)) per (design, pair)
        items = P * work.get("designs", 1)
        flops = items * (2.0 * T * K * (K + 1) + 4.0 * T * K)
        ach = flops / sec / 1e12
        return {"kernel": dom, "bound": "fp64", "achieved": ach, "peak": 1.25, "unit": "TFLOP/s",
                "frac": ach / 1.25, "traffic": None, "peak_src": "nominal GB300 FP64 (not measured)",
                "work": "FP64 X_w = L^-1 X and X_w'X_w per (design, pair)"}
    # the rest stream HBM (prep: Y in; rows/time-major and the fp16 split out)
    ld = (T + 63) // 64 * 64
    byts = V * (T * 4 + T * 4 + 2 * ld * 2 + 16)
    ach = byts / sec / 1e9
    return {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": ach / pk["hbm_gbs"], "traffic": None, "peak_src": pk["src"],
            "work": "bytes: Y read, residualised rows and fp16 hi/lo written"}


def learned_quality(args, w, Yd, Xd, kw, kw_l, prop, lay, g, tinfo) -> tuple[dict, float, int]:
    """Correctness of the learned-seeded fit on this workload.

    * against the GPU full grid (exhaustive argmin) on every voxel: agreement,
      and for the voxels that disagree the criterion gap
      (crit_learned - crit_full) / |crit_full|;
    * against the FP64 oracle (exhaustive, the float32 mode's scaling in
      float64) on a fixed sample (every (V // fp64_voxels)-th voxel):
      agreement with its argmin, the gap of the disagreeing voxels on the FP64
      surface, and the betas' and t's relative error (per voxel, max-norm).
    Returns (quality, window (voxel, pair) evaluations, fallback voxels)."""
    from fastfuncstuff_gb300 import fit_glm_arma11
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    V = Yd.shape[0]
    exh = fit_glm_arma11(Yd, Xd, return_device=True, **dict(kw, force_exhaustive_search=True))
    hier = fit_glm_arma11(Yd, Xd, return_device=True, **dict(kw, force_exhaustive_search=False))
    lr = fit_glm_arma11(Yd, Xd, return_device=True, **kw_l)
    same = (lr.arma_params == exh.arma_params).all(1)
    c_l = lr.reml_likelihood.double()
    c_f = exh.reml_likelihood.double()
    gap = ((c_l - c_f) / c_f.abs().clamp(min=1.0))[~same]
    f_all = engine.build_factors(Xd, G.make_grid(g, g), lay)
    ls = learned.learned_search(Yd, f_all, prop, lay, recenter=args.recenter, count_evals=True)
    pair_evals = float(ls.stats["pair_evals"].item()) if torch.is_tensor(ls.stats["pair_evals"]) else 0.0
    n_fb = int(round(ls.stats["fallback"] * V))
    q = {
        "agreement_with_full_grid": float(same.float().mean().item()),
        "disagreeing_voxels": int((~same).sum().item()),
        "crit_gap_max_of_disagreeing": float(gap.max().item()) if gap.numel() else 0.0,
        "disagreeing_with_gap_gt_1e-6": int((gap > 1e-6).sum().item()),
        "first_window_on_edge": float(ls.stats["edge_first"]), "full_grid_fallback": ls.stats["fallback"],
        "strip_voxels": int(ls.stats["strip_voxels"].item()) if ls.stats.get("strip_voxels") is not None else 0,
        "recenter_rounds": args.recenter, "window_pair_evals_per_voxel": pair_evals / V,
    }
    # context: the reference's default selector (AFNI's hierarchical descent
    # from (0, 0)) against the same exhaustive argmin, on the same voxels
    same_h = (hier.arma_params == exh.arma_params).all(1)
    gap_h = ((hier.reml_likelihood.double() - c_f) / c_f.abs().clamp(min=1.0))[~same_h]
    q["reference_default_selector"] = {
        "agreement_with_full_grid": float(same_h.float().mean().item()),
        "disagreeing_with_gap_gt_1e-6": int((gap_h > 1e-6).sum().item()),
        "crit_gap_max_of_disagreeing": float(gap_h.max().item()) if gap_h.numel() else 0.0,
    }
    if args.transfer:
        # a proposal trained on a family of four other designs of this
        # workload's kind (fresh task onsets and motion), used on this design
        from fastfuncstuff_gb300 import synth

        fam = torch.from_numpy(np.stack([synth.workload1_design(sd) for sd in (101, 102, 103, 104)])).to(Yd.device)
        prop_fam, info_fam = learned.train_proposal(fam, lay, g, g, n_voxels=args.train_voxels,
                                                    epochs=args.train_epochs)
        full_b = engine.search(Yd, f_all, hierarchical=False).best
        lt = learned.learned_search(Yd, f_all, prop_fam, lay, recenter=args.recenter)
        q["held_out_design"] = {
            "proposal": "trained on 4 other designs of this workload's kind (synth.workload1_design seeds 101-104), "
                        "none of them this fit's design",
            "agreement_with_full_grid": float((lt.best == full_b).float().mean().item()),
            "full_grid_fallback": lt.stats["fallback"],
            "train_s": round(info_fam["label_s"] + info_fam["train_s"], 2),
        }
    if args.fp64_voxels > 0:
        from oracle import reml as o

        step = max(1, V // args.fp64_voxels)
        sub = np.arange(0, V, step)[: args.fp64_voxels]
        t0 = time.perf_counter()
        ref = o.fit_glm_arma11(w.Y[sub], w.X, a_grid=g.numpy(), b_grid=g.numpy(), run_starts=w.run_starts,
                               use_double=True, fp64_scaled=True, force_exhaustive_search=True,
                               save_profile_likelihoods=True)
        grid = G.make_grid(g, g)
        pa = lr.arma_params[sub].cpu().numpy().astype(np.float32)
        idx_l = grid.index_of(pa[:, 0], pa[:, 1])
        agree = idx_l == ref.arma_index
        v = np.nonzero(~agree)[0]
        surf = ref.reml_lklhd_surface
        g64 = (surf[v, idx_l[v]] - surf[v, ref.arma_index[v]]) / np.maximum(np.abs(surf[v, ref.arma_index[v]]), 1.0)

        def rel(got, want):
            num = np.abs(got.astype(np.float64) - want).max(-1)
            return num / np.maximum(np.abs(want).max(-1), 1e-12)

        rb = rel(lr.betas[sub].cpu().numpy(), ref.betas)
        rt = rel(lr.tstats[sub].cpu().numpy(), ref.tstats)
        q["vs_fp64"] = {
            "sample": f"{sub.size} voxels (every {step}th), FP64 oracle exhaustive search and GLS "
                      f"({time.perf_counter() - t0:.1f} s on the host)",
            "agreement": float(agree.mean()), "disagreeing_voxels": int(v.size),
            "crit_gap_max_of_disagreeing": float(g64.max()) if v.size else 0.0,
            "beta_rel_err_max": float(rb[agree].max()), "tstat_rel_err_max": float(rt[agree].max()),
            "beta_rel_err_le_1e-4": float((rb <= 1e-4).mean()),
            "beta_rel_err_max_all_voxels": float(rb.max()),
        }
    q.update({k: round(v, 3) if isinstance(v, float) else v for k, v in tinfo.items()})
    return q, pair_evals, n_fb


def run_gb300(args) -> None:
    from fastfuncstuff_gb300 import fit_glm_arma11, synth
    from fastfuncstuff_gb300.glm import engine, learned
    from fastfuncstuff_gb300.glm import grid as G

    dist, rank, ws, local = dist_init()
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    cid = args.workload
    w = synth.workload(cid, V=args.voxels, seed=1000 + cid + 7919 * rank)
    V = w.Y.shape[0]
    g = torch.linspace(-0.8, 0.8, GRID)
    Yd = torch.from_numpy(w.Y).to(dev)
    kw = dict(tr=2.0, a_grid=g, b_grid=g, run_starts=w.run_starts, device=dev, verbose=False,
              force_exhaustive_search=args.selector == "exhaustive")
    grouped = w.designs is not None
    if grouped:  # one design per HRF group: the grouped API, full grid
        from fastfuncstuff_gb300 import fit_glm_arma11_grouped

        designs = {h: torch.from_numpy(x).to(dev) for h, x in w.designs.items()}
        kw["tau"] = w.tau
        T, K = next(iter(w.designs.values())).shape

        def fit(Yx, Xx, **k):
            return fit_glm_arma11_grouped(Yx, designs, w.groups, **k)
        Xd = None
        prop, tinfo, kw_l = None, {}, None
    else:
        Xd = torch.from_numpy(w.X).to(dev)
        T, K = w.X.shape
        fit = fit_glm_arma11
        lay = G.run_layout(w.T, w.run_starts)
        if args.proposal:
            prop = learned.ArmaProposal.load(args.proposal, dev)
            tinfo = {"proposal": f"loaded from {Path(args.proposal).name}"}
        else:
            prop, tinfo = learned.train_proposal(Xd, lay, g, g, n_voxels=args.train_voxels, epochs=args.train_epochs)
            if args.save_proposal and rank == 0:
                prop.save(args.save_proposal)
        kw_l = dict(kw, proposal=prop, proposal_recenter=args.recenter)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed(kwargs, label):
        def step():
            return fit(Yd, Xd, return_device=True, **kwargs)

        for _ in range(args.warmup):
            step()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            barrier()
            torch.cuda.nvtx.range_push(f"timed_{label}")  # selects the timed launches for an ncu launch list
            e0.record()
            for _ in range(args.steps):
                step()
            e1.record()
            barrier()
            torch.cuda.nvtx.range_pop()
        ms = e0.elapsed_time(e1) / args.steps
        if dist is not None:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        # the stage breakdown and launch count: as many steps again, eagerly,
        # under the per-call timer (outside the timed region; the timer
        # serialises the grid build with the prep, so each stage time is the
        # kernel's own)
        timer = engine.StageTimer()
        engine.set_stage_timer(timer)
        for _ in range(args.steps):  # eager: the timer does not see into graph replays
            fit(Yd, Xd, return_device=True, **dict(kwargs, cuda_graphs=False))
        barrier()
        engine.set_stage_timer(None)
        st = timer.summary()
        return ms, st, timer.launches // args.steps, clk.summary()

    ms_f, st_f, l_f, clk_f = timed(kw, "full_grid")
    value_f = ws * V / (ms_f / 1e3)
    pk = peaks()
    P = 561

    def dominant(st, voxels_of):
        """(name, roofline) of the entry point with the most device time per step."""
        name, d = max(st.items(), key=lambda kv: kv[1]["mean_ms"] * kv[1]["calls"])
        work = {"voxels": voxels_of(name)}
        return name, d["mean_ms"] * d["calls"] / args.steps, d["calls"] / args.steps, work

    dom_f, ms_df, n_df, work_f = dominant(st_f, lambda n: V)
    if grouped:
        work_f["designs"] = len(w.designs)
    roof_f = roofline(dom_f, ms_df, n_df, T, K, P, pk, clk_f["sm_mhz"], work_f)
    if grouped:
        ms_l, st_l, l_l, clk_l, value, roof, quality = ms_f, st_f, l_f, clk_f, value_f, roof_f, None
        st_e, ms_e = st_f, ms_f
    else:
        ms_l, st_l, l_l, clk_l = timed(kw_l, "learned")
        value = ws * V / (ms_l / 1e3)
        # the learned step is mostly replayed from CUDA graphs, which the
        # per-call timer does not see into: its stage breakdown comes from an
        # eager pass
        ms_e, st_e, l_e, _ = timed(dict(kw_l, cuda_graphs=False), "learned_eager")
        quality, pair_evals, n_fb = learned_quality(args, w, Yd, Xd, kw, kw_l, prop, lay, g, tinfo)
        # the eager step's GLS launches cover every voxel and, again, the
        # fallback voxels; its window kernels cover pair_evals (voxel, pair)s
        dom, ms_d, n_d, work = dominant(st_e, lambda n: V + n_fb if n == "ffs_reml_gls_grouped" else V)
        work["pair_evals"] = pair_evals
        roof = roofline(dom, ms_d, n_d, T, K, P, pk, clk_l["sm_mhz"], work)

    method = ("full grid, one design per HRF group (fit_glm_arma11_grouped)" if grouped else
              f"learned-seeded 5x5 window refine, {args.recenter} re-centred round, the strip next to the identity "
              f"line for voxels within 2 lattice steps of it, full grid for window edges and voxels a strip pair "
              f"beats; window rounds and fallback replayed from CUDA graphs, the window pairs' GLS launched "
              f"beside them")
    line = {
        "metric": METRIC, "value": value, "unit": "voxels/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_l, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded workload, see fastfuncstuff_gb300/synth.py)",
        "config": workload_config(V, cid, T, K),
        "method": method,
        "roofline": roof,
        "stages_ms": {k: round(v["mean_ms"] * v["calls"] / args.steps, 4) for k, v in st_e.items()},
        "stages_note": ("per-call device times of an eager (graphs off) pass of the same step, the grid build "
                        "serialised with the prep" if not grouped else ""),
        "ms_per_step_eager": ms_e,
        "gpu_launches": l_l if grouped else l_e,
        "clocks": clk_l,
        "learned": quality,
        "full_grid": {"value": value_f, "ms_per_step": ms_f, "selector": args.selector,
                      "learned_over_full": value / value_f, "roofline": roof_f,
                      "stages_ms": {k: round(v["mean_ms"] * v["calls"] / args.steps, 4) for k, v in st_f.items()},
                      "gpu_launches": l_f, "clocks": clk_f},
    }

    if grouped and args.grouped_learned:
        # the learned-seeded fit of the grouped workload: a proposal trained on
        # the family of the groups' designs, each design's voxels searched
        # against that design's view of one multi-design grid build
        fam = torch.stack([designs[h] for h in sorted(designs)])
        lay_g = G.run_layout(T, w.run_starts, w.tau)
        prop_g, tinfo_g = learned.train_proposal(fam, lay_g, g, g, n_voxels=args.train_voxels,
                                                 epochs=args.train_epochs)
        kw_g = dict(kw, proposal=prop_g, proposal_recenter=args.recenter)
        ms_g, st_g, l_g, clk_g = timed(kw_g, "grouped_learned")
        r_l = fit(Yd, Xd, return_device=True, **kw_g)
        r_f = fit(Yd, Xd, return_device=True, **dict(kw, force_exhaustive_search=True))  # the argmin it seeks
        same = (r_l.arma_params == r_f.arma_params).all(1)
        line["grouped_learned"] = {
            "value": ws * V / (ms_g / 1e3), "unit": "voxels/s", "ms_per_step": ms_g,
            "learned_over_full": ms_f / ms_g, "agreement_with_exhaustive_full_grid": float(same.float().mean()),
            "full_grid_fallback": float(r_l.learned_fallback), "gpu_launches": l_g, "clocks": clk_g,
            "stages_ms": {k: round(v["mean_ms"] * v["calls"] / args.steps, 4) for k, v in st_g.items()},
            "proposal": f"trained on the {fam.shape[0]} group designs", **tinfo_g}

    if args.dsort > 0 and not grouped and rank == 0:
        # the full-grid fit with Q voxelwise regressors per voxel (-dsort): the
        # search is unchanged, the final GLS is the extended one
        rng = np.random.default_rng(77)
        base = rng.standard_normal((args.dsort, T)).astype(np.float32)
        Dd = (torch.from_numpy(base).to(dev)[None] +
              0.3 * torch.randn(V, args.dsort, T, device=dev, generator=torch.Generator(dev).manual_seed(5)))
        kw_d = dict(kw, dsort=Dd)
        ms_d, st_d, l_d, clk_d = timed(kw_d, "dsort")
        dk = st_d.get("ffs_reml_gls_dsort", {"mean_ms": float("nan"), "calls": 1})
        q = args.dsort
        # per voxel: G'y, U'y, G'D, U'D (2 + 2q K x T products), whitening of y,
        # D and the residual, the residual itself (K + q per sample)
        flops = V * ((2 + 2 * q) * 2.0 * K * T + (2 + q) * 6.0 * T + 2.0 * (K + q) * T)
        sec = dk["mean_ms"] * 1e-3
        peak = 152 * 128 * 2 * clk_d["sm_mhz"] * 1e6 / 1e12 if clk_d.get("sm_mhz") else float("nan")
        line["dsort"] = {"q": q, "value": ws * V / (ms_d / 1e3), "unit": "voxels/s", "ms_per_step": ms_d,
                         "gls_dsort_ms": dk["mean_ms"], "gpu_launches": l_d, "clocks": clk_d,
                         "roofline": {"kernel": "ffs_reml_gls_dsort", "bound": "fp32", "achieved": flops / sec / 1e12,
                                      "peak": peak, "unit": "TFLOP/s", "frac": flops / sec / 1e12 / peak,
                                      "work": "G'y, U'y, G'D, U'D, the whitening recurrences and the residual"},
                         "stages_ms": {k: round(v["mean_ms"] * v["calls"] / args.steps, 4) for k, v in st_d.items()}}
    if rank == 0 and not args.no_e2e:
        # end to end through the public API from pinned host buffers
        Yh = torch.from_numpy(w.Y).pin_memory()
        Xh = None if grouped else torch.from_numpy(w.X)
        e2e = {}
        for name, kwh in ((("full_grid", kw),) if grouped else (("learned", kw_l), ("full_grid", kw))):
            for _ in range(2):
                r = fit(Yh, Xh, **kwh)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                r = fit(Yh, Xh, **kwh)
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / args.e2e_steps
            d2h = sum(t.numel() * t.element_size() for t in (r.betas, r.tstats, r.r2, r.arma_params,
                                                             r.arma_lambda, r.reml_likelihood, r.sigma2, r.fstats))
            h2d = Yh.numel() * 4 + (0 if Xh is None else Xh.numel() * 4)
            e2e[name] = {"value": V / dt, "unit": "voxels/s", "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h, "ms_per_step": dt * 1e3}
        line["e2e"] = e2e["full_grid" if grouped else "learned"]
        line["full_grid"]["e2e"] = e2e["full_grid"]
    if rank == 0 and not args.no_cpu_baseline and not grouped and cid == 1:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_voxels, args.cpu_exhaustive_voxels)
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
    ap.add_argument("--voxels", type=int, default=None, help="default: the workload's size")
    ap.add_argument("--workload", type=int, default=1, choices=[1, 2, 3, 4],
                    help="1: N=400 p=20 V=200k (default); 2: grouped designs, censored; 3: p=130; 4: V=500k")
    ap.add_argument("--selector", default="hierarchical", choices=["hierarchical", "exhaustive"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-voxels", type=int, default=20_000,
                    help="CPU baseline sample, default selector (the 561-pair precompute amortised as in a full fit)")
    ap.add_argument("--cpu-exhaustive-voxels", type=int, default=5_000,
                    help="CPU baseline sample of the exhaustive selector")
    ap.add_argument("--ref-voxels", type=int, default=20_000)
    ap.add_argument("--fp64-voxels", type=int, default=2000,
                    help="voxels of the learned fit checked against the FP64 oracle (0: skip)")
    ap.add_argument("--recenter", type=int, default=1)
    ap.add_argument("--no-transfer", dest="transfer", action="store_false",
                    help="skip the proposal trained on other designs (the held-out-design check)")
    ap.add_argument("--train-voxels", type=int, default=6_000_000)
    ap.add_argument("--train-epochs", type=int, default=40)
    ap.add_argument("--proposal", default=None, help="load a trained proposal (.npz) instead of training one")
    ap.add_argument("--save-proposal", default=None, help="save the proposal trained here (.npz)")
    ap.add_argument("--dsort", type=int, default=0,
                    help="also time the full-grid fit with this many voxelwise regressors (-dsort)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-grouped-learned", dest="grouped_learned", action="store_false",
                    help="grouped workload: skip the learned-seeded arm")
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
