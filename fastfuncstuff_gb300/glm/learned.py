"""Learned (a, b) proposal for the REML grid search: training and the seeded search.

The proposal has no counterpart in the reference; it is this build's way to
avoid evaluating all pairs. A 9 -> 64 -> 64 -> 2 GELU MLP maps each voxel's
OLS-residual autocorrelations at lags 1-8 (and T/1000) to an (a, b); the
search then evaluates only the 5 x 5 lattice window around it, and a voxel whose
best pair touches a valid lattice neighbour outside the window is searched over
the full grid. The selected pair is therefore the full grid's global argmin
whenever the criterion has no second basin outside the window -- agreement is
measured, not assumed.

Training data are simulated on the GPU (``ffs_arma_simulate``) with the fit's
own design, (a, b) drawn uniformly over the valid pairs, and labelled by the
full-grid exhaustive argmin (``engine.search``). Forward, backward and Adam are
the library's kernels (``ffs_mlp_*``); this module only sequences them.
"""

from __future__ import annotations

import ctypes as C
import io
import json
import time
import types
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import torch

from .. import _lib
from . import engine
from .grid import RemlGrid, RunLayout, lambda_is_zero

N_IN = 9


def _p(t):
    return None if t is None else t.data_ptr()


def _st():
    return torch.cuda.current_stream().cuda_stream


@dataclass
class ArmaProposal:
    """Trained proposal network (flat float32 parameters on the device)."""

    params: torch.Tensor
    meta: dict = field(default_factory=dict)

    def save(self, path) -> None:
        buf = io.BytesIO()
        np.savez_compressed(buf, params=self.params.detach().cpu().numpy(), meta=json.dumps(self.meta))
        Path(path).write_bytes(buf.getvalue())

    @classmethod
    def load(cls, path, device="cuda") -> "ArmaProposal":
        with np.load(path, allow_pickle=False) as d:
            params = torch.from_numpy(d["params"]).to(device)
            meta = json.loads(str(d["meta"]))
        n = _lib.load().ffs_mlp_param_count()
        if params.numel() != n:
            raise ValueError(f"{path}: {params.numel()} parameters, the network has {n}")
        return cls(params, meta)

    def forward(self, feats: torch.Tensor) -> torch.Tensor:
        out = torch.empty(feats.shape[0], 2, device=feats.device, dtype=torch.float32)
        engine._run("ffs_mlp_forward", _lib.load().ffs_mlp_forward, _p(self.params), _p(feats.contiguous()),
                    feats.shape[0], _p(out), _st())
        return out


def init_params(seed: int = 0, device="cuda") -> torch.Tensor:
    """He-style initial weights, zero biases (W1[64][9], b1, W2[64][64], b2, W3[2][64], b3)."""
    rng = np.random.default_rng(seed)
    parts = []
    for shape, fan_in in (((64, 9), 9), ((64,), None), ((64, 64), 64), ((64,), None), ((2, 64), 64), ((2,), None)):
        if fan_in is None:
            parts.append(np.zeros(shape).ravel())
        else:
            parts.append(rng.standard_normal(shape).ravel() * np.sqrt(2.0 / fan_in))
    return torch.from_numpy(np.concatenate(parts).astype(np.float32)).to(device)


def simulate(X: torch.Tensor, layout: RunLayout, a: torch.Tensor, b: torch.Tensor, seed: int) -> torch.Tensor:
    """(V, T) simulated voxels with ARMA(1,1) noise (a[v], b[v]) on design X."""
    dev = X.device
    T, K = X.shape
    V = a.shape[0]
    Y = torch.empty(V, T, device=dev, dtype=torch.float32)
    rs = torch.from_numpy(layout.run_start).to(dev)
    Xc = X.float().contiguous()
    engine._run("ffs_arma_simulate", _lib.load().ffs_arma_simulate, V, T, K, layout.n_runs, _p(rs), _p(Xc),
                _p(a.float().contiguous()), _p(b.float().contiguous()), int(seed) & (2**64 - 1), _p(Y), _st())
    return Y


def features(Y: torch.Tensor, factors: engine.GridFactors, layout: RunLayout, *, do_scale: bool = True) -> torch.Tensor:
    """(V, 9) proposal inputs of the voxels Y (V, T): lag 1..8 autocorrelations
    of each scaled, residualised series within runs, and T/1000 (one prep pass)."""
    return engine.prep(Y, factors, do_scale=do_scale, tensor_core=False, want_yr_t=False, layout=layout).feats


def mlp_grad(params, x, y, idx, n_total, grad, loss) -> None:
    B = x.shape[0] if idx is None else idx.shape[0]
    engine._run("ffs_mlp_grad", _lib.load().ffs_mlp_grad, _p(params), _p(x), _p(y), _p(idx), B, n_total, _p(grad),
                _p(loss), _st())


def adam(params, grad, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8) -> None:
    engine._run("ffs_mlp_adam", _lib.load().ffs_mlp_adam, _p(params), _p(grad), _p(m), _p(v), params.numel(),
                float(lr), float(b1), float(b2), float(eps), int(step), _st())


def training_set(X: torch.Tensor, factors: engine.GridFactors, layout: RunLayout, n: int, seed: int,
                 chunk: int = 250_000):
    """Simulated voxels, their features and full-grid exhaustive labels (a*, b*).

    A voxel whose argmin is an identity pair (lambda == 0: every such pair has
    the same criterion, so the whole line a = -b is its argmin) is labelled
    with (0, 0), the line's middle, rather than with the first identity pair
    the tie-break reports.
    """
    dev = X.device
    g = factors.grid
    a_t = torch.from_numpy(g.a).to(dev)
    b_t = torch.from_numpy(g.b).to(dev)
    ident = torch.from_numpy(lambda_is_zero(g.a, g.b)).to(dev)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    feats, labels = [], []
    for c0 in range(0, n, chunk):
        m = min(chunk, n - c0)
        idx = torch.randint(0, g.P, (m,), generator=gen).to(dev)
        Y = simulate(X, layout, a_t[idx], b_t[idx], seed * 7919 + c0)
        so = engine.search(Y, factors, hierarchical=False, projector="tc" if factors.U_hi is not None else "simt")
        feats.append(features(Y, factors, layout))
        best = so.best.long()
        best = torch.where(ident[best], torch.full_like(best, g.p0), best)
        labels.append(torch.stack([a_t[best], b_t[best]], 1))
    return torch.cat(feats), torch.cat(labels)


def train(x: torch.Tensor, y: torch.Tensor, *, epochs: int = 20, batch: int = 8192, lr: float = 2e-3,
          seed: int = 0, holdout: float = 0.02, params: torch.Tensor | None = None, log=None) -> tuple:
    """Adam training of the proposal on (features, labels); returns (ArmaProposal, history)."""
    dev = x.device
    n = x.shape[0]
    n_hold = int(n * holdout)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(n, generator=gen).to(dev)
    hold, tr = perm[:n_hold], perm[n_hold:]
    params = init_params(seed, dev) if params is None else params.clone()
    P = params.numel()
    grad = torch.zeros(P, device=dev)
    m = torch.zeros(P, device=dev)
    v = torch.zeros(P, device=dev)
    loss = torch.zeros(1, device=dev)
    hist = []
    step = 0
    n_tr = tr.numel()
    t0 = time.perf_counter()
    for ep in range(epochs):
        order = tr[torch.randperm(n_tr, generator=gen).to(dev)].to(torch.int32)
        loss.zero_()
        lr_ep = lr * (0.5 * (1 + np.cos(np.pi * ep / epochs)))  # cosine decay
        for s in range(0, n_tr, batch):
            bidx = order[s : s + batch]
            mlp_grad(params, x, y, bidx, bidx.numel(), grad, loss)
            step += 1
            adam(params, grad, m, v, lr_ep, step)
        tr_loss = float(loss.item()) / max(1, (n_tr + batch - 1) // batch)
        hold_loss = None
        if n_hold:
            out = ArmaProposal(params).forward(x[hold])
            hold_loss = float(((out - y[hold]) ** 2).sum(1).mean().item() / 2)
        hist.append({"epoch": ep, "train_loss": tr_loss, "holdout_loss": hold_loss})
        if log:
            log(hist[-1])
    meta = {"epochs": epochs, "batch": batch, "lr": lr, "n_train": int(n_tr), "seconds": time.perf_counter() - t0,
            "history": hist}
    return ArmaProposal(params, meta), hist


@dataclass
class LearnedOut:
    best: torch.Tensor
    best_crit: torch.Tensor
    scale: torch.Tensor
    fallback: torch.Tensor  # [V] int32, 1 where the full grid decided
    proposal: torch.Tensor  # [V, 2]
    stats: dict = field(default_factory=dict)


WIN_SLOTS = 25


_GRID_CONSTS: dict = {}


def _window_consts(f: engine.GridFactors):
    """Constants of the windowed refine: the grid's (cached by lattice content)
    and the factors' (device tensors, no host round trip)."""
    c = _grid_consts(f.grid, f.coef.device)
    fc = getattr(f, "_window_consts", None)
    if fc is None:
        g = f.grid
        c_p0 = (f.logdet_R[g.p0] + f.logdet_XtX[g.p0]).reshape(1).contiguous()
        fc = dict(c, c_p0=c_p0, dcf=((f.logdet_R + f.logdet_XtX) - c_p0).float().contiguous())
        f._window_consts = fc
    return fc


def _grid_consts(g: RemlGrid, dev):
    """The grid's constants of the windowed refine on dev (cached by lattice content)."""
    key = (g.a_axis.tobytes(), g.b_axis.tobytes(), g.lattice.tobytes(), str(dev))
    c = _GRID_CONSTS.get(key)
    if c is None:
        ident_np = lambda_is_zero(g.a, g.b)
        # non-identity pairs of the (clamped) 5 x 5 window of every lattice cell
        n_a, n_b = g.lattice.shape
        nonid = np.zeros((n_a, n_b), np.int64)
        ok = g.lattice >= 0
        nonid[ok] = (~ident_np[g.lattice[ok]]).astype(np.int64)
        a0 = np.clip(np.arange(n_a) - 2, 0, n_a - min(5, n_a))
        b0 = np.clip(np.arange(n_b) - 2, 0, n_b - min(5, n_b))
        cs = np.zeros((n_a + 1, n_b + 1), np.int64)
        cs[1:, 1:] = nonid.cumsum(0).cumsum(1)
        a1 = a0 + min(5, n_a)
        b1 = b0 + min(5, n_b)
        evals = (cs[a1][:, b1] - cs[a0][:, b1] - cs[a1][:, b0] + cs[a0][:, b0]).reshape(-1)
        c = dict(ident=torch.from_numpy(ident_np.astype(np.uint8)).to(dev), p_id=int(np.nonzero(ident_np)[0][0]),
                 a_ax=torch.from_numpy(g.a_axis).to(dev), b_ax=torch.from_numpy(g.b_axis).to(dev),
                 evals=torch.from_numpy(np.append(evals, 0)).to(dev))  # [ncell + 1]: 0 for a skipped voxel
        # lattice (Manhattan) distance of every pair to the nearest identity
        # pair, and the strip next to the identity line (distance 1)
        ia = np.searchsorted(g.a_axis, g.a)
        ib = np.searchsorted(g.b_axis, g.b)
        ida, idb = ia[ident_np], ib[ident_np]
        dist = (np.abs(ia[:, None] - ida[None, :]) + np.abs(ib[:, None] - idb[None, :])).min(1).astype(np.int32)
        c["dist_id"] = torch.from_numpy(dist).to(dev)
        strip = np.nonzero(dist == 1)[0][:STRIP_MAX]
        c["strip"] = {"n": int(strip.size), "pairs": torch.from_numpy(strip.astype(np.int64)).to(dev),
                      "pairs32": torch.from_numpy(strip.astype(np.int32)).to(dev)}
        _GRID_CONSTS[key] = c
    return c


STRIP_MAX = 64  # most pairs one ffs_reml_strip call takes
STAGE_CHUNKS = 8  # chunks of rows a staged run copies in and preps one after another
STRIP_K0 = 2  # voxels whose answer lies this close to the identity line get the strip next to it


def _band_sums_strip(pre, f, ids, count, pairs32, nq: int, V: int):
    """AFNI's banded R: y'R^-1 y of the compacted rows ids[i < *count] at the
    strip pairs, [nq][V] (ffs_reml_band_sums in strip mode); None for the
    exact R, whose recurrence the strip kernel runs itself."""
    if f.band_coef is None:
        return None
    lib = _lib.load()
    ssw = torch.empty(nq, V, dtype=torch.float32, device=pre.scale.device)
    engine._run("ffs_reml_band_sums", lib.ffs_reml_band_sums, V, _p(count), f.T, _p(ids), _p(pre.rows),
                _p(f.band_coef), f.band_w, _p(f.band), None, None, 0, None, None, 0, 0, None, _p(pairs32), nq,
                _p(ssw), _st())
    return ssw


def _strip_round_grouped(pre, f, out, *, flag, k0: int, grp: dict, pad: torch.Tensor):
    """_strip_round for grouped designs, every design in one pass: the
    near-line voxels (padding slots excluded) sorted by design
    (ffs_reml_group), their rows split to fp16 while gathered, one work-list
    projection (ffs_reml_segment_items: each design's segment against that
    design's U rows of the strip pairs) and one ffs_reml_strip launch that
    reads each row's design constants. Returns the device counts [items,
    list overflow]."""
    lib = _lib.load()
    dev = pre.scale.device
    c = _grid_consts(f.grid, dev)
    sc = c["strip"]
    if sc["n"] == 0:
        return None
    V = out["best"].numel()
    K, P, T, ld, D = f.K, f.P, f.T, f.ld, grp["D"]
    st = _st()
    nq = sc["n"]
    near = (c["dist_id"].index_select(0, out["best"].long()) <= k0) & (out["fb"] == 0) & ~pad
    keys = torch.where(near, grp["design"], torch.full_like(grp["design"], D)).contiguous()
    idx = torch.empty(V, dtype=torch.int32, device=dev)
    seg_end = torch.empty(D + 2, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_group", lib.ffs_reml_group, V, D + 1, _p(keys), _p(seg_end), _p(idx), st)
    count = seg_end[D - 1 : D]  # device count of the near-line voxels
    hi = torch.empty(V, ld, dtype=torch.int16, device=dev)
    lo = torch.empty(V, ld, dtype=torch.int16, device=dev)
    yexp = torch.empty(V, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_gather", lib.ffs_reml_gather, V, _p(count), T, ld, _p(idx), None, None, _p(pre.yexp),
                _p(pre.rows), _p(hi), _p(lo), _p(yexp), None, st)
    # the strip pairs' U rows of every design: [D][nq][K][ld]
    rows = (torch.arange(D, device=dev)[:, None] * P + sc["pairs"][None, :]).reshape(-1)
    u_hi = f.U_hi.view(D * P, K * ld).index_select(0, rows)
    u_lo = f.U_lo.view(D * P, K * ld).index_select(0, rows)
    uex = f.uexp.index_select(0, rows)
    max_pairs = min(nq, 256 // K)
    max_items = (-(-V // 128) + D) * -(-nq // max_pairs)
    items = torch.empty(max_items, 6, dtype=torch.int32, device=dev)
    counts = torch.zeros(2, dtype=torch.int32, device=dev)  # n_items, overflow
    engine._run("ffs_reml_segment_items", lib.ffs_reml_segment_items, D, _p(seg_end), nq, K, max_pairs, _p(items),
                _p(counts), max_items, counts.data_ptr() + 4, st)
    proj = torch.empty(nq, V, dtype=torch.float32, device=dev)
    pa = _lib.ProjectArgs(V=V, T=T, K=K, P=D * nq, ld_y=ld, ld_u=ld, yr_hi=_p(hi), yr_lo=_p(lo), u_hi=_p(u_hi),
                          u_lo=_p(u_lo), yexp=_p(yexp), uexp=_p(uex), yr_t=None, U=None, proj=_p(proj), flag=_p(flag))
    engine._run("ffs_reml_project_tc_list", lib.ffs_reml_project_tc_list, C.byref(pa), _p(items), _p(counts),
                max_items, max_pairs, 0, st)
    ssw = _band_sums_strip(pre, f, idx, count, sc["pairs32"], nq, V)
    engine._run("ffs_reml_strip", lib.ffs_reml_strip, V, _p(count), T, K, nq, _p(sc["pairs32"]), _p(idx),
                _p(pre.rows), _p(f.coef), _p(proj), _p(grp["dcf"]), _p(out["dbest"]), _p(out["crit0"]),
                _p(out["fb"]), _p(out["cell"]), _p(grp["design"]), P, _p(ssw), st)
    out["strip_voxels"] = count
    out.setdefault("_keep", []).append((keys, idx, seg_end, hi, lo, yexp, u_hi, u_lo, uex, items, proj, ssw))
    return counts


def _strip_round(pre, f, out, *, flag, k0: int):
    """The pairs next to the identity line (lattice distance 1) for the voxels
    whose answer lies within k0 lattice steps of it and that the full grid
    does not take anyway: there the criterion is nearly flat along the line
    and can have minima at several a, so a window holding one of them proves
    nothing about the others. The voxels are compacted on the device
    (ffs_reml_near_line), their rows split to fp16 while gathered, projected
    against the strip pairs' U rows in one tcgen05 launch (only the device
    count of rows) and evaluated by ffs_reml_strip, which sends a voxel whose
    strip pair beats its answer to the full grid."""
    lib = _lib.load()
    dev = pre.scale.device
    c = _window_consts(f)
    sc = c["strip"]
    if sc["n"] == 0:
        return
    V = out["best"].numel()
    K, P, T, ld = f.K, f.P, f.T, f.ld
    st = _st()
    ids = torch.empty(V, dtype=torch.int32, device=dev)
    count = torch.empty(1, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_near_line", lib.ffs_reml_near_line, V, _p(out["best"]), _p(c["dist_id"]), int(k0),
                _p(out["fb"]), _p(ids), _p(count), st)
    hi = torch.empty(V, ld, dtype=torch.int16, device=dev)
    lo = torch.empty(V, ld, dtype=torch.int16, device=dev)
    yexp = torch.empty(V, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_gather", lib.ffs_reml_gather, V, _p(count), T, ld, _p(ids), None, None, _p(pre.yexp),
                _p(pre.rows), _p(hi), _p(lo), _p(yexp), None, st)
    nq = sc["n"]
    u_hi = f.U_hi.view(P, K * ld).index_select(0, sc["pairs"])  # [nq][K][ld]: rows nq * K
    u_lo = f.U_lo.view(P, K * ld).index_select(0, sc["pairs"])
    uex = f.uexp.index_select(0, sc["pairs"])
    proj = torch.empty(nq, V, dtype=torch.float32, device=dev)
    pa = _lib.ProjectArgs(V=V, T=T, K=K, P=nq, ld_y=ld, ld_u=ld, yr_hi=_p(hi), yr_lo=_p(lo), u_hi=_p(u_hi),
                          u_lo=_p(u_lo), yexp=_p(yexp), uexp=_p(uex), yr_t=None, U=None, proj=_p(proj),
                          flag=_p(flag), V_dev=_p(count))
    engine._run("ffs_reml_project_tc", lib.ffs_reml_project_tc, C.byref(pa), st)
    ssw = _band_sums_strip(pre, f, ids, count, sc["pairs32"], nq, V)
    engine._run("ffs_reml_strip", lib.ffs_reml_strip, V, _p(count), T, K, nq, _p(sc["pairs32"]), _p(ids),
                _p(pre.rows), _p(f.coef), _p(proj), _p(c["dcf"]), _p(out["dbest"]), _p(out["crit0"]),
                _p(out["fb"]), _p(out["cell"]), None, 0, _p(ssw), st)
    if out.get("count_evals"):
        out["pair_evals"] = out.get("pair_evals", 0) + nq * count.sum()
    out["strip_voxels"] = count
    out.setdefault("_keep", []).append((ids, hi, lo, yexp, u_hi, u_lo, uex, proj, ssw))


def _window_round(pre, f, cen, out, *, flag, join=None, next_cen=None, grp=None):
    """Evaluate the 5 x 5 windows centred at cen (one lattice cell per voxel,
    or ncell = n_a * n_b for a voxel to skip), writing out[...] at the voxel
    ids, and into next_cen (when given) the centre of a re-centred round for
    each voxel taken (ncell: none). Nothing waits for the host: the number of
    voxels taken stays on the device. pre is the prep of every voxel (fp16
    operands and voxel-major rows). ``grp`` (grouped designs: a multi-design
    ``f``) gives each row's design and the per-design criterion constants;
    the rows are then sorted by centre and design, so every work item reads
    one design's U rows and every criterion tile one window."""
    lib = _lib.load()
    dev = pre.scale.device
    g = f.grid
    K, P, T, ld = f.K, f.P, f.T, f.ld
    st = _st()
    n_a, n_b = len(g.a_axis), len(g.b_axis)
    ncell = n_a * n_b
    n = cen.numel()
    c = _grid_consts(g, dev)
    # voxels sorted by window centre (for grouped designs by centre, then
    # design: a criterion tile spans a centre's designs, a work item one
    # design); the skipped ones (the last bucket) last
    nkey, keys, Pd = ncell, cen, 0
    if grp is not None:
        nkey, Pd = grp["D"] * ncell, P
        keys = torch.where(cen < ncell, cen * grp["D"] + grp["design"], torch.full_like(cen, nkey)).contiguous()
    idx = torch.empty(n, dtype=torch.int32, device=dev)
    cell_end = torch.empty(nkey + 2, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_group", lib.ffs_reml_group, n, nkey + 1, _p(keys), _p(cell_end), _p(idx), st)
    n_taken = cell_end[nkey - 1 : nkey]  # device count of the voxels with a window
    hi = torch.empty(n, ld, dtype=torch.int16, device=dev)
    lo = torch.empty(n, ld, dtype=torch.int16, device=dev)
    yexp = torch.empty(n, dtype=torch.int32, device=dev)
    # the tensor-core operands in window order (the window criterion reads the
    # voxel-major rows through idx)
    engine._run("ffs_reml_gather", lib.ffs_reml_gather, n, _p(n_taken), T, ld, _p(idx), _p(pre.yr_hi), _p(pre.yr_lo),
                _p(pre.yexp), _p(pre.rows), _p(hi), _p(lo), _p(yexp), None, st)
    # projections of every window pair on the tensor cores
    max_pairs = max(1, min(5, 256 // K))
    max_tiles = (n + 127) // 128 + min(n, nkey)
    max_items = WIN_SLOTS * max_tiles
    items = torch.empty(max_items, 6, dtype=torch.int32, device=dev)
    tiles = torch.empty(max_tiles, 2, dtype=torch.int32, device=dev)
    counts = torch.zeros(3, dtype=torch.int32, device=dev)  # n_items, overflow, n_tiles
    engine._run("ffs_reml_window_items", lib.ffs_reml_window_items, nkey, _p(cell_end), n_a, n_b, _p(f.lattice),
                K, max_pairs, _p(items), _p(counts), max_items, _p(tiles), counts.data_ptr() + 8, max_tiles,
                counts.data_ptr() + 4, Pd, st)
    if join is not None:  # the factors may still be in flight on another stream
        join()
    c = dict(c, dcf=grp["dcf"], c_p0=grp["c_p0"]) if grp is not None else _window_consts(f)
    winproj = torch.empty(n, WIN_SLOTS, dtype=torch.float32, device=dev)
    ja = _lib.ProjectArgs(V=n, T=T, K=K, P=P * f.n_designs, ld_y=ld, ld_u=ld, yr_hi=_p(hi), yr_lo=_p(lo),
                          u_hi=_p(f.U_hi), u_lo=_p(f.U_lo), yexp=_p(yexp), uexp=_p(f.uexp), yr_t=None, U=None,
                          proj=_p(winproj), flag=_p(flag))
    engine._run("ffs_reml_project_tc_list", lib.ffs_reml_project_tc_list, C.byref(ja), _p(items), _p(counts),
                max_items, max_pairs, WIN_SLOTS, st)
    ssw = None
    if f.band_coef is not None:
        # AFNI's banded R: y'R^-1 y of every window slot by the band's forward
        # substitution, read by the window kernel in place of its recurrence
        ssw = torch.empty(n, WIN_SLOTS, dtype=torch.float32, device=dev)
        engine._run("ffs_reml_band_sums", lib.ffs_reml_band_sums, n, None, T, _p(idx), _p(pre.rows),
                    _p(f.band_coef), f.band_w, _p(f.band), _p(tiles), counts.data_ptr() + 8, max_tiles, _p(cen),
                    _p(f.lattice), n_a, n_b, _p(c["ident"]), None, 0, _p(ssw), st)
        out.setdefault("_keep", []).append(ssw)
    engine._run("ffs_reml_window", lib.ffs_reml_window, n, T, K, n_a, n_b, _p(f.lattice), _p(idx), _p(cen),
                _p(tiles), counts.data_ptr() + 8, max_tiles, _p(pre.rows), _p(f.coef), _p(winproj), _p(c["dcf"]),
                _p(c["ident"]), c["p_id"], _p(c["c_p0"]),
                _p(out["best"]), _p(out["dbest"]), _p(out["crit0"]), _p(out["fb"]), _p(out["cell"]), _p(next_cen),
                _p(grp["design"]) if grp is not None else None, Pd, _p(ssw), st)
    if out.get("count_evals"):  # statistics only: (voxel, pair) windows evaluated
        out["pair_evals"] = out.get("pair_evals", 0) + c["evals"][cen.long()].sum()
    return counts


@dataclass
class WindowState:
    """Device results of the window rounds (nothing read back yet)."""

    best: torch.Tensor      # [V] int32 the windows' pair per voxel
    best_crit: torch.Tensor  # [V] float32
    scale: torch.Tensor     # [V] float32
    fb: torch.Tensor        # [V] int32 1: the full grid must decide
    proposal: torch.Tensor  # [V, 2]
    small: torch.Tensor     # int32 [fallback count, wait flag, list overflows...]
    stats: dict


def learned_prep(Y: torch.Tensor, factors: engine.GridFactors, layout: RunLayout, *, do_scale: bool = True,
                 q0: torch.Tensor | None = None, y_ref: torch.Tensor | None = None,
                 out: engine.PrepOut | None = None) -> engine.PrepOut:
    """The prep of the learned-seeded search: each voxel's scale, its
    residualised rows (voxel-major), the exponents of their fp16 split and
    the proposal's features (into ``out``'s buffers when given)."""
    return engine.prep(Y, factors, do_scale=do_scale, tensor_core=True, want_yr_t=False, layout=layout,
                       want_rows=True, q0=q0, split=False, y_ref=y_ref, y_copy=Y if y_ref is not None else None,
                       out=out)


def learned_windows(Y: torch.Tensor, factors: engine.GridFactors, proposal: ArmaProposal, layout: RunLayout, *,
                    do_scale: bool = True, recenter: int = 0, q0: torch.Tensor | None = None,
                    join=None, strip_k0: int = STRIP_K0, y_ref: torch.Tensor | None = None,
                    count_evals: bool = False, pre: engine.PrepOut | None = None) -> WindowState:
    """The window rounds of the learned-seeded search, with no host round trip
    (so they also run inside a CUDA graph): prep with the proposal features,
    the MLP, the 5 x 5 window of every voxel, ``recenter`` re-centred rounds
    for the voxels on a window edge, then the strip next to the identity line
    for the voxels whose answer lies within ``strip_k0`` lattice steps of it
    (-1: none); a voxel that a strip pair beats takes the full grid. With
    ``q0`` (engine.design_basis) the prep does not read the factors;
    ``join()`` is then called before their first use (they may be built on
    another stream meanwhile). With ``y_ref`` (engine.prep) the rows are read
    from the address it holds and written into Y as read. ``count_evals``
    adds the number of (voxel, pair) criteria evaluated to the statistics.
    ``pre`` (learned_prep of every voxel) skips the prep; Y then only gives
    the shape."""
    lib = _lib.load()
    dev = Y.device
    V, T = Y.shape
    f = factors
    if f.U_hi is None:
        raise ValueError("the learned search needs the tensor-core operands of the factors")
    g = f.grid
    st = _st()
    c = _grid_consts(g, dev)
    # the windows' rows are split to fp16 while they are gathered (from rows)
    p1 = pre
    if p1 is None:
        if y_ref is None:
            Y = Y.float().contiguous()
        p1 = learned_prep(Y, f, layout, do_scale=do_scale, q0=q0, y_ref=y_ref)
    scale = p1.scale
    prop = proposal.forward(p1.feats)
    center = torch.empty(V, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_centers", lib.ffs_reml_centers, V, _p(prop), _p(c["a_ax"]), len(g.a_axis), _p(c["b_ax"]),
                len(g.b_axis), _p(center), st)
    out = dict(best=torch.empty(V, dtype=torch.int32, device=dev), dbest=torch.empty(V, dtype=torch.float32, device=dev),
               crit0=torch.empty(V, dtype=torch.float64, device=dev), fb=torch.zeros(V, dtype=torch.int32, device=dev),
               cell=torch.empty(V, dtype=torch.int32, device=dev), count_evals=count_evals)
    if not 0 <= recenter <= 6:
        raise ValueError("recenter: 0 to 6 re-centred rounds")
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    # each round writes the next one's centres: the voxels on a window edge
    # are re-centred on the window's best pair, the rest skipped (ncell)
    nxt = [torch.empty(V, dtype=torch.int32, device=dev) for _ in range(min(recenter, 2))]
    counts = [_window_round(p1, f, center, out, flag=flag, join=join, next_cen=nxt[0] if recenter else None)]
    # the share of voxels on the first window's edge: statistics only
    stats = {"edge_first": (out["fb"].float().mean() if count_evals else float("nan")) if recenter else None}
    ncell = len(g.a_axis) * len(g.b_axis)
    for r in range(recenter):
        cen = nxt[r % 2]
        after = None
        if r + 1 < recenter:  # a round writes only the voxels it takes
            after = nxt[(r + 1) % 2]
            after.fill_(ncell)
        counts.append(_window_round(p1, f, cen, out, flag=flag, next_cen=after))
    if strip_k0 >= 0:  # on the last round's answers
        _strip_round(p1, f, out, flag=flag, k0=strip_k0)
    stats["strip_voxels"] = out.get("strip_voxels")
    fb = out["fb"]
    # best_crit, and the numbers the host reads back: [fallback count, wait
    # flag, each round's list overflow]
    best_crit = torch.empty(V, dtype=torch.float32, device=dev)
    small = torch.empty(2 + len(counts), dtype=torch.int32, device=dev)
    extra = (C.c_void_p * (1 + len(counts)))(flag.data_ptr(), *[cn.data_ptr() + 4 for cn in counts])
    engine._run("ffs_reml_window_finish", lib.ffs_reml_window_finish, V, _p(out["crit0"]), _p(out["dbest"]),
                _p(fb), _p(best_crit), _p(small), len(extra), extra, st)
    stats["pair_evals"] = out.get("pair_evals")  # device scalar (with count_evals): (voxel, pair) windows evaluated
    return WindowState(best=out["best"], best_crit=best_crit, scale=scale, fb=fb, proposal=prop, small=small,
                       stats=stats)


def learned_fallback(Y: torch.Tensor, factors: engine.GridFactors, ws: WindowState, small_host: torch.Tensor, *,
                     do_scale: bool = True) -> LearnedOut:
    """The full grid for the voxels the windows left undecided; small_host is
    ws.small read back to the host."""
    dev = Y.device
    V = Y.shape[0]
    n_fb, code = int(small_host[0]), int(small_host[1])
    if code != 0:
        raise RuntimeError(f"ffs_reml_project_tc_list: a bounded wait expired (code {code})")
    if bool((small_host[2:] != 0).any()):
        raise RuntimeError("ffs_reml_window_items: work list overflow")
    fb = ws.fb
    # the fallback voxels' ids in order, compacted on the device
    pos = torch.where(fb != 0, torch.cumsum(fb, 0) - 1, torch.full_like(fb, n_fb)).long()
    sel = torch.empty(n_fb + 1, dtype=torch.long, device=dev).scatter_(0, pos, torch.arange(V, device=dev))[:n_fb]
    stats = dict(ws.stats)
    if stats["edge_first"] is None:
        stats["edge_first"] = n_fb / V
    stats["fallback"] = n_fb / V
    best, best_crit = ws.best, ws.best_crit
    if n_fb:
        so = engine.search(Y.index_select(0, sel), factors, hierarchical=False, projector="tc", do_scale=do_scale)
        best = best.index_copy(0, sel, so.best)
        best_crit = best_crit.index_copy(0, sel, so.best_crit)
    lo = LearnedOut(best=best, best_crit=best_crit, scale=ws.scale, fallback=fb, proposal=ws.proposal, stats=stats)
    lo.fallback_idx = sel
    return lo


def learned_search(Y: torch.Tensor, factors: engine.GridFactors, proposal: ArmaProposal, layout: RunLayout, *,
                   do_scale: bool = True, recenter: int = 0, before_fallback=None, q0=None,
                   join=None, strip_k0: int = STRIP_K0, count_evals: bool = False) -> LearnedOut:
    """Learned-seeded REML search: the 5 x 5 window around each proposal, the
    full grid for voxels whose best pair sits on the window edge (or whose
    window, holding no identity pair, has nothing below the identity pairs'
    criterion), and for voxels near the identity line whose answer a pair of
    the strip next to that line beats (``strip_k0``, see ``learned_windows``).

    ``recenter`` > 0 first re-evaluates such voxels that many times with the
    window centred on their best pair; the full grid then takes those still on
    an edge. ``before_fallback(best, scale)`` is called (with the windows'
    answer for every voxel) before the one host round trip that lists the
    fallback voxels, so work it enqueues keeps the GPU busy meanwhile;
    ``LearnedOut.fallback_idx`` lists the voxels whose pair changed after it.
    """
    Y = Y.float().contiguous()
    ws = learned_windows(Y, factors, proposal, layout, do_scale=do_scale, recenter=recenter, q0=q0, join=join,
                         strip_k0=strip_k0, count_evals=count_evals)
    # copy the few numbers the host needs to pinned memory behind an event,
    # queue the caller's work, and wait for that event only
    host = torch.empty(ws.small.numel(), dtype=torch.int32, pin_memory=True)
    host.copy_(ws.small, non_blocking=True)
    ready = torch.cuda.Event()
    ready.record()
    if before_fallback is not None:
        before_fallback(ws.best.clone(), ws.scale)
    ready.synchronize()
    return learned_fallback(Y, factors, ws, host, do_scale=do_scale)


def grouped_learned_fit(Y: torch.Tensor, factors: engine.GridFactors, design: np.ndarray, Xs: torch.Tensor,
                        proposal: ArmaProposal, layout: RunLayout, *, do_scale: bool = True, recenter: int = 0,
                        gls_kw: dict | None = None, lj=None, slots: engine.DesignSlots | None = None,
                        strip_k0: int = STRIP_K0):
    """The learned-seeded fit of a grouped fit (one design per voxel group),
    every design in one pass per stage: ``factors`` is the multi-design build
    of Xs (D, T, K) and ``design`` [V] (host) each voxel's design. The voxels
    sit in the design slots of the grouped search (engine.design_slots: each
    design's voxels padded to whole tiles), the prep residualises each tile
    against its design's basis and forms the proposal's features, and the
    window rounds sort the rows by window centre and design: every work item
    reads one design's U rows, every criterion tile holds one window's rows
    of any design, each row with its design's criterion constants. The
    strip next to the identity line (``strip_k0``, -1: off) evaluates each
    near-line voxel against its design's strip pairs, all designs in one
    pass. The
    voxels a window leaves undecided take the grouped full-grid search; the
    GLS refits every voxel against its own design. ``slots``: the design
    slots of ``design`` when the caller has them.
    Returns (best, best_crit, scale, GlsOut, voxels the full grid decided)."""
    lib = _lib.load()
    dev = Y.device
    Y = Y.float().contiguous()
    V, T = Y.shape
    f = factors
    g = f.grid
    D, P, K, ld = f.n_designs, f.P, f.K, f.ld
    st = _st()
    if slots is None:
        slots = engine.design_slots(np.asarray(design).reshape(-1), D, K, P, dev)
    Vp = slots.Vp
    n_a, n_b = len(g.a_axis), len(g.b_axis)
    ncell = n_a * n_b
    c = _grid_consts(g, dev)
    # the prep of every slot (zero rows in the padding) against its design's
    # basis, U of (0, 0) per design
    q0 = f.U.view(D, P, K, -1)[:, g.p0].contiguous()
    pre = engine.PrepOut(scale=torch.empty(V, dtype=torch.float32, device=dev), yr_t=None, yr_hi=None, yr_lo=None,
                         yexp=torch.empty(Vp, dtype=torch.int32, device=dev))
    pre.feats = torch.empty(Vp, 9, dtype=torch.float32, device=dev)
    pre.rows = torch.empty(Vp, T, dtype=torch.float32, device=dev)
    rs = engine.const_dev(layout.run_start, dev)
    pa = _lib.PrepArgs(V=Vp, T=T, K=K, Y=_p(Y), Q0=_p(q0), do_scale=int(do_scale), center=0, ld_y=ld,
                       scale=_p(pre.scale), yr_t=None, yr_hi=None, yr_lo=None, yexp=_p(pre.yexp),
                       idx=_p(slots.idx), feats=_p(pre.feats), n_runs=layout.n_runs, run_start=_p(rs),
                       yr_rows=_p(pre.rows), center_dev=_p(f.center_flag), tile_design=_p(slots.tile32))
    engine._run("ffs_reml_prep", lib.ffs_reml_prep, C.byref(pa), st)
    prop = proposal.forward(pre.feats)
    center = torch.empty(Vp, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_centers", lib.ffs_reml_centers, Vp, _p(prop), _p(c["a_ax"]), n_a, _p(c["b_ax"]), n_b,
                _p(center), st)
    center = torch.where(slots.idx >= 0, center, torch.full_like(center, ncell))  # the padding takes no window
    # each slot's design and the criterion constants of every design
    dslot = slots.tile32.repeat_interleave(32).contiguous()
    ldx = f.logdet_XtX.view(D, P)
    c_p0 = (f.logdet_R[g.p0] + ldx[:, g.p0]).contiguous()
    dcf = ((f.logdet_R[None, :] + ldx) - c_p0[:, None]).float().reshape(-1).contiguous()
    grp = {"design": dslot, "D": D, "dcf": dcf, "c_p0": c_p0}
    out = dict(best=torch.zeros(Vp, dtype=torch.int32, device=dev),  # a valid pair in the padding slots too
               dbest=torch.empty(Vp, dtype=torch.float32, device=dev),
               crit0=torch.empty(Vp, dtype=torch.float64, device=dev), fb=torch.zeros(Vp, dtype=torch.int32, device=dev),
               cell=torch.empty(Vp, dtype=torch.int32, device=dev))
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    # the next round's centres: a round writes those of the rows it takes, so
    # the padding slots (never taken) keep "no window"
    nxt = [torch.full((Vp,), ncell, dtype=torch.int32, device=dev) for _ in range(min(recenter, 2))]
    counts = [_window_round(pre, f, center, out, flag=flag, next_cen=nxt[0] if recenter else None, grp=grp)]
    for r in range(recenter):
        after = None
        if r + 1 < recenter:
            after = nxt[(r + 1) % 2]
            after.fill_(ncell)
        counts.append(_window_round(pre, f, nxt[r % 2], out, flag=flag, next_cen=after, grp=grp))
    if strip_k0 >= 0:  # the strip next to the identity line
        sc_counts = _strip_round_grouped(pre, f, out, flag=flag, k0=strip_k0, grp=grp, pad=slots.idx < 0)
        if sc_counts is not None:
            counts.append(sc_counts)
    best_crit = torch.empty(Vp, dtype=torch.float32, device=dev)
    small = torch.empty(2 + len(counts), dtype=torch.int32, device=dev)
    extra = (C.c_void_p * (1 + len(counts)))(flag.data_ptr(), *[cn.data_ptr() + 4 for cn in counts])
    engine._run("ffs_reml_window_finish", lib.ffs_reml_window_finish, Vp, _p(out["crit0"]), _p(out["dbest"]),
                _p(out["fb"]), _p(best_crit), _p(small), len(extra), extra, st)
    host = small.cpu()
    if int(host[1]) != 0:
        raise RuntimeError(f"ffs_reml_project_tc_list: a bounded wait expired (code {int(host[1])})")
    if bool((host[2:] != 0).any()):
        raise RuntimeError("a projection work list of the window rounds or the strip overflowed")
    # back to voxel order; the undecided voxels through the grouped full grid
    best = out["best"].index_select(0, slots.real)
    crit = best_crit.index_select(0, slots.real)
    fbv = out["fb"].index_select(0, slots.real)
    n_fb = int(host[0])
    if n_fb:
        sel = torch.nonzero(fbv).reshape(-1)
        gid_sub = np.asarray(design).reshape(-1)[sel.cpu().numpy()]
        sub = engine.design_slots(gid_sub, D, K, P, dev)
        so = engine.search_designs(Y.index_select(0, sel), f, sub, hierarchical=False, do_scale=do_scale)
        best.index_copy_(0, sel, so.best)
        crit.index_copy_(0, sel, so.best_crit)
    go = engine.gls(Y, pre.scale, best, f, Xs, lj=lj, design=slots.design, **(gls_kw or {}))
    return best, crit, pre.scale, go, float(n_fb)


def train_proposal(X: torch.Tensor, layout: RunLayout, a_grid, b_grid, *, n_voxels: int = 6_000_000,
                   epochs: int = 40, batch: int = 8192, lr: float = 3e-3, seed: int = 5):
    """Train a proposal on the GPU: n_voxels simulated with (a, b) drawn
    uniformly over the valid pairs, labelled by the full-grid exhaustive
    argmin, then Adam on the library's forward/backward kernels. X is one
    design (T, K), or a family of designs (D, T, K) of one run layout that
    share the voxels equally (a proposal for designs it was not trained on).
    Returns (ArmaProposal, info) with the seconds spent."""
    from .grid import make_grid

    t0 = time.perf_counter()
    grid = make_grid(a_grid, b_grid)
    Xs = X if X.ndim == 3 else X[None]
    D = Xs.shape[0]
    parts = []
    for d in range(D):
        n_d = n_voxels // D + (1 if d < n_voxels % D else 0)
        f = engine.build_factors(Xs[d], grid, layout)
        parts.append(training_set(Xs[d], f, layout, n_d, seed=seed + 7 * d))
    x = torch.cat([p[0] for p in parts]) if D > 1 else parts[0][0]
    y = torch.cat([p[1] for p in parts]) if D > 1 else parts[0][1]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    prop, hist = train(x, y, epochs=epochs, batch=batch, lr=lr, seed=seed)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    info = {"train_voxels": n_voxels, "epochs": epochs, "train_designs": D, "label_s": t1 - t0,
            "train_s": t2 - t1, "holdout_loss": hist[-1]["holdout_loss"]}
    prop.meta.update(info)
    return prop, info


class LearnedFitGraph:
    """The learned-seeded fit of one shape: two CUDA graphs and one GLS.

    Graph A builds the grid factors of X on a side stream while the prep with
    the proposal features (against the design basis of X), the MLP and the
    first window round's grouping and gathers run on the main one; the window
    rounds then join them. It ends by copying the few numbers the host needs
    (fallback count, wait flag, list overflows) to pinned memory. ``run``
    replays A, records an event, launches the GLS of every voxel at its
    window pair (into new output tensors: device memory, or pinned host
    memory written over the host link), waits for the event only (the GLS
    keeps the GPU busy meanwhile), then runs the full grid and the GLS of the
    fallback voxels from graph C beside it and merges their rows into the
    outputs. The data are read where they lie (device memory, or pinned host
    memory streamed by the prep) through an address that each run writes on
    the device; the design is copied into a static buffer.
    """

    def __init__(self, Y: torch.Tensor, X: torch.Tensor, grid: RemlGrid, layout: RunLayout,
                 proposal: ArmaProposal, *, recenter: int, do_scale: bool, gls_kw: dict, factor_kw: dict,
                 staged: bool = False):
        dev = X.device
        # the data's static buffer: the prep reads each run's rows from the
        # address in y_ref (device memory, or pinned host memory read in place)
        # and writes them here for the later stages
        self.Y = torch.empty(tuple(Y.shape), dtype=torch.float32, device=dev)
        # staged: the data are copied in by the copy engine in chunks (see
        # run); else rows are read in place when 16-byte rows allow it
        # (T % 4 == 0), otherwise each run copies the data into the static
        # buffer first
        self.staged = staged
        self.inplace = not staged and Y.shape[1] % 4 == 0
        self.y_ref = torch.zeros(1, dtype=torch.int64, device=dev)
        self.y_ref_host = torch.zeros(1, dtype=torch.int64, pin_memory=True)
        self.X = X.float().contiguous().clone()
        self.grid, self.layout, self.proposal = grid, layout, proposal
        self.recenter, self.do_scale, self.gls_kw, self.factor_kw = recenter, do_scale, gls_kw, factor_kw
        self.cflag, self.ccoef = engine.constant_flag(self.X)
        self.host = torch.empty(3 + recenter, dtype=torch.int32, pin_memory=True)
        self.side = torch.cuda.Stream(dev)  # the grid build runs beside the prep chain
        self.side_fb = torch.cuda.Stream(self.Y.device)  # the fallback runs beside the window pairs' GLS
        self._fb_graphs: dict = {}
        if staged:
            self._init_staged(Y)
            return
        self._set_source(Y)
        # one eager pass fills the host-side caches (device constants, tensor
        # maps, kernel attributes) that a capture must not create
        self._body_a()
        torch.cuda.synchronize()
        self.ga = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.ga, capture_error_mode="thread_local"):
            self._body_a()

    def _init_staged(self, Y: torch.Tensor) -> None:
        """Graphs of a staged run: A0 (the design basis and the grid build),
        one prep graph per chunk of rows, and A1 (the MLP, the window rounds
        and the strip), with the prep's outputs in static buffers."""
        dev = self.Y.device
        V, T = self.Y.shape
        step = -(-V // STAGE_CHUNKS)
        step = -(-step // 32) * 32  # whole 32-voxel tiles of the prep
        self.bounds = [(c0, min(V, c0 + step)) for c0 in range(0, V, step)]
        self.copied = [torch.cuda.Event() for _ in self.bounds]
        self.copy_stream = torch.cuda.Stream(dev)
        self.prep_stream = torch.cuda.Stream(dev)
        self.pre = engine.PrepOut(scale=torch.empty(V, dtype=torch.float32, device=dev), yr_t=None, yr_hi=None,
                                  yr_lo=None, yexp=torch.empty(V, dtype=torch.int32, device=dev))
        self.pre.feats = torch.empty(V, 9, dtype=torch.float32, device=dev)
        self.pre.rows = torch.empty(V, T, dtype=torch.float32, device=dev)
        self.Y.copy_(Y)
        self._body_a0()
        for i in range(len(self.bounds)):
            self._body_prep(i)
        self._body_a1()
        torch.cuda.synchronize()
        self.ga0 = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.ga0, capture_error_mode="thread_local"):
            self._body_a0()
        self.gp = []
        for i in range(len(self.bounds)):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, capture_error_mode="thread_local"):
                self._body_prep(i)
            self.gp.append(g)
        self.ga1 = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.ga1, capture_error_mode="thread_local"):
            self._body_a1()

    def _body_a0(self):
        self.q0 = None
        center = (self.cflag, self.ccoef)
        if self.X.shape[1] <= engine.BASIS_MAX_K:
            self.q0, cflag, ccoef = engine.design_basis(self.X, with_constant=True)
            center = (cflag, ccoef)
        self.f = engine.build_factors(self.X, self.grid, self.layout, center=center, **self.factor_kw)

    def _body_prep(self, i: int):
        c0, c1 = self.bounds[i]
        pr = self.pre
        view = engine.PrepOut(scale=pr.scale[c0:c1], yr_t=None, yr_hi=None, yr_lo=None, yexp=pr.yexp[c0:c1])
        view.feats, view.rows = pr.feats[c0:c1], pr.rows[c0:c1]
        learned_prep(self.Y[c0:c1], self.f, self.layout, do_scale=self.do_scale, q0=self.q0, out=view)

    def _body_a1(self):
        self.ws = learned_windows(self.Y, self.f, self.proposal, self.layout, do_scale=self.do_scale,
                                  recenter=self.recenter, q0=self.q0, pre=self.pre)
        self.host.copy_(self.ws.small, non_blocking=True)

    def _replay_staged(self, Y: torch.Tensor) -> None:
        """The copy engine brings Y in by chunks while graph A0 builds the
        grid factors; each chunk's prep runs once both its rows and the
        factors are there; graph A1 follows the last of them."""
        if tuple(Y.shape) != tuple(self.Y.shape) or Y.dtype != torch.float32 or not Y.is_contiguous():
            raise ValueError("the learned fit's graph reads float32 contiguous data of its own shape")
        main = torch.cuda.current_stream()
        start = torch.cuda.Event()
        start.record(main)  # the previous run's readers of the static buffers are behind it
        cs, ps = self.copy_stream, self.prep_stream
        cs.wait_event(start)
        with torch.cuda.stream(cs):
            for (c0, c1), ev in zip(self.bounds, self.copied):
                self.Y[c0:c1].copy_(Y[c0:c1], non_blocking=True)
                ev.record(cs)
        self._src = Y  # kept alive until the copies have read it
        self.ga0.replay()
        built = torch.cuda.Event()
        built.record(main)
        ps.wait_event(built)
        with torch.cuda.stream(ps):
            for g, ev in zip(self.gp, self.copied):
                ps.wait_event(ev)
                g.replay()
        main.wait_stream(ps)
        self.ga1.replay()

    def _body_a(self):
        main = torch.cuda.current_stream()
        overlap = self.X.shape[1] <= engine.BASIS_MAX_K
        q0 = join = None
        center = (self.cflag, self.ccoef)
        if overlap:
            # the design basis and the centring test first (one kernel), then
            # the grid build on the side stream beside the prep chain
            q0, cflag, ccoef = engine.design_basis(self.X, with_constant=True)
            center = (cflag, ccoef)
        self.f = engine.build_factors(self.X, self.grid, self.layout, center=center,
                                      stream=self.side if overlap else None, **self.factor_kw)
        if overlap:
            built = torch.cuda.Event()
            built.record(self.side)

            def join():
                main.wait_event(built)
        self.ws = learned_windows(self.Y, self.f, self.proposal, self.layout, do_scale=self.do_scale,
                                  recenter=self.recenter, q0=q0, join=join,
                                  y_ref=self.y_ref if self.inplace else None)
        self.host.copy_(self.ws.small, non_blocking=True)

    def _set_source(self, Y: torch.Tensor) -> None:
        """Point y_ref at Y's rows (float32, contiguous, 16-byte aligned device
        memory; host data take a staged plan)."""
        if tuple(Y.shape) != tuple(self.Y.shape) or Y.dtype != torch.float32 or not Y.is_contiguous():
            raise ValueError("the learned fit's graph reads float32 contiguous data of its own shape")
        if not self.inplace:
            self.Y.copy_(Y, non_blocking=True)
            self._src = Y
            return
        if not Y.is_cuda or Y.data_ptr() % 16:
            raise ValueError("this plan reads 16-byte aligned device memory in place; host data take a staged plan")
        addr = Y.data_ptr()
        self.y_ref_host[0] = addr
        self.y_ref.copy_(self.y_ref_host, non_blocking=True)
        self._src = Y  # kept alive until the run that reads it has finished

    def run(self, Y: torch.Tensor, X: torch.Tensor, *, host_out: bool = False):
        """(LearnedOut, engine.GlsOut) of data Y (V, T) and design X (T, K).
        Y is a CUDA tensor (the prep reads its rows in place) or, for a staged
        plan, a pinned host tensor (copied in by chunks beside the grid build,
        each chunk's prep as soon as its rows are there). With
        ``host_out`` the GLS outputs are pinned host tensors written by the
        kernels over the host link while they run (read them after a
        synchronisation of the current stream)."""
        main = torch.cuda.current_stream()
        if not self.staged:
            self._set_source(Y)
        self.X.copy_(X)
        if self.X.shape[1] > engine.BASIS_MAX_K:  # else graph A runs the centring test
            flag, coef = engine.constant_flag(self.X)
            self.cflag.copy_(flag)
            self.ccoef.copy_(coef)
        if self.staged:
            self._replay_staged(Y)
        else:
            self.ga.replay()
        ready = torch.cuda.Event()
        ready.record()
        # the GLS of every voxel at its window pair, launched while graph A
        # runs (its outputs are new tensors of this call)
        go = engine.gls(self.Y, self.ws.scale, self.ws.best, self.f, self.X, host_out=host_out, **self.gls_kw)
        ready.synchronize()
        n_fb, code = int(self.host[0]), int(self.host[1])
        if code != 0:
            raise RuntimeError(f"ffs_reml_project_tc_list: a bounded wait expired (code {code})")
        if bool((self.host[2:] != 0).any()):
            raise RuntimeError("ffs_reml_window_items: work list overflow")
        # the fallback voxels' full grid and GLS: graph C (of a padded voxel
        # count) on a second stream, beside the window pairs' GLS (both only read
        # the graphs' buffers)
        fs = self.side_fb
        fc = self._fallback_graph(n_fb) if n_fb else None
        if fc is not None:
            fs.wait_event(ready)
            with torch.cuda.stream(fs):
                fc.graph.replay()
            done = torch.cuda.Event()
            done.record(fs)
        V = self.Y.shape[0]
        stats = dict(self.ws.stats)
        if stats["edge_first"] is None:
            stats["edge_first"] = n_fb / V
        stats["fallback"] = n_fb / V
        if fc is not None:
            main.wait_event(done)
        # graph A's buffers are overwritten by the next run: its answers are
        # copied into new tensors, with the full grid's rows for the fallback
        # voxels, and those rows replace the window answers' rows of the GLS
        # outputs; one merge launch for all of them
        ws = self.ws
        keep = [(ws.best, fc.so.best if fc else None), (ws.best_crit, fc.so.best_crit if fc else None),
                (ws.scale, None), (ws.fb, None), (ws.proposal, None)]
        outs = [torch.empty_like(src) for src, _ in keep]
        fields = [(dst.data_ptr(), src.data_ptr(), _p(sub), src[0].numel() * src.element_size())
                  for dst, (src, sub) in zip(outs, keep)]
        if fc is not None:
            for k, v in vars(go).items():
                if not k.startswith("_") and v is not None:
                    fields.append((engine.device_view(v), None, getattr(fc.gs, k).data_ptr(),
                                   v[0].numel() * v.element_size()))
        arr = (_lib.MergeField * len(fields))(*[_lib.MergeField(*f) for f in fields])
        lib = _lib.load()
        engine._run("ffs_merge_rows", lib.ffs_merge_rows, V, _p(fc.pos) if fc else None, len(fields), arr, _st())
        lo = LearnedOut(best=outs[0], best_crit=outs[1], scale=outs[2], fallback=outs[3], proposal=outs[4],
                        stats=stats)
        # the fallback voxels, in no particular order
        lo.fallback_idx = (fc.ids[:n_fb].long() if fc else
                           torch.empty(0, dtype=torch.long, device=self.Y.device))
        return lo, go

    def _fallback_graph(self, n_fb: int):
        """Graph C: the full-grid search and GLS of up to n_pad >= n_fb
        fallback voxels (their ids compacted on the device from the window
        rounds' flags; rows past the real count repeat voxel 0 and are
        ignored), captured once per padded count (a multiple of 256)."""
        n_pad = (n_fb + 255) // 256 * 256
        fc = self._fb_graphs.get(n_pad)
        if fc is not None:
            return fc
        while len(self._fb_graphs) >= 3:
            self._fb_graphs.pop(next(iter(self._fb_graphs)))
        dev = self.Y.device
        V = self.Y.shape[0]
        fc = types.SimpleNamespace(ids=torch.empty(n_pad, dtype=torch.int32, device=dev),
                                   pos=torch.empty(V, dtype=torch.int32, device=dev),
                                   count=torch.empty(1, dtype=torch.int32, device=dev))
        lib = _lib.load()

        def body():
            # the fallback voxels' ids (slots past their count hold voxel 0)
            # and each voxel's slot, for the merge of the outputs
            engine._run("ffs_reml_compact", lib.ffs_reml_compact, V, _p(self.ws.fb), n_pad, _p(fc.ids),
                        _p(fc.pos), _p(fc.count), _st())
            Yf = self.Y.index_select(0, fc.ids)
            fc.so = engine.search(Yf, self.f, hierarchical=False, projector="tc", do_scale=self.do_scale)
            fc.gs = engine.gls(Yf, fc.so.scale, fc.so.best, self.f, self.X, **self.gls_kw)

        with torch.cuda.stream(self.side_fb):
            body()  # fills the host-side caches a capture must not create
        self.side_fb.synchronize()
        fc.graph = torch.cuda.CUDAGraph()
        # its own memory pool: graph C runs concurrently with the window pairs' GLS
        with torch.cuda.graph(fc.graph, capture_error_mode="thread_local"):
            body()
        self._fb_graphs[n_pad] = fc
        return fc


_GRAPHS: dict = {}


def graph_for(Y, X, grid, layout, proposal, *, recenter, do_scale, gls_kw, factor_kw) -> LearnedFitGraph:
    """The cached LearnedFitGraph of this shape and these options (built on
    first use); host data (pinned memory) get a staged plan."""
    fk = tuple((k, None if v is None else v.key() if hasattr(v, "key") else np.asarray(v).tobytes())
               for k, v in sorted(factor_kw.items()))
    key = (tuple(Y.shape), tuple(X.shape), str(X.device), grid.a.tobytes(), grid.b.tobytes(), grid.lambda_fp32,
           grid.ltop, None if grid.band is None else grid.band.tobytes(),
           layout.run_start.tobytes(), layout.tau.tobytes(), id(proposal.params), proposal.params._version,
           recenter, do_scale, tuple(sorted(gls_kw.items())), fk, not Y.is_cuda)
    gr = _GRAPHS.get(key)
    if gr is None:
        while len(_GRAPHS) >= 2:  # a plan holds a few GB of static buffers
            _GRAPHS.pop(next(iter(_GRAPHS)))
        gr = LearnedFitGraph(Y, X, grid, layout, proposal, recenter=recenter, do_scale=do_scale, gls_kw=gls_kw,
                             factor_kw=factor_kw, staged=not Y.is_cuda)
        _GRAPHS[key] = gr
    return gr
