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
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import torch

from .. import _lib
from . import engine
from .grid import RemlGrid, RunLayout

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


def features(yr_t: torch.Tensor, layout: RunLayout) -> torch.Tensor:
    T, V = yr_t.shape
    dev = yr_t.device
    feats = torch.empty(V, N_IN, device=dev, dtype=torch.float32)
    rs = torch.from_numpy(layout.run_start).to(dev)
    engine._run("ffs_reml_features", _lib.load().ffs_reml_features, V, T, layout.n_runs, _p(rs), _p(yr_t),
                _p(feats), _st())
    return feats


def mlp_grad(params, x, y, idx, n_total, grad, loss) -> None:
    B = x.shape[0] if idx is None else idx.shape[0]
    engine._run("ffs_mlp_grad", _lib.load().ffs_mlp_grad, _p(params), _p(x), _p(y), _p(idx), B, n_total, _p(grad),
                _p(loss), _st())


def adam(params, grad, m, v, lr, step, b1=0.9, b2=0.999, eps=1e-8) -> None:
    engine._run("ffs_mlp_adam", _lib.load().ffs_mlp_adam, _p(params), _p(grad), _p(m), _p(v), params.numel(),
                float(lr), float(b1), float(b2), float(eps), int(step), _st())


def training_set(X: torch.Tensor, factors: engine.GridFactors, layout: RunLayout, n: int, seed: int,
                 chunk: int = 250_000):
    """Simulated voxels, their features and full-grid exhaustive labels (a*, b*)."""
    dev = X.device
    g = factors.grid
    a_t = torch.from_numpy(g.a).to(dev)
    b_t = torch.from_numpy(g.b).to(dev)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    feats, labels = [], []
    for c0 in range(0, n, chunk):
        m = min(chunk, n - c0)
        idx = torch.randint(0, g.P, (m,), generator=gen).to(dev)
        Y = simulate(X, layout, a_t[idx], b_t[idx], seed * 7919 + c0)
        so = engine.search(Y, factors, hierarchical=False, projector="tc" if factors.U_hi is not None else "simt",
                           keep_yr=True)
        feats.append(features(so.yr_t, layout))
        best = so.best.long()
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


def learned_search(Y: torch.Tensor, factors: engine.GridFactors, proposal: ArmaProposal, layout: RunLayout, *,
                   do_scale: bool = True, Ut: torch.Tensor | None = None) -> LearnedOut:
    """Learned-seeded REML search: 5 x 5 window around each proposal, full grid on edge hits."""
    lib = _lib.load()
    dev = Y.device
    V, T = Y.shape
    g = factors.grid
    K, P = factors.K, factors.P
    st = _st()
    Y = Y.float().contiguous()
    pre = engine.prep(Y, factors, do_scale=do_scale, tensor_core=False)
    feats = features(pre.yr_t, layout)
    prop = proposal.forward(feats)
    a_ax = torch.from_numpy(g.a_axis).to(dev)
    b_ax = torch.from_numpy(g.b_axis).to(dev)
    center = torch.empty(V, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_centers", lib.ffs_reml_centers, V, _p(prop), _p(a_ax), len(g.a_axis), _p(b_ax),
                len(g.b_axis), _p(center), st)
    ncell = len(g.a_axis) * len(g.b_axis)
    order = torch.empty(V, dtype=torch.int32, device=dev)
    work = torch.empty(ncell + 1, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_group", lib.ffs_reml_group, V, ncell, _p(center), _p(work), _p(order), st)
    if Ut is None:
        Ut = transpose_u(factors)
    best = torch.empty(V, dtype=torch.int32, device=dev)
    dbest = torch.empty(V, dtype=torch.float32, device=dev)
    crit0 = torch.empty(V, dtype=torch.float64, device=dev)
    fb = torch.empty(V, dtype=torch.int32, device=dev)
    engine._run("ffs_reml_window", lib.ffs_reml_window, V, T, K, P, g.p0, len(g.a_axis), len(g.b_axis),
                _p(factors.lattice), _p(center), _p(order), _p(pre.yr_t), _p(factors.coef), _p(Ut),
                _p(factors.logdet_R), _p(factors.logdet_XtX), _p(best), _p(dbest), _p(crit0), _p(fb), st)
    best_crit = (crit0 + dbest.double()).float()
    # full grid for the voxels whose best pair touched the window edge
    sel = torch.nonzero(fb, as_tuple=True)[0]
    if sel.numel():
        so = engine.search(Y.index_select(0, sel), factors, hierarchical=False,
                           projector="tc" if factors.U_hi is not None else "simt", do_scale=do_scale)
        best.index_copy_(0, sel, so.best)
        best_crit.index_copy_(0, sel, so.best_crit)
    return LearnedOut(best=best, best_crit=best_crit, scale=pre.scale, fallback=fb, proposal=prop)


def transpose_u(factors: engine.GridFactors) -> torch.Tensor:
    P, K, T = factors.U.shape
    Ut = torch.empty(P, T, K, device=factors.U.device, dtype=torch.float32)
    engine._run("ffs_transpose_u", _lib.load().ffs_transpose_u, P, K, T, _p(factors.U), _p(Ut), _st())
    return Ut
