"""The reference's default CPU fit restated with torch CPU kernels -- timed CPU baseline only.

This is the CPU baseline that ``bench.py`` times (``cpu_baseline`` and
``--impl reference``): the reference's own CPU algorithm for the float32 default
fit (fastfuncstuff/glm/arma.py:3650-5878 on ``device=cpu``), written with the
same batched torch CPU linear algebra the reference uses, so that its cost on the
host cores is the reference's cost:

  1. per-voxel std scaling (arma.py:3952-3954);
  2. batched dense correlation + Cholesky + L^-1 for the longest run, leading
     blocks serving the other runs (whiten.py:197-271), X_w, Cholesky of
     X_w'X_w, Q and the logdets (arma.py:1459-1506);
  3. the hierarchical descent with one subset GEMM per visited pair
     (arma.py:2021-2221), or the exhaustive loop (arma.py:1973-2010);
  4. the GLS refit per chosen pair: betas, float64 sigma2 accumulation, t,
     F, R^2 and lambda, unscaled (arma.py:4829-5560, :5827-5862).

It is test infrastructure: the product path never imports it.
``tests/test_cpu_port.py`` pins its selections and GLS outputs to the
reference's own float32 outputs on the golden fixtures, in both selector
modes.
"""

from __future__ import annotations

import numpy as np
import torch


def _grid(a_grid, b_grid):
    a = torch.as_tensor(np.asarray(a_grid), dtype=torch.float32)
    b = torch.as_tensor(np.asarray(b_grid), dtype=torch.float32)

    def zero(g):
        near = g.abs() < 1e-6
        if bool(near.any()):
            g = g.clone()
            g[near] = 0.0
            return g
        return torch.sort(torch.cat([torch.zeros(1), g]))[0]

    a, b = zero(a), zero(b)
    am, bm = torch.meshgrid(a, b, indexing="ij")
    a, b = am.reshape(-1), bm.reshape(-1)
    ok = (a.abs() < 1) & (b.abs() < 1)
    den = 1 - a**2
    ok &= den.abs() >= 1e-6
    ok &= (1 + b**2 + 2 * a * b) / (den + 1e-10) > 0
    lam = (a + b) * (1 + a * b) / (1 + b**2 + 2 * a * b)
    ok &= lam >= 0
    return a[ok], b[ok], lam[ok]


def _factors(X: torch.Tensor, a, lam, lens):
    """Dense L^-1 of the longest run per pair and the design factors (float32)."""
    m = max(lens)
    lag = (torch.arange(m)[:, None] - torch.arange(m)[None, :]).abs()
    k = torch.arange(m, dtype=torch.float32)
    corr = lam[:, None] * a[:, None] ** (k[None, :] - 1).clamp(min=0)
    corr[:, 0] = 1.0
    R = corr[:, lag]
    L = torch.linalg.cholesky(R)
    logd = torch.log(torch.diagonal(L, dim1=1, dim2=2) + 1e-10)
    cum = torch.cumsum(logd, 1)
    logdet_R = 2 * sum(cum[:, n - 1] for n in lens)
    Linv = torch.linalg.solve_triangular(L, torch.eye(m).expand_as(L), upper=False)
    Xw = torch.empty((a.shape[0],) + tuple(X.shape))
    s = 0
    for n in lens:
        Xw[:, s : s + n] = Linv[:, :n, :n] @ X[s : s + n]
        s += n
    Lx = torch.linalg.cholesky(Xw.transpose(1, 2) @ Xw)
    Q = torch.linalg.solve_triangular(Lx, Xw.transpose(1, 2), upper=False).transpose(1, 2)
    logdet_X = 2 * torch.log(torch.diagonal(Lx, dim1=1, dim2=2).abs() + 1e-10).sum(1)
    return Linv, Xw, Q, logdet_R + logdet_X


def _whiten_rows(Y, Linv_p, lens):
    out = torch.empty_like(Y)
    s = 0
    for n in lens:
        out[:, s : s + n] = Y[:, s : s + n] @ Linv_p[:n, :n].T
        s += n
    return out


def fit(data, design, a_grid, b_grid, run_starts=None, exhaustive=False, threads=None, task_indices=None):
    """The default float32 CPU fit (``exhaustive`` for the reference's
    force_exhaustive_search). Returns a dict of per-voxel outputs as the
    reference's ``ARMA11Results`` holds them: ``index`` (pair index),
    ``arma_params``, ``betas``, ``tstats``, ``sigma2``, ``fstats``, ``r2``,
    ``arma_lambda`` and ``reml_likelihood``."""
    if threads:
        torch.set_num_threads(int(threads))
    Y = torch.as_tensor(np.asarray(data), dtype=torch.float32)
    X = torch.as_tensor(np.asarray(design), dtype=torch.float32)
    V, T = Y.shape
    K = X.shape[1]
    starts = sorted(set([0] + [int(s) for s in np.asarray(run_starts if run_starts is not None else []).reshape(-1)]))
    lens = [e - s for s, e in zip(starts, starts[1:] + [T])]
    scale = Y.std(dim=1).clamp(min=1e-8)
    Ys = Y / scale[:, None]
    a, b, lam = _grid(a_grid, b_grid)
    P = a.shape[0]
    Linv, Xw, Q, const = _factors(X, a, lam, lens)
    pinv = torch.linalg.pinv(X.double()).float()
    Yr = Ys - (Ys @ pinv.T) @ X.T

    def crit(p, rows):
        Yw = _whiten_rows(Yr[rows], Linv[p], lens)
        rss = Yw.pow(2).sum(1, dtype=torch.float64) - (Yw @ Q[p]).pow(2).sum(1, dtype=torch.float64)
        return (const[p].double() + (T - K) * torch.log(rss + 1e-10)).float()

    a_ax = torch.unique(a)
    b_ax = torch.unique(b)
    table = torch.full((a_ax.numel(), b_ax.numel()), -1, dtype=torch.long)
    ai = torch.searchsorted(a_ax, a)
    bi = torch.searchsorted(b_ax, b)
    table[ai, bi] = torch.arange(P)
    best = torch.full((V,), float("inf"))
    za = int(torch.nonzero(a_ax.abs() < 1e-6)[0])
    zb = int(torch.nonzero(b_ax.abs() < 1e-6)[0])
    ba = torch.full((V,), za, dtype=torch.long)
    bb = torch.full((V,), zb, dtype=torch.long)
    allv = torch.arange(V)
    if exhaustive:
        for p in range(P):
            c = crit(p, allv)
            imp = c < best
            best[imp] = c[imp]
            ba[imp] = ai[p]
            bb[imp] = bi[p]
    else:
        def ev(i, j, rows):
            p = int(table[i, j])
            if p < 0 or rows.numel() == 0:
                return
            c = crit(p, rows)
            imp = c < best[rows]
            r = rows[imp]
            best[r] = c[imp]
            ba[r] = i
            bb[r] = j

        ev(za, zb, allv)
        n_a, n_b = a_ax.numel(), b_ax.numel()
        ltop = max(0, min(n_a, n_b).bit_length() - 2)
        for lev in range(ltop, -1, -1):
            step = 1 << lev
            if lev == ltop:
                lo_a, hi_a = torch.zeros(V, dtype=torch.long), torch.full((V,), n_a - 1)
                lo_b, hi_b = torch.zeros(V, dtype=torch.long), torch.full((V,), n_b - 1)
            else:
                lo_a, hi_a = (ba - step).clamp(0, n_a - 1), (ba + step).clamp(0, n_a - 1)
                lo_b, hi_b = (bb - step).clamp(0, n_b - 1), (bb + step).clamp(0, n_b - 1)
            for j in range(0, n_b, step):
                inb = (j >= lo_b) & (j <= hi_b)
                if not bool(inb.any()):
                    continue
                for i in range(0, n_a, step):
                    if table[i, j] < 0:
                        continue
                    win = inb & (i >= lo_a) & (i <= hi_a)
                    ev(i, j, torch.nonzero(win).flatten())
    idx = table[ba, bb]
    # GLS per chosen pair (arma.py:4853-4905, :5227-5363): betas, float64
    # sigma2, t, F (task columns when given) and R^2 of the scaled data
    betas = torch.empty(V, K)
    tstats = torch.empty(V, K)
    sigma2 = torch.empty(V)
    fstats = torch.empty(V)
    r2 = torch.empty(V)
    dof = max(1, T - K)
    ti = list(task_indices) if task_indices else None
    for p in torch.unique(idx).tolist():
        rows = torch.nonzero(idx == p).flatten()
        XtX = Xw[p].T @ Xw[p]
        A = torch.cholesky_inverse(torch.linalg.cholesky(XtX))
        Yw = _whiten_rows(Ys[rows], Linv[p], lens)
        bp = (Yw @ Xw[p]) @ A.T
        rw = Yw - bp @ Xw[p].T
        s2 = (rw.pow(2).sum(1, dtype=torch.float64) / dof).float()
        tstats[rows] = bp / (torch.sqrt(s2[:, None] * torch.diagonal(A)[None, :]) + 1e-10)
        if ti is not None:
            M = torch.linalg.inv(A[ti][:, ti] + 1e-8 * torch.eye(len(ti)))
            bt = bp[:, ti]
            fstats[rows] = ((bt @ M) * bt).sum(1) / (s2 * len(ti) + 1e-10)
        else:
            fstats[rows] = ((bp @ XtX) * bp).sum(1) / (s2 * K + 1e-10)
        yv = Ys[rows]
        pred = bp @ X.T
        ss_res = (yv - pred).pow(2).sum(1)
        ss_tot = (yv - yv.mean(1, keepdim=True)).pow(2).sum(1)
        r2[rows] = torch.where(ss_tot <= 1e-10, torch.zeros_like(ss_tot),
                               torch.clamp(1.0 - ss_res / ss_tot.clamp(min=1e-10), max=1.0))
        betas[rows] = bp * scale[rows, None]
        sigma2[rows] = s2 * scale[rows] ** 2
    pa, pb = a[idx], b[idx]
    lam_out = (pb + pa) * (1 + pa * pb) / (((1 + (2 * pa) * pb) + pb * pb) + 1e-10)
    return {"index": idx.numpy(), "arma_params": torch.stack([pa, pb], 1).numpy(), "betas": betas.numpy(),
            "tstats": tstats.numpy(), "sigma2": sigma2.numpy(), "fstats": fstats.numpy(), "r2": r2.numpy(),
            "arma_lambda": lam_out.numpy(), "reml_likelihood": best.numpy()}
