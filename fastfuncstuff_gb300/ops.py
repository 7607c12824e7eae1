"""The library's entry points registered as torch custom operators (``ffs_gb300::``).

``torch.ops.ffs_gb300.fit_arma11`` runs one ARMA(1,1) REML voxelwise fit (the
default float32 path of fastfuncstuff/glm/arma.py:3650, full grid) on
caller-owned CUDA tensors and returns new CUDA tensors; ``reml_search`` and
``reml_gls`` are its two halves (fastfuncstuff/glm/arma.py:1886-2018 and
:4784-5590). Every op has a fake (meta) implementation, so the ops trace under
``torch.compile`` / ``torch.export`` as opaque calls into libffs_reml.so.
"""

from __future__ import annotations

import numpy as np
import torch

from .glm import engine
from .glm.grid import make_grid, run_layout


def _factors(X: torch.Tensor, a_grid: torch.Tensor, b_grid: torch.Tensor, run_starts: list[int]):
    T = X.shape[0]
    layout = run_layout(T, list(run_starts) if run_starts else None, None)
    grid = make_grid(a_grid.detach().cpu(), b_grid.detach().cpu())
    return engine.build_factors(X, grid, layout), layout


@torch.library.custom_op("ffs_gb300::reml_search", mutates_args=())
def reml_search(Y: torch.Tensor, X: torch.Tensor, a_grid: torch.Tensor, b_grid: torch.Tensor,
                run_starts: list[int], hierarchical: bool) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """(V, T) data, (T, K) design -> (params (V, 2) = (a, b), criterion (V,), scale (V,))."""
    f, _ = _factors(X, a_grid, b_grid, run_starts)
    out = engine.search(Y.float().contiguous(), f, hierarchical=hierarchical)
    best = out.best.long()
    params = torch.stack([f.a[best], f.b[best]], 1)
    return params, out.best_crit, out.scale


@reml_search.register_fake
def _(Y, X, a_grid, b_grid, run_starts, hierarchical):
    V = Y.shape[0]
    return Y.new_empty(V, 2), Y.new_empty(V), Y.new_empty(V)


@torch.library.custom_op("ffs_gb300::reml_gls", mutates_args=())
def reml_gls(Y: torch.Tensor, X: torch.Tensor, params: torch.Tensor, a_grid: torch.Tensor, b_grid: torch.Tensor,
             run_starts: list[int]) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor,
                                             torch.Tensor]:
    """GLS refit at each voxel's (a, b) = params[v] (a grid point) ->
    (betas (V, K), tstats (V, K), sigma2, fstats, r2, lambda)."""
    f, _ = _factors(X, a_grid, b_grid, run_starts)
    g = f.grid
    idx = g.index_of(params[:, 0].detach().cpu().numpy().astype(np.float32),
                     params[:, 1].detach().cpu().numpy().astype(np.float32))
    if (idx < 0).any():
        raise ValueError("reml_gls: params holds a pair that is not a valid grid point")
    best = torch.from_numpy(idx.astype(np.int32)).to(Y.device)
    Yf = Y.float().contiguous()
    scale = torch.empty(Y.shape[0], dtype=torch.float32, device=Y.device)
    pre = engine.prep(Yf, f, tensor_core=False, want_yr_t=False, scale=scale)
    o = engine.gls(Yf, pre.scale, best, f, X)
    return o.betas, o.tstats, o.sigma2, o.fstats, o.r2, o.lam


@reml_gls.register_fake
def _(Y, X, params, a_grid, b_grid, run_starts):
    V, K = Y.shape[0], X.shape[1]
    return (Y.new_empty(V, K), Y.new_empty(V, K), Y.new_empty(V), Y.new_empty(V), Y.new_empty(V), Y.new_empty(V))


@torch.library.custom_op("ffs_gb300::fit_arma11", mutates_args=())
def fit_arma11(Y: torch.Tensor, X: torch.Tensor, a_grid: torch.Tensor, b_grid: torch.Tensor, run_starts: list[int],
               hierarchical: bool) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor,
                                            torch.Tensor, torch.Tensor, torch.Tensor]:
    """One full fit -> (betas, tstats, sigma2, fstats, r2, params (V, 2), lambda, reml criterion)."""
    from .glm.arma import fit_glm_arma11

    r = fit_glm_arma11(Y, X, 2.0, a_grid=a_grid, b_grid=b_grid, run_starts=list(run_starts) or None,
                       device=Y.device, verbose=False, force_exhaustive_search=not hierarchical, return_device=True)
    return r.betas, r.tstats, r.sigma2, r.fstats, r.r2, r.arma_params, r.arma_lambda, r.reml_likelihood


@fit_arma11.register_fake
def _(Y, X, a_grid, b_grid, run_starts, hierarchical):
    V, K = Y.shape[0], X.shape[1]
    e = Y.new_empty
    return e(V, K), e(V, K), e(V), e(V), e(V), e(V, 2), e(V), e(V)
