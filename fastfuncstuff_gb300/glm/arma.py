"""The ARMA(1,1) REML voxelwise GLM with the reference's Python API, on one GB300.

``fit_glm_arma11`` and ``fit_glm_arma11_grouped`` take the arguments of
fastfuncstuff/glm/arma.py:3650-3692 and :2836-2843 and return an
``ARMA11Results`` with the same fields, as CPU tensors. The work runs in
libffs_reml.so's sm_103a kernels (see ``engine``); there is no CPU path.

What is computed is the reference's default float32 fit:

* the grid of valid (a, b) pairs, in the reference's order (``grid.make_grid``);
* per voxel: std scaling, residualisation against the design, the REML
  criterion at every pair, and the hierarchical (default) or exhaustive
  (``force_exhaustive_search``) selector;
* the GLS refit at the chosen pair: betas, t, sigma2, F, R^2, lambda, GLT
  contrasts, partial / semi-partial R^2, Ljung-Box, residuals and predictions,
  unscaled by the voxel's std.

``use_double=True`` selects the reference's FP64-mode semantics (validity filter
and lambda in float64, no std scaling: the likelihood is that of the raw data)
and returns float64 tensors; the arithmetic is this build's (FP64 factors,
fp32 / split-bf16 voxel work).

Options outside this path (the OLS side fits) raise NotImplementedError;
AFNI-faithful mode (``set_afni_mode``) runs every fit path with AFNI's banded
R.
"""

from __future__ import annotations

import math
import warnings
from collections.abc import Callable
from typing import Any

import numpy as np
import torch

from . import engine
from .._lib import FFS_DSORT_QMAX
from .grid import (
    RemlGrid,
    build_censor_run_info,
    compute_arma_lambda,
    ensure_zero_in_grid,
    estimate_valid_grid_pairs,
    get_default_arma_grids,
    grid_of_pairs,
    ljung_box_plan,
    make_grid,
    parse_grid_arg,
    run_bounds,
    run_layout,
    set_afni_mode,
)

__all__ = [
    "ARMA11Results",
    "VOXEL_SCATTER_ATTRS",
    "build_censor_run_info",
    "compute_arma_lambda",
    "ensure_zero_in_grid",
    "estimate_valid_grid_pairs",
    "fit_glm_arma11",
    "fit_glm_arma11_grouped",
    "fit_glm_arma11_perhrf",
    "get_default_arma_grids",
    "parse_grid_arg",
    "precompute_reml_grid",
    "run_bounds",
    "search_voxels_precomputed_grid",
    "set_afni_mode",
]

# Per-voxel arrays of ARMA11Results (fastfuncstuff/glm/arma.py:186-213).
VOXEL_SCATTER_ATTRS = [
    "betas", "tstats", "r2", "r2_partial", "r2_partial_nuisance", "r2_semipartial",
    "r2_semipartial_nuisance", "arma_params", "arma_lambda", "reml_likelihood", "sigma2", "fstats",
    "residuals", "residuals_whitened", "predicted", "contrast_betas", "contrast_tstats",
    "contrast_fstats", "contrast_r2_partial", "contrast_r2_semipartial", "dsort_betas", "dsort_tstats",
    "ljung_box", "set_fstats", "set_sd", "set_coef",
]


class ARMA11Results:
    """Container for ARMA(1,1) GLM results (fields of fastfuncstuff/glm/arma.py:585-692)."""

    def __init__(self):
        self.betas = None
        self.tstats = None
        self.r2 = None
        self.r2_partial = None
        self.r2_partial_nuisance = None
        self.r2_semipartial = None
        self.r2_semipartial_nuisance = None
        self.arma_params = None
        self.arma_lambda = None
        self.reml_likelihood = None
        self.residuals = None
        self.predicted = None
        self.residuals_whitened = None
        self.ljung_box = None
        self.ljung_box_dof = None
        self.sigma2 = None
        self.var_betas = None
        self.original_shape = None
        self.fstats = None
        self.set_fstats = None
        self.set_sd = None
        self.set_coef = None
        self.nuisance_sets = None
        self.voxel_mean = None
        self.dof = None
        self.tr = None
        self.voxel_mask = None
        self.full_shape = None
        self.fitted_column_indices = None
        self.n_regressors_full = None
        self.contrast_labels = None
        self.contrast_betas = None
        self.contrast_tstats = None
        self.contrast_fstats = None
        self.contrast_r2_partial = None
        self.contrast_r2_semipartial = None
        self.affine = None
        self.ols_results = None
        self.dsort_betas = None
        self.dsort_tstats = None
        self.dsort_labels = None
        self.nods_results = None
        self.reml_lklhd_surface = None
        self.reml_surface_params = None
        self._deferred_ols_write_callback = None


def _to_tensor(x, dtype=torch.float32) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.detach().to(dtype=dtype)
    return torch.as_tensor(np.asarray(x), dtype=dtype)


def _unsupported(name: str) -> None:
    raise NotImplementedError(
        f"{name} is not part of the ARMA(1,1) REML hot path this GB300 build implements"
    )


def precompute_reml_grid(X, n_timepoints: int, a_grid, b_grid, device=None, *, run_starts=None, tau=None,
                         use_double: bool = False, task_indices=None, glt_matrices=None) -> engine.GridFactors:
    """The per-pair factors of a design (replaces fastfuncstuff/glm/arma.py:1371-1531).

    Returns the device-resident ``GridFactors`` (logdets, the recurrence
    coefficients standing in for L^-1, U = L^-T Q, the GLS matrices).
    """
    device = engine.require_cuda(device)
    X = _to_tensor(X).to(device)
    if X.shape[0] != n_timepoints:
        raise ValueError(f"Timepoints mismatch: n_timepoints={n_timepoints}, design has {X.shape[0]}")
    grid = make_grid(a_grid, b_grid, use_double=use_double)
    layout = run_layout(n_timepoints, run_starts, tau)
    glt = None
    if glt_matrices is not None:
        glt = np.stack([np.asarray(g, np.float32).reshape(-1) for g in glt_matrices])
    return engine.build_factors(X, grid, layout, task_indices=task_indices, glt=glt,
                                with_tc=X.shape[1] <= TC_MAX_K)


def search_voxels_precomputed_grid(X, Y_batch, factors: engine.GridFactors, device=None, *,
                                   hierarchical: bool = False, return_profile: bool = False):
    """Search seam of fastfuncstuff/glm/arma.py:1886-2018 on the GPU.

    Returns ``(best_params (V, 2), best_likelihoods (V,))`` and, with
    ``return_profile``, also ``(surface (V, P), param_list)``. The data are
    scaled by their std first, as the float32 fit does.
    """
    device = engine.require_cuda(device)
    Y = _to_tensor(Y_batch).to(device)
    out = engine.search(Y, factors, hierarchical=hierarchical, projector=_projector(factors),
                        keep_surface=return_profile)
    g = factors.grid
    best = out.best.long()
    params = torch.stack([torch.from_numpy(g.a).to(device)[best], torch.from_numpy(g.b).to(device)[best]], 1)
    if return_profile:
        surface = (out.surf.double() + out.crit0[None, :]).float().t().contiguous()
        return params, out.best_crit, surface, g.param_list()
    return params, out.best_crit


# Widest design the tcgen05 projection takes (one 256-column MMA tile holds a
# pair's K columns); wider designs are projected on the CUDA cores.
TC_MAX_K = 256


def _projector(factors: engine.GridFactors) -> str:
    """The projection kernel of the factors: tcgen05 when they carry its fp16
    operands (K <= TC_MAX_K), else the CUDA-core kernel."""
    return "tc" if factors.U_hi is not None else "simt"


_SIDE: dict = {}


def _side_stream(device) -> torch.cuda.Stream:
    """A second stream of device (the grid build runs there beside the prep)."""
    key = str(device)
    if key not in _SIDE:
        _SIDE[key] = torch.cuda.Stream(device)
    return _SIDE[key]


def _batch_size(V: int, T: int, P: int, K: int, batch_size, device) -> int:
    if batch_size:
        return max(1, min(int(batch_size), V))
    per_voxel = 4 * (3 * P + 6 * T + 4 * K + 16)
    free, _ = torch.cuda.mem_get_info(device)
    return max(1, min(V, int(0.5 * free // per_voxel)))


def fit_glm_arma11(
    data,
    design,
    tr: float,
    a_grid=None,
    b_grid=None,
    estimate_per_voxel: bool = True,
    batch_size: int | None = None,
    want_residuals: bool = False,
    want_predicted: bool = False,
    want_ljung_box: bool = False,
    want_r2_partial: bool = False,
    r2_partial_mode: str = "full",
    want_r2_semipartial: bool = False,
    r2_semipartial_mode: str = "full",
    want_ols: bool = False,
    want_ols_residuals: bool = False,
    want_ols_predicted: bool = False,
    ols_write_callback: Callable | None = None,
    precomputed_arma_params=None,
    device=None,
    verbose: bool = True,
    cholesky_on_cpu: bool = True,
    use_double: bool = False,
    use_qr: bool = False,
    debug_memory: bool = False,
    force_exhaustive_search: bool = False,
    glt_labels: list[str] | None = None,
    glt_matrices: list | None = None,
    task_indices: list[int] | None = None,
    use_grid_batching: bool | None = None,
    spatial_metadata: dict | None = None,
    legacy_contrasts: bool = False,
    save_profile_likelihoods: bool = False,
    run_starts=None,
    autocorr_cache: Any = None,
    dsort=None,
    dsort_labels=None,
    dsort_run_bounds=None,
    want_dsort_nods: bool = False,
    tau=None,
    column_sets=None,
    *,
    return_device: bool = False,
    proposal=None,
    proposal_recenter: int = 0,
    cuda_graphs: bool = True,
    _group_designs=None,
) -> ARMA11Results:
    """Fit a GLM with ARMA(1,1) REML prewhitening (fastfuncstuff/glm/arma.py:3650).

    Arguments mean what they mean in the reference. ``cholesky_on_cpu``,
    ``use_qr``, ``use_grid_batching``, ``debug_memory``, ``legacy_contrasts`` and
    ``autocorr_cache`` tune the reference's CPU/GPU memory plan and have no
    counterpart here (the factors are built on the GPU in FP64, with the QR
    fallback applied per pair when the Cholesky of X_w'X_w fails). Extra
    keywords: ``return_device`` (keep result tensors on the GPU), ``proposal`` (a trained
    ``learned.ArmaProposal``: search each voxel's 5 x 5 window around its
    proposal, the full grid for window-edge voxels) and ``proposal_recenter``
    (re-centred window rounds before that fallback), ``cuda_graphs`` (replay
    the learned-seeded fit of one voxel batch, and the grouped fit of
    fit_glm_arma11_grouped, from CUDA graphs).
    """
    if want_ols or want_ols_residuals or want_ols_predicted or ols_write_callback is not None:
        _unsupported("the OLS side fit (want_ols)")
    if want_dsort_nods and dsort is None:
        raise ValueError("want_dsort_nods needs dsort")
    if not estimate_per_voxel and _group_designs is not None:
        _unsupported("global ARMA estimation (estimate_per_voxel=False) of grouped designs")
    out_dtype = torch.float64 if use_double else torch.float32

    Y = data if isinstance(data, torch.Tensor) else torch.from_numpy(np.asarray(data))
    original_shape = None
    if Y.ndim == 4:
        original_shape = tuple(Y.shape[:3])
        Y = Y.reshape(-1, Y.shape[-1])
    elif Y.ndim != 2:
        raise ValueError(f"Data must be 2D or 4D, got {Y.ndim}D")
    X = _to_tensor(design)
    V, T = Y.shape
    if X.ndim != 2 or X.shape[0] != T:
        raise ValueError(f"Timepoints mismatch: Data has {T}, Design has {X.shape[0]}")
    K = X.shape[1]
    if T - K <= 0:
        warnings.warn("Non-positive degrees of freedom detected in ARMA(1,1) fit; statistics may be "
                      "unreliable", stacklevel=2)
    dof = max(1, T - K)
    device = engine.require_cuda(device)
    Xd = X.to(device=device, dtype=torch.float32)

    glt = None
    if glt_labels and glt_matrices:
        rows = []
        for gm in glt_matrices:
            g = np.asarray(gm, dtype=np.float32)
            if g.ndim == 2 and g.shape[0] != 1:
                raise NotImplementedError(
                    f"Multi-row GLT contrasts (F-tests) not yet supported. Got shape {g.shape}")
            rows.append(g.reshape(-1))
        glt = np.stack(rows)
    ti = list(task_indices) if task_indices else None
    Dd = None
    if dsort is not None:
        # voxelwise regressors: (a, b) is estimated on the base design only; the
        # final GLS of every voxel is redone with [X | D_v] (gls_dsort)
        Dd = engine.dsort_prepare(dsort, V, T, dsort_run_bounds, device)
        if Dd.shape[1] > FFS_DSORT_QMAX:
            raise NotImplementedError(f"-dsort with {Dd.shape[1]} columns (at most {FFS_DSORT_QMAX})")
    sets = None
    if column_sets:
        sets = engine.column_sets_plan(column_sets, _group_designs[0].cpu().numpy() if _group_designs is not None
                                       else X.numpy())
    layout = run_layout(T, run_starts, tau)
    lj = ljung_box_plan(T, K, run_starts, tau) if want_ljung_box else None

    res = ARMA11Results()
    res.original_shape = original_shape
    res.fitted_column_indices = ti
    res.n_regressors_full = K
    res.dof = dof
    res.tr = tr

    if precomputed_arma_params is not None:
        pa = _to_tensor(precomputed_arma_params).reshape(-1, 2)
        if pa.shape[0] != V:
            raise ValueError(f"precomputed_arma_params must have shape ({V}, 2), got {tuple(pa.shape)}")
        pairs, inv = np.unique(pa.numpy().astype(np.float32), axis=0, return_inverse=True)
        grid = grid_of_pairs(pairs[:, 0], pairs[:, 1], use_double=use_double)
        factors = engine.build_factors(Xd, grid, layout, task_indices=ti, glt=glt, with_tc=False, sets=sets,
                                       afull=Dd is not None and bool(column_sets))
        best_all = torch.from_numpy(inv.reshape(-1).astype(np.int32))
        crit_all = None
    else:
        if a_grid is None and b_grid is None:
            a_grid, b_grid = get_default_arma_grids()
        elif a_grid is None:
            a_grid = get_default_arma_grids()[0]
        elif b_grid is None:
            b_grid = get_default_arma_grids()[1]
        grid = make_grid(a_grid, b_grid, use_double=use_double)
        factors = None  # built below, unless the CUDA-graph plan builds them inside its graph
        best_all = crit_all = None

    global_crit = None
    if not estimate_per_voxel and best_all is None:
        # one (a, b) for every voxel, from the mean series (unscaled), by the
        # full grid's exhaustive argmin; its criterion is every voxel's
        # (fastfuncstuff/glm/arma.py:5603-5628)
        factors = engine.build_factors(Xd, grid, layout, task_indices=ti, glt=glt, with_tc=K <= TC_MAX_K,
                                       sets=sets, afull=Dd is not None and bool(column_sets))
        # the mean in the fit's dtype (the reference's data.mean(0)), searched
        # in float32 like every series
        ym = Y.to(device=device, dtype=out_dtype).mean(0, keepdim=True).float()
        so = engine.search(ym, factors, hierarchical=False, projector=_projector(factors), do_scale=False)
        best_all = so.best.expand(V).to(torch.int32).cpu()
        global_crit = so.best_crit[:1].expand(V)
    P = grid.P
    bs = _batch_size(V, T, P, K, batch_size, device)
    use_graph = (best_all is None and proposal is not None and cuda_graphs and lj is None and bs >= V
                 and Dd is None and _group_designs is None)
    # results for the host straight from the GLS kernels (pinned memory
    # written over the host link while they run) when nothing else reads them
    # on the device
    host_gls = (use_graph and not return_device and not use_double and not ti and sets is None
                and not (want_r2_partial or want_r2_semipartial))
    afull = Dd is not None and bool(column_sets)
    q0 = join = None
    slots = None
    gplan = None
    if _group_designs is not None:
        # grouped fit (fit_glm_arma11_grouped): every design's factors in one
        # grid build, every voxel against its own design in one pass per stage
        Xs, gid = _group_designs
        bs = V
        if (cuda_graphs and lj is None and Dd is None and sets is None and not save_profile_likelihoods
                and proposal is None):
            # the whole grouped fit replayed from one CUDA graph
            gplan = engine.grouped_graph_for(Y, Xs, grid, layout, gid, hierarchical=not force_exhaustive_search,
                                             do_scale=not use_double,
                                             gls_kw=dict(want_residuals=want_residuals,
                                                         want_predicted=want_predicted),
                                             factor_kw=dict(task_indices=ti, glt=glt, with_tc=True))
            slots = gplan.slots
        else:
            factors = engine.build_factors(Xs, grid, layout, task_indices=ti, glt=glt, with_tc=True, sets=sets,
                                           afull=afull)
            slots = engine.design_slots(gid, Xs.shape[0], K, P, device)
    if factors is None and not use_graph and gplan is None:
        # the grid build runs on a side stream while the residualisation of the
        # first batch (against the design basis) runs on the main one
        overlap = K <= engine.BASIS_MAX_K
        # beside the prep on a side stream, except under the per-call stage
        # timer, whose stage times are then each kernel's own
        side = _side_stream(device) if overlap and not engine.stage_timer_active() else None
        center = None
        if overlap:
            # Q0 and the centring test of the design (one kernel pair), queued
            # first: the build's stream waits for them
            q0, cflag, ccoef = engine.design_basis(Xd, with_constant=True)
            center = (cflag, ccoef)
        factors = engine.build_factors(Xd, grid, layout, task_indices=ti, glt=glt,
                                       with_tc=K <= TC_MAX_K, stream=side, sets=sets,
                                       afull=afull, center=center)
        if overlap:
            built = torch.cuda.Event()
            built.record(side)
            main = torch.cuda.current_stream()

            def join():
                main.wait_event(built)
    keep = [] if return_device else None
    chunks = {k: [] for k in ("best", "crit", "surf", "betas", "tstats", "sigma2", "fstats", "r2", "lam",
                              "cb", "ct", "resid", "resid_w", "pred", "lb", "scale")}
    factors_used = factors
    dchunks = []
    proj = "tc" if factors is None else _projector(factors)
    if proposal is not None and best_all is None:
        from . import learned

        layout_l = layout
        fb_voxels = 0.0  # voxels the full grid decided (host numbers the search reads back anyway)
    for v0 in range(0, V, bs):
        v1 = min(V, v0 + bs)
        if use_graph and not Y.is_cuda and Y.dtype == torch.float32 and Y.is_pinned() and Y.is_contiguous():
            # pinned host data: a staged plan copies the rows in by chunks
            # beside the grid build and preps each chunk as it lands
            Yb = Y[v0:v1]
        else:
            Yb = Y[v0:v1].to(device=device, dtype=torch.float32, non_blocking=True)
        go = None
        if use_graph:
            plan = learned.graph_for(Yb, Xd, grid, layout_l, proposal, recenter=proposal_recenter,
                                     do_scale=not use_double,
                                     gls_kw=dict(want_residuals=want_residuals, want_predicted=want_predicted),
                                     factor_kw=dict(task_indices=ti, glt=glt, with_tc=K <= TC_MAX_K, sets=sets))
            lo, go = plan.run(Yb, Xd, host_out=host_gls)
            factors_used = plan.f
            best, scale = lo.best, lo.scale
            chunks["best"].append(best)
            chunks["crit"].append(lo.best_crit)
            fb_voxels += lo.stats["fallback"] * (v1 - v0)
        elif best_all is None and proposal is not None and slots is not None:
            # grouped designs: each design's voxels searched and refit against
            # that design's view of the one multi-design build
            best, crit_g, scale, go, nf = learned.grouped_learned_fit(
                Yb, factors, _group_designs[1][v0:v1], _group_designs[0], proposal, layout_l,
                do_scale=not use_double, recenter=proposal_recenter,
                gls_kw=dict(want_residuals=want_residuals, want_predicted=want_predicted), lj=lj, slots=slots)
            chunks["best"].append(best)
            chunks["crit"].append(crit_g)
            fb_voxels += nf
        elif best_all is None and proposal is not None:
            # the GLS of every voxel at its window's pair is queued before the
            # host waits for the list of fallback voxels; their rows are redone
            first = {}

            def gls_first(best_w, scale_w):
                first["go"] = engine.gls(Yb, scale_w, best_w, factors, Xd, want_residuals=want_residuals,
                                         want_predicted=want_predicted, lj=lj)

            lo = learned.learned_search(Yb, factors, proposal, layout_l, do_scale=not use_double,
                                        recenter=proposal_recenter, before_fallback=gls_first, q0=q0, join=join)
            best, scale = lo.best, lo.scale
            chunks["best"].append(best)
            chunks["crit"].append(lo.best_crit)
            fb_voxels += lo.stats["fallback"] * (v1 - v0)
            go = first["go"]
            sel = lo.fallback_idx
            if sel.numel():
                gs = engine.gls(Yb.index_select(0, sel), scale.index_select(0, sel), best.index_select(0, sel),
                                factors, Xd, want_residuals=want_residuals, want_predicted=want_predicted, lj=lj)
                for fld in ("betas", "tstats", "sigma2", "fstats", "r2", "lam", "cbeta", "ct", "resid",
                            "resid_w", "pred", "ljung_box"):
                    t_all, t_sub = getattr(go, fld), getattr(gs, fld)
                    if t_all is not None:
                        t_all.index_copy_(0, sel, t_sub)
        elif gplan is not None:
            so, go = gplan.run(Yb, _group_designs[0])
            factors_used = gplan.f
            best, scale = so.best, so.scale
            chunks["best"].append(best)
            chunks["crit"].append(so.best_crit)
        elif slots is not None:
            so = engine.search_designs(Yb, factors, slots, hierarchical=not force_exhaustive_search,
                                       do_scale=not use_double)
            best, scale = so.best, so.scale
            chunks["best"].append(best)
            chunks["crit"].append(so.best_crit)
            go = engine.gls(Yb, scale, best, factors, _group_designs[0], want_residuals=want_residuals,
                            want_predicted=want_predicted, lj=lj, design=slots.design)
        elif best_all is None:
            so = engine.search(Yb, factors, hierarchical=not force_exhaustive_search, projector=proj,
                               do_scale=not use_double, keep_surface=save_profile_likelihoods, q0=q0, join=join)
            best, scale = so.best, so.scale
            chunks["best"].append(best)
            chunks["crit"].append(so.best_crit)
            if save_profile_likelihoods:
                chunks["surf"].append((so.surf.double() + so.crit0[None, :]).float().t())
        else:
            if join is not None:
                join()
            best = best_all[v0:v1].to(device)
            scale = _voxel_scale(Yb, not use_double)
            chunks["best"].append(best)
        if go is None:
            go = engine.gls(Yb, scale, best, factors, Xd, want_residuals=want_residuals,
                            want_predicted=want_predicted, lj=lj)
        if Dd is not None:
            do = engine.gls_dsort(Yb, scale, best, factors, _group_designs[0] if slots is not None else Xd,
                                  Dd[v0:v1], want_residuals=want_residuals, want_predicted=want_predicted, lj=lj,
                                  design=slots.design if slots is not None else None, column_sets=column_sets)
            dchunks.append(do)
        if sets is not None:
            chunks["scale"].append(scale)
        for name, t in (("betas", go.betas), ("tstats", go.tstats), ("sigma2", go.sigma2),
                        ("fstats", go.fstats), ("r2", go.r2), ("lam", go.lam), ("cb", go.cbeta),
                        ("ct", go.ct), ("resid", go.resid), ("resid_w", go.resid_w), ("pred", go.pred),
                        ("lb", go.ljung_box)):
            if t is not None:
                chunks[name].append(t)

    def cat(name):
        xs = chunks[name]
        if not xs:
            return None
        return xs[0] if len(xs) == 1 else torch.cat(xs)  # one batch: no copy

    pending = []  # host copies queued on the stream, waited for once before returning

    def out(t, dtype=None):
        if t is None:
            return None
        if not t.is_cuda:  # written by the kernels into pinned host memory
            pending.append(t)
            return t.to(dtype=dtype or out_dtype)
        t = t.to(dtype=dtype or out_dtype)
        if return_device:
            return t
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t, non_blocking=True)
        pending.append(h)
        return h

    best = cat("best")
    ab_t = engine.const_dev(np.stack([grid.a, grid.b], 1), device)  # [P][2]
    res.arma_params = out(ab_t.index_select(0, best))
    if precomputed_arma_params is not None:
        res.arma_params = out(_to_tensor(precomputed_arma_params).reshape(-1, 2).to(device))
        res.reml_likelihood = out(torch.zeros(V, device=device))
    elif global_crit is not None:
        res.reml_likelihood = out(global_crit)
    else:
        res.reml_likelihood = out(cat("crit"))
    lam = cat("lam")
    if use_double:
        ab = res.arma_params.to(device=device, dtype=torch.float64)
        av, bv = ab[:, 0], ab[:, 1]
        lam = (bv + av) * (1 + av * bv) / (1 + 2 * av * bv + bv**2 + 1e-10)
    res.arma_lambda = out(lam)
    betas, tstats = cat("betas"), cat("tstats")
    sel = torch.as_tensor(ti, device=device) if ti else None
    res.betas = out(betas if sel is None else betas[:, sel])
    res.tstats = out(tstats if sel is None else tstats[:, sel])
    res.sigma2 = out(cat("sigma2"))
    res.fstats = out(cat("fstats"))
    res.r2 = out(cat("r2"), torch.float32)
    if want_r2_partial or want_r2_semipartial:
        _partial_r2(res, tstats, res.r2, ti, K, dof, want_r2_partial, r2_partial_mode,
                    want_r2_semipartial, r2_semipartial_mode, out)
    if glt is not None:
        res.contrast_labels = glt_labels
        res.contrast_betas = out(cat("cb"))
        ct = cat("ct")
        res.contrast_tstats = out(ct)
        if want_r2_partial:
            res.contrast_r2_partial = out(ct**2 / (ct**2 + dof))
        if want_r2_semipartial:
            rem = torch.clamp(1.0 - cat("r2").to(ct.dtype)[:, None], min=0.0)
            res.contrast_r2_semipartial = out(ct**2 / (ct**2 + dof) * rem)
    if sets is not None:
        # the column sets' Wald F, temporal SD and coefficient (NaN for a set
        # outside the design), fastfuncstuff/glm/arma.py:3564-3586
        F, sd, coef = engine.set_stats(betas, cat("sigma2"), cat("scale"), best, factors_used,
                                       design=slots.design if slots is not None else None)
        res.set_fstats, res.set_sd, res.set_coef = out(F), out(sd), out(coef)
    if want_residuals:
        res.residuals = out(cat("resid"))
        res.residuals_whitened = out(cat("resid_w"))
    if want_predicted:
        res.predicted = out(cat("pred"))
    if want_ljung_box:
        res.ljung_box = out(cat("lb"), torch.float32) if chunks["lb"] else out(torch.zeros(V), torch.float32)
        res.ljung_box_dof = lj[3]
    if Dd is not None:
        _apply_dsort(res, dchunks, ti, K, T, dsort_labels, want_dsort_nods, want_r2_partial, r2_partial_mode,
                     want_r2_semipartial, r2_semipartial_mode, out, device)
    if save_profile_likelihoods and chunks["surf"]:
        res.reml_lklhd_surface = out(cat("surf"))
        res.reml_surface_params = grid.param_list()
    if proposal is not None and best_all is None:
        # fraction of voxels the full grid decided
        res.learned_fallback = fb_voxels / V
    if spatial_metadata:
        res.voxel_mask = spatial_metadata.get("voxel_mask")
        res.full_shape = spatial_metadata.get("volume_shape")
        res.affine = spatial_metadata.get("affine")
    if pending:
        torch.cuda.current_stream(device).synchronize()
    if verbose:
        print(f"ARMA(1,1) REML: {V:,} voxels x {P} pairs, T={T}, K={K} on {torch.cuda.get_device_name(device)}")
    return res


def _apply_dsort(res, dchunks, ti, K, T, labels, want_nods, want_p, mode_p, want_s, mode_s, out, device):
    """Overwrite the fit's GLS outputs with those of the -dsort GLS
    (fastfuncstuff/glm/arma.py:3449-3536, :5781-5824): base betas and t
    (task-filtered), dsort_betas / dsort_tstats, sigma2, F, R^2, GLT, partial
    R^2 with dof T - K - q, residuals, Ljung-Box and column sets; with
    ``want_nods`` the base-design fit is kept as ``nods_results``."""
    import copy

    if want_nods:
        res.nods_results = copy.copy(res)

    def cat(name):
        xs = [getattr(d, name) for d in dchunks]
        return torch.cat(xs) if xs and xs[0] is not None else None

    q = dchunks[0].dbetas.shape[1]
    dof = max(1, T - K - q)
    res.dof = dof
    status = torch.stack([d.status for d in dchunks]).amax()
    betas, tstats = cat("betas"), cat("tstats")
    sel = torch.as_tensor(ti, device=device) if ti else None
    res.betas = out(betas if sel is None else betas[:, sel])
    res.tstats = out(tstats if sel is None else tstats[:, sel])
    res.dsort_betas = out(cat("dbetas"))
    res.dsort_tstats = out(cat("dtstats"))
    res.dsort_labels = list(labels) if labels else [f"dsort#{k}" for k in range(q)]
    res.sigma2 = out(cat("sigma2"))
    res.fstats = out(cat("fstats"))
    r2 = cat("r2")
    res.r2 = out(r2, torch.float32)
    if want_p or want_s:
        _partial_r2(res, tstats, res.r2, ti, K, dof, want_p, mode_p, want_s, mode_s, out)
    if res.contrast_betas is not None:
        res.contrast_betas = out(cat("cbeta"))
        ct = cat("ct")
        res.contrast_tstats = out(ct)
        if want_p:
            res.contrast_r2_partial = out(ct**2 / (ct**2 + dof))
        if want_s:
            rem = torch.clamp(1.0 - r2.to(ct.dtype)[:, None], min=0.0)
            res.contrast_r2_semipartial = out(ct**2 / (ct**2 + dof) * rem)
    if res.residuals is not None:
        res.residuals = out(cat("resid"))
        res.residuals_whitened = out(cat("resid_w"))
    if res.predicted is not None:
        res.predicted = out(cat("pred"))
    if res.ljung_box is not None and dchunks[0].ljung_box is not None:
        res.ljung_box = out(cat("ljung_box"), torch.float32)
    if dchunks[0].set_fstats is not None:
        res.set_fstats, res.set_sd, res.set_coef = out(cat("set_fstats")), out(cat("set_sd")), out(cat("set_coef"))
    if int(status.item()):
        warnings.warn("-dsort: a voxel's regressors lie in the span of the design at its (a, b); their betas "
                      "there are not determined", stacklevel=3)


def _voxel_scale(Y: torch.Tensor, do_scale: bool) -> torch.Tensor:
    if not do_scale:
        return torch.ones(Y.shape[0], device=Y.device, dtype=torch.float32)
    return Y.double().std(dim=1).float().clamp(min=1e-8)


def _partial_r2(res, tstats, r2, ti, K, dof, want_p, mode_p, want_s, mode_s, out):
    """Partial and semi-partial R^2 from the t statistics.

    Follows fastfuncstuff/glm/arma.py:5298-5419: partial = t^2/(t^2 + dof), split
    into task / nuisance columns, optionally rescaled by the variance left after
    the nuisance columns (mode "task"); semi-partial = partial * (1 - R^2).
    """
    t2 = tstats.double() ** 2
    full = t2 / (t2 + dof)
    if ti is not None:
        nuis = sorted(set(range(K)) - set(ti))
        task = full[:, ti]
        nu = full[:, nuis] if nuis else None
    else:
        task, nu = full, None
    dt = torch.float64 if res.betas.dtype == torch.float64 else torch.float32
    if want_p:
        if mode_p == "task" and nu is not None:
            res.r2_partial = out(task / torch.clamp(1.0 - nu.sum(1, keepdim=True), min=0.01), dt)
        else:
            res.r2_partial = out(task, dt)
        if nu is not None:
            res.r2_partial_nuisance = out(nu, dt)
    if want_s:
        rem = torch.clamp(1.0 - r2.to(device=tstats.device, dtype=torch.float64)[:, None], min=0.0)
        st = task * rem
        sn = nu * rem if nu is not None else None
        if mode_s == "task" and sn is not None:
            res.r2_semipartial = out(st / torch.clamp(1.0 - sn.sum(1, keepdim=True), min=0.01), dt)
        else:
            res.r2_semipartial = out(st, dt)
        if sn is not None:
            res.r2_semipartial_nuisance = out(sn, dt)


def fit_glm_arma11_grouped(data, designs_by_group: dict, group_indices, tr: float, group_label: str = "group",
                           **fit_kwargs) -> ARMA11Results:
    """REML with one design per voxel group, scattered back (fastfuncstuff/glm/arma.py:2836-3183).

    Every design must share the shape of the first (ValueError), and every group
    id present must have a design (KeyError). The grid, the recurrence
    coefficients and the logdet(R) are design-independent and identical across
    groups; each group's voxels are fit against its own design.
    """
    Y = data if isinstance(data, torch.Tensor) else torch.from_numpy(np.asarray(data))
    gid = torch.as_tensor(np.asarray(group_indices.cpu() if isinstance(group_indices, torch.Tensor)
                                     else group_indices)).long().reshape(-1)
    V = Y.shape[0]
    if gid.shape[0] != V:
        raise ValueError(f"group_indices length {gid.shape[0]} != data n_voxels {V}")
    groups = sorted(int(h) for h in gid.unique().tolist())
    missing = [h for h in groups if h not in designs_by_group]
    if missing:
        raise KeyError(f"{group_label} ids {missing} present in voxels but missing from designs_by_group "
                       f"(have {sorted(designs_by_group.keys())})")
    shape0 = tuple(_to_tensor(designs_by_group[groups[0]]).shape)
    for h in groups[1:]:
        if tuple(_to_tensor(designs_by_group[h]).shape) != shape0:
            raise ValueError(f"designs_by_group[{h}] shape differs from {shape0} -- per-{group_label} "
                             "designs must share dims")
    pre = fit_kwargs.pop("precomputed_arma_params", None)
    fit_kwargs.setdefault("verbose", False)
    batched_ok = (pre is None and not fit_kwargs.get("save_profile_likelihoods", False)
                  and fit_kwargs.get("batch_size") is None and fit_kwargs.get("estimate_per_voxel", True)
                  and shape0[1] <= TC_MAX_K and len(groups) > 1)
    if batched_ok:
        # one fit over all groups: the designs stacked (D, T, K), each voxel
        # tagged with its design's index
        device = engine.require_cuda(fit_kwargs.get("device"))
        Xs = torch.stack([_to_tensor(designs_by_group[h]) for h in groups]).to(device=device,
                                                                                dtype=torch.float32)
        dense = np.searchsorted(np.asarray(groups), gid.numpy()).astype(np.int32)
        kw = dict(fit_kwargs)
        kw["device"] = device
        return fit_glm_arma11(Y, Xs[0], tr, _group_designs=(Xs, dense), **kw)
    per = {}
    dsort_all = fit_kwargs.get("dsort")
    for h in groups:
        m = gid == h
        kw = dict(fit_kwargs)
        if pre is not None:
            kw["precomputed_arma_params"] = _to_tensor(pre).reshape(-1, 2)[m]
        if dsort_all is not None:  # each group's voxels' regressors (fastfuncstuff/glm/arma.py:3035-3036)
            kw["dsort"] = (dsort_all if isinstance(dsort_all, torch.Tensor)
                           else torch.as_tensor(np.asarray(dsort_all)))[m.to(torch.bool)]
        per[h] = (m, fit_glm_arma11(Y[m], designs_by_group[h], tr, **kw))
    merged = ARMA11Results()
    first = per[groups[0]][1]
    for attr in ("dof", "tr", "fitted_column_indices", "n_regressors_full", "contrast_labels",
                 "ljung_box_dof", "reml_surface_params"):
        setattr(merged, attr, getattr(first, attr))
    for attr in VOXEL_SCATTER_ATTRS + ["reml_lklhd_surface"]:
        ref = next((getattr(r, attr) for _, r in per.values() if getattr(r, attr) is not None), None)
        if ref is None:
            continue
        full = torch.zeros((V,) + tuple(ref.shape[1:]), dtype=ref.dtype, device=ref.device)
        for m, r in per.values():
            v = getattr(r, attr)
            if v is not None:
                full[m.to(full.device)] = v
        setattr(merged, attr, full)
    return merged


def fit_glm_arma11_perhrf(data, designs_by_hrf: dict, hrf_indices, tr: float, **fit_kwargs) -> ARMA11Results:
    """Per-voxel HRF REML (fastfuncstuff/glm/arma.py:3186-3204)."""
    return fit_glm_arma11_grouped(data, designs_by_hrf, hrf_indices, tr, group_label="HRF", **fit_kwargs)
