"""Device-side orchestration of the REML kernels (libffs_reml.so).

Every function here works on CUDA tensors, allocates its outputs through
torch's caching allocator, and launches the library's kernels on torch's
current stream. Nothing synchronises the device and nothing leaves the GPU, so
a whole fit can be captured in a CUDA graph (see ``RemlPlan``).

Layouts (V voxels, T time points, K design columns, P pairs):
  Y        [V][T] fp32 voxel-major data
  yr_t     [T][V] fp32 residualised, scaled data (time-major, for the O(T)
           recurrences)
  yr_hi/lo [V][ld] fp16 bits of the same, scaled by 2^yexp[v] (the projection
           GEMM's A operand)
  U_hi/lo  [P*K][ld] fp16 bits of U = L^-T Q scaled by 2^uexp[p] (its B operand)
  proj     [P][V], surf [P][V]
"""

from __future__ import annotations

import copy
import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from .. import _lib
from .grid import RemlGrid, RunLayout

LD_ALIGN = 64  # k extent of one tcgen05 pipeline stage


def _p(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


# kernels each library entry point launches (for launch accounting)
LAUNCHES = {"ffs_grid_build": 1, "ffs_grid_build_designs": 1, "ffs_reml_prep": 1, "ffs_reml_project_tc": 1, "ffs_reml_project_simt": 1,
            "ffs_reml_surface": 1, "ffs_reml_select": 1, "ffs_reml_group": 3, "ffs_reml_gls": 1,
            "ffs_reml_gls_ex": 1, "ffs_reml_gls_grouped": 2, "ffs_reml_gather": 1, "ffs_reml_window_items": 2,
            "ffs_reml_window": 1, "ffs_reml_project_tc_list": 1, "ffs_mlp_forward": 1, "ffs_reml_centers": 1,
            "ffs_design_basis": 2, "ffs_reml_strip": 1, "ffs_reml_near_line": 1, "ffs_reml_window_finish": 1,
            "ffs_reml_compact": 1, "ffs_merge_rows": 1, "ffs_reml_segment_items": 2,
            "ffs_reml_band_sums": 1}


class StageTimer:
    """Records a CUDA event pair around every library call on the current stream.

    ``launches`` counts this library's kernel launches; ``summary()`` returns,
    per entry point, its number of calls and mean device time in ms (call it
    after synchronising).
    """

    def __init__(self):
        self.events: list[tuple[str, torch.cuda.Event, torch.cuda.Event]] = []
        self.launches = 0

    def summary(self) -> dict:
        out: dict = {}
        for name, e0, e1 in self.events:
            d = out.setdefault(name, [0, 0.0])
            d[0] += 1
            d[1] += e0.elapsed_time(e1)
        return {k: {"calls": n, "mean_ms": t / n} for k, (n, t) in out.items()}


_TIMER: StageTimer | None = None


def set_stage_timer(timer: StageTimer | None) -> None:
    global _TIMER
    _TIMER = timer


def stage_timer_active() -> bool:
    return _TIMER is not None


def _run(name: str, fn, *args, launches: int | None = None) -> None:
    t = _TIMER
    if t is None or torch.cuda.is_current_stream_capturing():
        _lib.check(fn(*args), name)
        return
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    _lib.check(fn(*args), name)
    e1.record()
    t.events.append((name, e0, e1))
    t.launches += LAUNCHES.get(name, 1) if launches is None else launches


_CONST_CACHE: dict = {}


def const_dev(arr: np.ndarray, dev) -> torch.Tensor:
    """Read-only device copy of a small host array, cached by content.

    A blocking host->device copy synchronises the stream; constants that the
    same fit (or the next) needs again are copied once instead.
    """
    arr = np.ascontiguousarray(arr)
    key = (str(dev), arr.dtype.str, arr.shape, arr.tobytes())
    t = _CONST_CACHE.get(key)
    if t is None:
        if len(_CONST_CACHE) > 512:
            _CONST_CACHE.clear()
        t = torch.from_numpy(arr.copy()).to(dev)
        _CONST_CACHE[key] = t
    return t


def ld_t(T: int) -> int:
    """Row stride of the library's K x T matrices (U, G, Q0, Xt): T rounded up
    to a multiple of 4 (16-byte rows); the padding samples are zero."""
    return (T + 3) & ~3


def padded_design_t(X: torch.Tensor) -> torch.Tensor:
    """X' as [K][ld_t(T)] fp32 with zero padding (the GLS's design operand)."""
    T, K = X.shape
    Xt = torch.zeros(K, ld_t(T), device=X.device, dtype=torch.float32)
    Xt[:, :T] = X.to(torch.float32).t()
    return Xt


_TUNED: dict = {}


def autotune_projection(T: int, K: int, P: int, dev, V: int = 65536, reps: int = 3) -> dict:
    """Choose the tcgen05 projection's tile shape for this (T, K, P) by timing.

    The candidates are the B tiles of 256, 128 and 64 MMA columns (256 // K,
    128 // K, 64 // K pairs per tile); each runs the grid-mode projection of V
    synthetic voxels against P synthetic pairs (fp16 operands of the real
    shapes) ``reps`` times after one warm-up, timed with CUDA events, and the
    fastest is set through ``ffs_reml_tune_tc_pairs`` (process-wide, per K).
    The choice changes no result, only the speed; it is made once per shape
    and device and cached. Returns {"pairs": best, "ms": {pairs: time}}."""
    key = (T, K, P, str(dev))
    lib = _lib.load()
    if key in _TUNED:  # the table is per K: restore this shape's choice
        _lib.check(lib.ffs_reml_tune_tc_pairs(K, _TUNED[key]["pairs"]), "ffs_reml_tune_tc_pairs")
        return _TUNED[key]
    cands = sorted({n // K for n in (256, 128, 64) if n // K >= 1}, reverse=True)
    if len(cands) == 1 or P <= 1:
        _lib.check(lib.ffs_reml_tune_tc_pairs(K, cands[0]), "ffs_reml_tune_tc_pairs")
        _TUNED[key] = {"pairs": cands[0], "ms": {}}
        return _TUNED[key]
    ld = padded_ld(T)
    gen = torch.Generator(device=dev).manual_seed(1)
    f16 = dict(device=dev, dtype=torch.float16)
    y_hi = torch.randn(V, ld, generator=gen, **f16).view(torch.int16)
    y_lo = (torch.randn(V, ld, generator=gen, **f16) * 1e-3).view(torch.int16)
    u_hi = torch.randn(P * K, ld, generator=gen, **f16).view(torch.int16)
    u_lo = (torch.randn(P * K, ld, generator=gen, **f16) * 1e-3).view(torch.int16)
    yexp = torch.zeros(V, dtype=torch.int32, device=dev)
    uexp = torch.zeros(P, dtype=torch.int32, device=dev)
    proj = torch.empty(P, V, dtype=torch.float32, device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    ja = _lib.ProjectArgs(V=V, T=T, K=K, P=P, ld_y=ld, ld_u=ld, yr_hi=_p(y_hi), yr_lo=_p(y_lo), u_hi=_p(u_hi),
                          u_lo=_p(u_lo), yexp=_p(yexp), uexp=_p(uexp), yr_t=None, U=None, proj=_p(proj),
                          flag=_p(flag))
    st = _stream()
    times = {}
    for g in cands:
        _lib.check(lib.ffs_reml_tune_tc_pairs(K, g), "ffs_reml_tune_tc_pairs")
        _lib.check(lib.ffs_reml_project_tc(C.byref(ja), st), "ffs_reml_project_tc")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            _lib.check(lib.ffs_reml_project_tc(C.byref(ja), st), "ffs_reml_project_tc")
        e1.record()
        e1.synchronize()
        times[g] = e0.elapsed_time(e1) / reps
    if int(flag.item()) != 0:
        raise RuntimeError("ffs_reml_project_tc: a bounded wait expired during autotuning")
    best = min(times, key=times.get)
    _lib.check(lib.ffs_reml_tune_tc_pairs(K, best), "ffs_reml_tune_tc_pairs")
    _TUNED[key] = {"pairs": best, "ms": times}
    return _TUNED[key]


def padded_ld(T: int) -> int:
    return (T + LD_ALIGN - 1) // LD_ALIGN * LD_ALIGN


def require_cuda(device) -> torch.device:
    device = torch.device(device) if device is not None else torch.device("cuda")
    if device.type != "cuda":
        raise ValueError(f"fastfuncstuff_gb300 runs on a CUDA device only (got {device})")
    if not torch.cuda.is_available():
        raise RuntimeError("fastfuncstuff_gb300 needs a CUDA GPU; none is available")
    _lib.load()
    return device


@dataclass
class GridFactors:
    """Per-pair FP64-derived factors written by ``ffs_grid_build``."""

    grid: RemlGrid
    T: int
    K: int
    ld: int
    coef: torch.Tensor
    logdet_R: torch.Tensor
    logdet_XtX: torch.Tensor
    U: torch.Tensor
    U_hi: torch.Tensor | None
    U_lo: torch.Tensor | None
    G: torch.Tensor
    Adiag: torch.Tensor
    XtX: torch.Tensor
    info: torch.Tensor
    Ftask: torch.Tensor | None
    glt_var: torch.Tensor | None
    a: torch.Tensor
    b: torch.Tensor
    chunk_start: torch.Tensor
    chunk_pairs: torch.Tensor
    lattice: torch.Tensor
    task_idx: torch.Tensor | None
    glt: torch.Tensor | None
    Gsum: torch.Tensor | None = None
    center_flag: torch.Tensor | None = None  # device int32[1]: centre the voxels (constant in span(X))
    uexp: torch.Tensor | None = None
    n_designs: int = 1  # > 1: design-dependent factors are [n_designs * P] (design-major)
    Fsets: torch.Tensor | None = None  # [n_designs * P][msum] column-set blocks
    sets: "ColumnSets | None" = None
    Afull: torch.Tensor | None = None  # [n_designs * P][K][K] (X_w'X_w)^-1
    band: torch.Tensor | None = None  # AFNI-faithful banded R: int32 [P] band of each pair
    band_w: int = 0                   # row stride of band_L / band_coef (max band + 1)
    band_L: torch.Tensor | None = None  # [P][T][band_w] FP64 Cholesky rows of the banded R
    band_coef: torch.Tensor | None = None  # [P][T][band_w] fp32 whitening coefficients

    @property
    def P(self) -> int:
        return self.grid.P


def constant_flag(X: torch.Tensor, tol: float = 1e-6) -> tuple[torch.Tensor, torch.Tensor]:
    """On X's device, without a host round trip: (flag int32[1], c float32[K])
    with flag = 1 and X c = 1 (FP64 normal equations) when the constant series
    lies in the column span of X, flag = 0 and c = 0 otherwise."""
    Xd = X.detach().to(torch.float64)
    if Xd.ndim == 3:  # D designs: one flag (the constant in every span), c [D][K]
        oks, cs = zip(*(constant_flag(x, tol) for x in Xd))
        return torch.stack(oks).amin(0), torch.stack(cs)
    T, K = Xd.shape
    ones = torch.ones(T, 1, dtype=torch.float64, device=Xd.device)
    L, info = torch.linalg.cholesky_ex(Xd.T @ Xd)
    c = torch.cholesky_solve(Xd.T @ ones, L)
    res = torch.linalg.vector_norm(Xd @ c - ones)
    ok = (info == 0) & (res <= tol * math.sqrt(T))  # a failed factorisation gives NaN: not ok
    c = torch.where(ok, c.reshape(-1), torch.zeros(K, dtype=torch.float64, device=Xd.device))
    return ok.to(torch.int32).reshape(1), c.to(torch.float32)


def constant_coefficients(X: np.ndarray, tol: float = 1e-6) -> np.ndarray | None:
    """c with X c = 1 (FP64 least squares) when the constant series lies in the
    column span of X, else None."""
    Xd = np.asarray(X, dtype=np.float64)
    ones = np.ones(Xd.shape[0])
    coef, *_ = np.linalg.lstsq(Xd, ones, rcond=None)
    if float(np.linalg.norm(Xd @ coef - ones)) <= tol * np.sqrt(Xd.shape[0]):
        return coef
    return None


def constant_in_span(X: np.ndarray, tol: float = 1e-6) -> bool:
    """True when the constant series lies in the column span of X (FP64 least squares)."""
    return constant_coefficients(X, tol) is not None


@dataclass
class ColumnSets:
    """The column sets of a fit (the reference's ``column_sets``) laid out for
    the kernels: the sets whose columns all lie in the design, as offsets
    (set_ptr) into one index list (set_idx), each with its output column
    (set_col); the other sets' statistics stay NaN. ``C`` [n_designs][msum]
    holds each set's Xc_S' Xc_S / T (Xc the column-centred design) block."""

    n_out: int
    set_ptr: np.ndarray
    set_idx: np.ndarray
    set_col: np.ndarray
    C: np.ndarray

    @property
    def n_sets(self) -> int:
        return len(self.set_col)

    @property
    def msum(self) -> int:
        q = np.diff(self.set_ptr)
        return int((q * q).sum())

    def key(self) -> bytes:
        return b"|".join(a.tobytes() for a in (np.array([self.n_out]), self.set_ptr, self.set_idx, self.set_col))

    def device_arrays(self, dev):
        return const_dev(self.set_ptr.astype(np.int32), dev), const_dev(self.set_idx.astype(np.int32), dev)


def column_sets_plan(column_sets, designs) -> ColumnSets:
    """``column_sets`` (lists of column indices) against the design(s) (T, K)
    or (D, T, K), as fastfuncstuff/glm/arma.py:3542-3561 reads them: a set
    naming a column >= K (or empty) has no statistics; a negative index is an
    error."""
    Xs = np.asarray(designs, dtype=np.float64)
    if Xs.ndim == 2:
        Xs = Xs[None]
    _, T, K = Xs.shape
    ptr, idx, col = [0], [], []
    for g, cols in enumerate(column_sets):
        cols = [int(c) for c in cols]
        if any(c < 0 for c in cols):
            raise IndexError(f"column_sets[{g}] has a negative column index: {cols}")
        if not cols or any(c >= K for c in cols):
            continue
        idx.extend(cols)
        ptr.append(len(idx))
        col.append(g)
    ptr, idx = np.asarray(ptr, np.int64), np.asarray(idx, np.int64)
    blocks = []
    for X in Xs:
        Xc = X - X.mean(0, keepdims=True)
        per = [(Xc[:, idx[ptr[s]:ptr[s + 1]]].T @ Xc[:, idx[ptr[s]:ptr[s + 1]]] / T).reshape(-1)
               for s in range(len(col))]
        blocks.append(np.concatenate(per) if per else np.zeros(0))
    return ColumnSets(n_out=len(column_sets), set_ptr=ptr, set_idx=idx, set_col=np.asarray(col, np.int64),
                      C=np.stack(blocks).astype(np.float32))


def set_stats(betas: torch.Tensor, sigma2: torch.Tensor, scale: torch.Tensor, best: torch.Tensor,
              f: GridFactors, design: torch.Tensor | None = None):
    """(set_fstats, set_sd, set_coef) [V][n_out] of the fitted voxels (betas
    [V][K] of every column and sigma2 as ``gls`` returns them, unscaled; best
    the pair of each voxel; ``design`` each voxel's design in a grouped fit).
    NaN where a set names a column outside the design."""
    cs = f.sets
    V = betas.shape[0]
    dev = betas.device
    out = [torch.full((V, cs.n_out), float("nan"), device=dev, dtype=torch.float32) for _ in range(3)]
    if cs.n_sets == 0 or V == 0:
        return tuple(out)
    lib = _lib.load()
    ptr, idx = cs.device_arrays(dev)
    col = const_dev(cs.set_col.astype(np.int32), dev)
    Cd = const_dev(cs.C, dev)
    bst = best.to(device=dev, dtype=torch.int32).contiguous()
    dsg = design.to(device=dev, dtype=torch.int32).contiguous() if design is not None else None
    b = betas.to(torch.float32).contiguous()
    s2 = sigma2.to(torch.float32).contiguous()
    sc = scale.to(torch.float32).contiguous()
    a = _lib.SetStatsArgs(V=V, K=b.shape[1], n_sets=cs.n_sets, n_out=cs.n_out, set_ptr=_p(ptr), set_idx=_p(idx),
                          set_col=_p(col), msum=cs.msum, Fsets=_p(f.Fsets), Csets=_p(Cd), best=_p(bst),
                          design=_p(dsg), n_pairs=f.P if dsg is not None else 0, betas=_p(b), sigma2=_p(s2),
                          scale=_p(sc), set_fstats=_p(out[0]), set_sd=_p(out[1]), set_coef=_p(out[2]))
    _run("ffs_reml_set_stats", lib.ffs_reml_set_stats, C.byref(a), _stream())
    out[0]._keep = (ptr, idx, col, Cd, bst, dsg, b, s2, sc)
    return tuple(out)


def build_factors(X: torch.Tensor, grid: RemlGrid, layout: RunLayout, *, task_indices=None,
                  glt: np.ndarray | None = None, with_tc: bool = True, center=None,
                  stream: torch.cuda.Stream | None = None, max_ctas: int = 0,
                  sets: ColumnSets | None = None, afull: bool = False) -> GridFactors:
    """Run the FP64 grid build for design ``X`` (T, K) on its device.

    ``sets`` (``column_sets_plan``) adds each column set's inv(A_SS + 1e-8 I)
    per pair (``Fsets``) for ``set_stats``; ``afull`` all of (X_w'X_w)^-1
    (``Afull``, for the column sets of a -dsort fit).

    ``center`` = (flag, coefficients) from ``constant_flag(X)`` when the caller
    has them already (the CUDA-graph plan computes them outside its capture).
    With ``stream`` the grid build runs there (the buffers are allocated on the
    current stream, which must wait for ``stream`` before it reads them);
    ``max_ctas`` > 0 caps its CTAs (the rest of the GPU stays free for work
    beside it).

    lambda is always evaluated in float64 from the float32 (a, b) values (the
    FP64 fit's value); the fit's mode only decides the validity filter and the
    reported per-voxel lambda.
    """
    dev = X.device
    D = X.shape[0] if X.ndim == 3 else 1  # (D, T, K): one design per voxel group
    T, K = X.shape[-2:]
    P = grid.P
    ld = padded_ld(T)
    f32 = dict(device=dev, dtype=torch.float32)
    Xc = X.to(**f32).contiguous()
    a = const_dev(grid.a, dev)
    b = const_dev(grid.b, dev)
    run_start = const_dev(layout.run_start, dev)
    tau = const_dev(layout.tau, dev)
    task_idx = None
    if task_indices is not None and len(task_indices) > 0:
        task_idx = const_dev(np.asarray(list(task_indices), np.int32), dev)
    glt_t = None if glt is None else const_dev(np.asarray(glt, np.float32).reshape(-1, K), dev)
    nt = 0 if task_idx is None else task_idx.numel()
    ng = 0 if glt_t is None else glt_t.shape[0]
    lib = _lib.load()
    cflag, ccoef = constant_flag(Xc) if center is None else center
    single = D == 1 and max_ctas <= 0  # else the designs entry point, which takes a CTA cap
    wbytes = lib.ffs_grid_work_bytes(T, K, P) if single else lib.ffs_grid_work_bytes_designs(T, K, P, D, max_ctas)
    work = torch.empty(int(wbytes) // 8 + 1, dtype=torch.float64, device=dev)
    DP = D * P
    f = GridFactors(
        grid=grid, T=T, K=K, ld=ld,
        coef=torch.empty(P, T, 4, **f32),
        logdet_R=torch.empty(P, dtype=torch.float64, device=dev),
        logdet_XtX=torch.empty(DP, dtype=torch.float64, device=dev),
        U=torch.empty(DP, K, ld_t(T), **f32),
        U_hi=torch.empty(DP * K, ld, dtype=torch.int16, device=dev) if with_tc else None,
        U_lo=torch.empty(DP * K, ld, dtype=torch.int16, device=dev) if with_tc else None,
        G=torch.empty(DP, K, ld_t(T), **f32),
        Adiag=torch.empty(DP, K, **f32),
        XtX=torch.empty(DP, K, K, **f32),
        info=torch.empty(DP, dtype=torch.int32, device=dev),
        Ftask=torch.empty(DP, nt, nt, **f32) if nt else None,
        glt_var=torch.empty(DP, ng, **f32) if ng else None,
        a=a, b=b,
        chunk_start=const_dev(grid.chunk_start, dev),
        chunk_pairs=const_dev(grid.chunk_pairs, dev),
        lattice=const_dev(grid.lattice.reshape(-1), dev),
        task_idx=task_idx, glt=glt_t,
        Gsum=None,
        center_flag=cflag,
        uexp=torch.empty(DP, dtype=torch.int32, device=dev) if with_tc else None,
        n_designs=D,
    )
    if afull:
        f.Afull = torch.empty(DP, K, K, **f32)
    if grid.band is not None:
        # AFNI-faithful mode: R banded per pair, factored as a band (once per
        # pair for every design)
        f.band_w = int(grid.band.max()) + 1
        if f.band_w > _lib.FFS_BAND_MAX_W:
            raise NotImplementedError(f"the AFNI-faithful band of {f.band_w - 1} lags exceeds "
                                      f"{_lib.FFS_BAND_MAX_W - 1} (a grid with |a| near 1 or a small corcut)")
        f.band = const_dev(grid.band, dev)
        f.band_L = torch.empty(P, T, f.band_w, dtype=torch.float64, device=dev)
        f.band_coef = torch.empty(P, T, f.band_w, **f32)
    if sets is not None and sets.n_sets:
        f.sets = sets
        f.Fsets = torch.empty(DP, sets.msum, **f32)
        sets_dev = sets.device_arrays(dev)
    else:
        sets_dev = (None, None)
    d = _lib.GridDesc(T=T, K=K, P=P, n_runs=layout.n_runs, run_start=_p(run_start), tau=_p(tau),
                      a=_p(a), b=_p(b), X=_p(Xc), lambda_fp32=0, ld_u=ld,
                      n_task=nt, task_idx=_p(task_idx), n_glt=ng, glt=_p(glt_t),
                      n_sets=sets.n_sets if f.Fsets is not None else 0, set_ptr=_p(sets_dev[0]),
                      set_idx=_p(sets_dev[1]), band_w=f.band_w, band=_p(f.band))
    # no Gsum from the kernel: G'1 is the FP64 coefficient vector of the constant (set below)
    o = _lib.GridOut(coef=_p(f.coef), logdet_R=_p(f.logdet_R), logdet_XtX=_p(f.logdet_XtX), U=_p(f.U),
                     U_hi=_p(f.U_hi), U_lo=_p(f.U_lo), uexp=_p(f.uexp), G=_p(f.G), Adiag=_p(f.Adiag), XtX=_p(f.XtX),
                     info=_p(f.info), Ftask=_p(f.Ftask), glt_var=_p(f.glt_var), Gsum=None, work=_p(work),
                     Fsets=_p(f.Fsets), Afull=_p(f.Afull), band_L=_p(f.band_L), band_coef=_p(f.band_coef))
    def launch():
        if single:
            _run("ffs_grid_build", lib.ffs_grid_build, C.byref(d), C.byref(o), _stream())
        else:
            # more than one design: a pre-pass factors R once per pair
            _run("ffs_grid_build_designs", lib.ffs_grid_build_designs, C.byref(d), D, max_ctas, C.byref(o),
                 _stream(), launches=2 if D > 1 else 1)

    if stream is None:
        launch()
    else:
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(stream):
            launch()
    # G' X = I for every pair, so G'1 = c exactly when the constant is in
    # span(X): the centring correction of the GLS uses the FP64 coefficients
    # rather than sums of the fp32 G (the flag decides on the device)
    f.Gsum = ccoef.reshape(D, 1, K).expand(D, P, K).reshape(DP, K).contiguous()
    f._keep = (Xc, run_start, tau, work, sets_dev)  # inputs must outlive the launch
    return f


def design_view(f: GridFactors, d: int, center_flag: torch.Tensor | None = None) -> GridFactors:
    """The factors of design d of a multi-design build as a single-design
    GridFactors (views into the build's buffers, no copy): what a fit of that
    design's voxels alone reads. ``center_flag`` (constant_flag of the
    design) replaces the build's flag, which holds for every design at once."""
    if f.n_designs == 1:
        return f
    P, K = f.P, f.K
    sl = slice(d * P, (d + 1) * P)
    v = copy.copy(f)
    v.n_designs = 1
    for name in ("logdet_XtX", "U", "G", "Adiag", "XtX", "info", "Ftask", "glt_var", "Gsum", "uexp", "Fsets",
                 "Afull"):
        t = getattr(f, name)
        setattr(v, name, None if t is None else t[sl])
    for name in ("U_hi", "U_lo"):
        t = getattr(f, name)
        setattr(v, name, None if t is None else t[d * P * K:(d + 1) * P * K])
    if center_flag is not None:
        v.center_flag = center_flag
    v.__dict__.pop("_window_consts", None)  # per-design constants of the learned refine
    return v


@dataclass
class SearchOut:
    best: torch.Tensor        # [V] int32 pair index
    best_crit: torch.Tensor   # [V] float32 criterion (scaled-data likelihood)
    scale: torch.Tensor       # [V] float32 per-voxel std
    surf: torch.Tensor | None = None   # [P][V] criterion relative to (0,0)
    crit0: torch.Tensor | None = None  # [V] float64 criterion at (0,0)
    yr_t: torch.Tensor | None = None   # [T][V] residualised, scaled data


@dataclass
class PrepOut:
    scale: torch.Tensor
    yr_t: torch.Tensor
    yr_hi: torch.Tensor | None
    yr_lo: torch.Tensor | None
    yexp: torch.Tensor | None


# the one-CTA design basis pays off (beside the grid build) for small designs;
# wider ones take Q0 from the grid build (U of the pair (0, 0))
BASIS_MAX_K = 32


def _view(ptr, t):
    return None if t is None else ptr(t)


def device_view(t: torch.Tensor) -> int | None:
    """The device address of t's data -- device memory, or pinned host
    memory mapped into the device's address space -- or None when kernels may
    not read it in place (pageable host memory)."""
    if t.is_cuda:
        return t.data_ptr()
    if not t.is_pinned():
        return None
    out = C.c_void_p()
    if _lib.load().ffs_device_view(C.c_void_p(t.data_ptr()), C.byref(out)) != _lib.FFS_OK:
        return None
    return out.value


def design_basis(X: torch.Tensor, with_constant: bool = False):
    """Q0 [K][ld_t(T)]: the orthonormal basis of the design's columns (FP64 Cholesky),
    from X alone, so the residualisation need not wait for the grid build.

    ``with_constant`` also returns the centring test of ``constant_flag``
    (flag int32[1], c float32[K]) from the same kernel: (q0, flag, c)."""
    lib = _lib.load()
    dev = X.device
    T, K = X.shape
    Xc = X.to(torch.float32).contiguous()
    work = torch.empty(int(lib.ffs_design_basis_work_bytes(T, K)) // 8 + 1, dtype=torch.float64, device=dev)
    q0 = torch.empty(K, ld_t(T), dtype=torch.float32, device=dev)
    info = torch.empty(1, dtype=torch.int32, device=dev)
    flag = torch.empty(1, dtype=torch.int32, device=dev) if with_constant else None
    coef = torch.empty(K, dtype=torch.float32, device=dev) if with_constant else None
    _run("ffs_design_basis", lib.ffs_design_basis, T, K, _p(Xc), _p(work), _p(q0), _p(info), _p(flag), _p(coef),
         _stream())
    q0._keep = (Xc, work, info)
    return (q0, flag, coef) if with_constant else q0


def prep(Y: torch.Tensor, f: GridFactors, *, do_scale: bool = True, tensor_core: bool = True,
         idx: torch.Tensor | None = None, want_yr_t: bool = True, layout: RunLayout | None = None,
         scale: torch.Tensor | None = None, want_rows: bool = False, q0: torch.Tensor | None = None,
         split: bool = True, y_ref: torch.Tensor | None = None, y_copy: torch.Tensor | None = None,
         out: PrepOut | None = None) -> PrepOut:
    """Per-voxel scaling and residualisation (and the fp16 split for the GEMM).

    With ``tensor_core`` and ``split=False`` only the split's exponents
    (``yexp``) are formed: a caller that gathers a subset of the rows splits
    them from ``rows`` while gathering (``ffs_reml_gather``).

    ``idx`` (int32, device) processes the rows Y[idx] in that order (every
    output but ``scale`` is indexed by position in ``idx``; ``scale`` by the
    row of Y, into ``scale`` when given). With ``layout`` the lag 1..8
    autocorrelation features of the residualised rows are returned in
    ``PrepOut.feats``; ``want_rows`` adds the residualised rows voxel-major
    (``PrepOut.rows``).

    ``y_ref`` (int64 [1] on the device) holds the address the rows are read
    from instead of Y's -- device memory or pinned host memory mapped into
    the device's address space (``device_view``) -- and ``y_copy`` ([V][T])
    receives the rows as read; Y then only gives the shape.

    ``out`` gives the buffers to write (its scale, yexp, feats and rows, of
    the rows processed; e.g. views of a larger prep's outputs) instead of new
    ones; the formed outputs it lacks are allocated.
    """
    lib = _lib.load()
    dev = Y.device
    V, T = Y.shape
    n = V if idx is None else idx.numel()
    K, ld = f.K, f.ld
    if y_ref is None:
        Y = Y.to(dtype=torch.float32).contiguous()
    given = {} if out is None else {k: getattr(out, k, None) for k in ("scale", "yexp", "feats", "rows")}
    if scale is None:
        scale = given.get("scale")
    if scale is None:
        scale = torch.empty(V, dtype=torch.float32, device=dev)
    yr_t = torch.empty(T, n, dtype=torch.float32, device=dev) if want_yr_t else None
    yr_hi = torch.empty(n, ld, dtype=torch.int16, device=dev) if tensor_core and split else None
    yr_lo = torch.empty(n, ld, dtype=torch.int16, device=dev) if tensor_core and split else None
    yexp = None
    if tensor_core:
        yexp = given.get("yexp")
        if yexp is None:
            yexp = torch.empty(n, dtype=torch.int32, device=dev)
    feats = rs = None
    if layout is not None:
        feats = given.get("feats")
        if feats is None:
            feats = torch.empty(n, 9, dtype=torch.float32, device=dev)
        rs = const_dev(layout.run_start, dev)
    rows = None
    if want_rows:
        rows = given.get("rows")
        if rows is None:
            rows = torch.empty(n, T, dtype=torch.float32, device=dev)
    if q0 is None:
        q0 = f.U[f.grid.p0]  # orthonormal basis of the design columns ([K][T]): U of (0, 0)
    pa = _lib.PrepArgs(V=n, T=T, K=K, Y=_p(Y), Q0=_p(q0), do_scale=int(do_scale), center=0, ld_y=ld,
                       scale=_p(scale), yr_t=_p(yr_t), yr_hi=_p(yr_hi), yr_lo=_p(yr_lo), yexp=_p(yexp),
                       idx=_p(idx), feats=_p(feats), n_runs=0 if layout is None else layout.n_runs,
                       run_start=_p(rs), yr_rows=_p(rows), center_dev=_p(f.center_flag),
                       Y_ref=_p(y_ref), Y_copy=_p(y_copy))
    if y_ref is not None:
        pa.Y = None
    _run("ffs_reml_prep", lib.ffs_reml_prep, C.byref(pa), _stream())
    out = PrepOut(scale, yr_t, yr_hi, yr_lo, yexp)
    out.feats = feats
    out.rows = rows
    out._keep = rs
    return out


def search(Y: torch.Tensor, f: GridFactors, *, hierarchical: bool = True, projector: str = "tc",
           do_scale: bool = True, keep_surface: bool = False, keep_yr: bool = False,
           q0: torch.Tensor | None = None, join=None) -> SearchOut:
    """REML grid search of every voxel of ``Y`` (V, T) against the factors ``f``.

    ``projector`` picks the projection kernel: "tc" (tcgen05 fp16-split GEMM) or
    "simt" (fp32 CUDA cores).
    """
    lib = _lib.load()
    dev = Y.device
    V, T = Y.shape
    K, P, ld = f.K, f.P, f.ld
    st = _stream()
    use_tc = projector == "tc"
    if use_tc and f.U_hi is None:
        raise ValueError("the factors were built without the tensor-core operands")
    if projector not in ("tc", "simt"):
        raise ValueError(f"unknown projector {projector!r}")
    pr = prep(Y, f, do_scale=do_scale, tensor_core=use_tc, q0=q0)
    if join is not None:  # the factors may still be in flight on another stream
        join()

    proj = torch.empty(P, V, dtype=torch.float32, device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    if use_tc and not torch.cuda.is_current_stream_capturing():
        autotune_projection(T, K, P, dev)
    ja = _lib.ProjectArgs(V=V, T=T, K=K, P=P, ld_y=ld, ld_u=ld, yr_hi=_p(pr.yr_hi), yr_lo=_p(pr.yr_lo),
                          u_hi=_p(f.U_hi), u_lo=_p(f.U_lo), yexp=_p(pr.yexp), uexp=_p(f.uexp),
                          yr_t=_p(pr.yr_t), U=_p(f.U), proj=_p(proj), flag=_p(flag))
    if use_tc:
        _run("ffs_reml_project_tc", lib.ffs_reml_project_tc, C.byref(ja), st)
    else:
        _run("ffs_reml_project_simt", lib.ffs_reml_project_simt, C.byref(ja), st)

    surf = torch.empty(P, V, dtype=torch.float32, device=dev)
    crit0 = torch.empty(V, dtype=torch.float64, device=dev)
    sa = _lib.SurfaceArgs(V=V, T=T, K=K, P=P, p0=f.grid.p0, yr_t=_p(pr.yr_t), coef=_p(f.coef),
                          logdet_R=_p(f.logdet_R), logdet_XtX=_p(f.logdet_XtX), proj=_p(proj),
                          chunk_start=_p(f.chunk_start), n_chunks=f.chunk_start.numel() - 1,
                          chunk_pairs=_p(f.chunk_pairs), surf=_p(surf), crit0=_p(crit0),
                          band_coef=_p(f.band_coef), band_w=f.band_w, band=_p(f.band))
    _run("ffs_reml_surface", lib.ffs_reml_surface, C.byref(sa), st)

    best = torch.empty(V, dtype=torch.int32, device=dev)
    best_crit = torch.empty(V, dtype=torch.float32, device=dev)
    g = f.grid
    se = _lib.SelectArgs(V=V, P=P, surf=_p(surf), crit0=_p(crit0), hierarchical=int(hierarchical),
                         n_a=len(g.a_axis), n_b=len(g.b_axis), ltop=g.ltop, za=g.za, zb=g.zb,
                         lattice=_p(f.lattice), best=_p(best), best_crit=_p(best_crit))
    _run("ffs_reml_select", lib.ffs_reml_select, C.byref(se), st)
    out = SearchOut(best=best, best_crit=best_crit, scale=pr.scale)
    out._flag = flag
    if keep_surface:
        out.surf, out.crit0 = surf, crit0
    if keep_yr:
        out.yr_t = pr.yr_t
    return out


@dataclass
class DesignSlots:
    """Voxel layout of a grouped fit (one design per voxel group).

    The voxels of each design occupy a run of slots padded to a multiple of 256,
    so every 32-voxel tile of the residualisation, 128-row tile of the
    projection and 256-voxel tile of the criterion belongs to one design.
    """

    V: int                 # voxels
    Vp: int                # slots
    idx: torch.Tensor      # [Vp] int32 voxel of each slot, -1 for padding
    real: torch.Tensor     # [V] int64 slot of each voxel
    design: torch.Tensor   # [V] int32 design of each voxel
    tile32: torch.Tensor   # [Vp / 32] int32
    tile256: torch.Tensor  # [Vp / 256] int32
    items: torch.Tensor    # [n_items][6] int32 projection work list (ffs_tc_item)
    n_items: torch.Tensor  # [1] int32
    max_pairs: int


def design_slots(gid: np.ndarray, n_designs: int, K: int, P: int, dev) -> DesignSlots:
    """Slots and the (design, voxel tile, pair block) projection work list of a
    grouped fit; ``gid`` [V] holds each voxel's design index (host)."""
    gid = np.asarray(gid, dtype=np.int64).reshape(-1)
    V = gid.size
    order = np.argsort(gid, kind="stable")
    counts = np.bincount(gid, minlength=n_designs)
    padded = (counts + 255) // 256 * 256
    start = np.concatenate([[0], np.cumsum(padded)])
    first = np.concatenate([[0], np.cumsum(counts)])
    Vp = int(start[-1])
    idx = np.full(Vp, -1, np.int32)
    real = np.empty(V, np.int64)
    for d in range(n_designs):
        vox = order[first[d]:first[d + 1]]
        idx[start[d]:start[d] + counts[d]] = vox
        real[vox] = np.arange(start[d], start[d] + counts[d])
    tile_of = np.repeat(np.arange(n_designs, dtype=np.int32), padded // 32)
    g = max(1, min(P, 256 // K))
    p0 = np.arange(0, P, g, dtype=np.int64)
    npair = np.minimum(g, P - p0)
    rows = []
    for d in range(n_designs):  # design-major, then voxel tile, then pair block
        v0 = np.arange(int(start[d]), int(start[d + 1]), 128, dtype=np.int64)
        vv, pp = np.meshgrid(v0, p0, indexing="ij")
        nn = np.broadcast_to(npair, vv.shape)
        rows.append(np.stack([vv, np.full_like(vv, 128), (d * P + pp) * K, nn, vv, pp], -1).reshape(-1, 6))
    items = np.concatenate(rows).astype(np.int32) if rows else np.zeros((0, 6), np.int32)
    return DesignSlots(V=V, Vp=Vp, idx=torch.from_numpy(idx).to(dev), real=torch.from_numpy(real).to(dev),
                       design=torch.from_numpy(gid.astype(np.int32)).to(dev),
                       tile32=torch.from_numpy(tile_of).to(dev),
                       tile256=torch.from_numpy(tile_of[::8].copy()).to(dev),
                       items=torch.from_numpy(items).to(dev),
                       n_items=torch.tensor([items.shape[0]], dtype=torch.int32, device=dev), max_pairs=g)


def search_designs(Y: torch.Tensor, f: GridFactors, slots: DesignSlots, *, hierarchical: bool = True,
                   do_scale: bool = True) -> SearchOut:
    """Full-grid REML search of a grouped fit: every voxel against its group's
    design, all designs in one launch per stage (residualisation, tcgen05
    projection work list, criterion, selection)."""
    lib = _lib.load()
    dev = Y.device
    V, T = Y.shape
    K, P, ld, D = f.K, f.P, f.ld, f.n_designs
    if f.U_hi is None:
        raise ValueError("the factors were built without the tensor-core operands")
    st = _stream()
    Vp = slots.Vp
    Y = Y.to(dtype=torch.float32).contiguous()
    q0 = f.U.view(D, P, K, -1)[:, f.grid.p0].contiguous()  # [D][K][ld_t]: U of (0, 0) per design
    scale = torch.empty(V, dtype=torch.float32, device=dev)
    yr_t = torch.empty(T, Vp, dtype=torch.float32, device=dev)
    yr_hi = torch.empty(Vp, ld, dtype=torch.int16, device=dev)
    yr_lo = torch.empty(Vp, ld, dtype=torch.int16, device=dev)
    yexp = torch.empty(Vp, dtype=torch.int32, device=dev)
    pa = _lib.PrepArgs(V=Vp, T=T, K=K, Y=_p(Y), Q0=_p(q0), do_scale=int(do_scale), center=0, ld_y=ld,
                       scale=_p(scale), yr_t=_p(yr_t), yr_hi=_p(yr_hi), yr_lo=_p(yr_lo), yexp=_p(yexp),
                       idx=_p(slots.idx), feats=None, n_runs=0, run_start=None, yr_rows=None,
                       center_dev=_p(f.center_flag), tile_design=_p(slots.tile32))
    _run("ffs_reml_prep", lib.ffs_reml_prep, C.byref(pa), st)

    proj = torch.empty(P, Vp, dtype=torch.float32, device=dev)
    flag = torch.zeros(1, dtype=torch.int32, device=dev)
    ja = _lib.ProjectArgs(V=Vp, T=T, K=K, P=D * P, ld_y=ld, ld_u=ld, yr_hi=_p(yr_hi), yr_lo=_p(yr_lo),
                          u_hi=_p(f.U_hi), u_lo=_p(f.U_lo), yexp=_p(yexp), uexp=_p(f.uexp), yr_t=None, U=None,
                          proj=_p(proj), flag=_p(flag))
    n_items = slots.items.shape[0]
    _run("ffs_reml_project_tc_list", lib.ffs_reml_project_tc_list, C.byref(ja), _p(slots.items), _p(slots.n_items),
         n_items, slots.max_pairs, 0, st)

    surf = torch.empty(P, Vp, dtype=torch.float32, device=dev)
    crit0 = torch.empty(Vp, dtype=torch.float64, device=dev)
    sa = _lib.SurfaceArgs(V=Vp, T=T, K=K, P=P, p0=f.grid.p0, yr_t=_p(yr_t), coef=_p(f.coef),
                          logdet_R=_p(f.logdet_R), logdet_XtX=_p(f.logdet_XtX), proj=_p(proj),
                          chunk_start=_p(f.chunk_start), n_chunks=f.chunk_start.numel() - 1,
                          chunk_pairs=_p(f.chunk_pairs), surf=_p(surf), crit0=_p(crit0),
                          tile_design=_p(slots.tile256), band_coef=_p(f.band_coef), band_w=f.band_w,
                          band=_p(f.band))
    _run("ffs_reml_surface", lib.ffs_reml_surface, C.byref(sa), st)

    best = torch.empty(Vp, dtype=torch.int32, device=dev)
    best_crit = torch.empty(Vp, dtype=torch.float32, device=dev)
    g = f.grid
    se = _lib.SelectArgs(V=Vp, P=P, surf=_p(surf), crit0=_p(crit0), hierarchical=int(hierarchical),
                         n_a=len(g.a_axis), n_b=len(g.b_axis), ltop=g.ltop, za=g.za, zb=g.zb,
                         lattice=_p(f.lattice), best=_p(best), best_crit=_p(best_crit))
    _run("ffs_reml_select", lib.ffs_reml_select, C.byref(se), st)
    out = SearchOut(best=best[slots.real], best_crit=best_crit[slots.real], scale=scale)
    out._flag = flag
    out._keep = (q0, yr_t, yr_hi, yr_lo, yexp, proj, surf, crit0)
    return out


@dataclass
class GlsOut:
    betas: torch.Tensor   # [V][K] (unscaled)
    tstats: torch.Tensor  # [V][K]
    sigma2: torch.Tensor
    fstats: torch.Tensor
    r2: torch.Tensor
    lam: torch.Tensor
    cbeta: torch.Tensor | None = None
    ct: torch.Tensor | None = None
    resid: torch.Tensor | None = None
    resid_w: torch.Tensor | None = None
    pred: torch.Tensor | None = None
    ljung_box: torch.Tensor | None = None


def gls(Y: torch.Tensor, scale: torch.Tensor, best: torch.Tensor, f: GridFactors, X: torch.Tensor, *,
        want_residuals: bool = False, want_predicted: bool = False, lj=None,
        design: torch.Tensor | None = None, host_out: bool = False) -> GlsOut:
    """GLS refit of every voxel at its pair ``best`` (indices into ``f``).

    Grouped fits pass X as (D, T, K) and ``design`` [V] (each voxel's design):
    voxels are then grouped by design * P + pair. With ``host_out`` the
    outputs are pinned host tensors that the kernel writes over the host link
    as it goes (valid once the stream has passed the launch)."""
    lib = _lib.load()
    dev = Y.device
    V, T = Y.shape
    K, P = f.K, f.P
    st = _stream()
    Y = Y.to(dtype=torch.float32).contiguous()
    n_pairs = 0
    if design is not None:
        best = (design.to(torch.int32) * P + best.to(torch.int32)).contiguous()
        n_pairs = P
        P = P * f.n_designs
    order = torch.empty(V, dtype=torch.int32, device=dev)
    work = torch.empty(P + 1, dtype=torch.int32, device=dev)
    _run("ffs_reml_group", lib.ffs_reml_group, V, P, _p(best), _p(work), _p(order), st)
    X = X.to(device=dev)
    Xt = padded_design_t(X) if X.ndim == 2 else torch.stack([padded_design_t(x) for x in X])
    f32 = dict(dtype=torch.float32, pin_memory=True) if host_out else dict(device=dev, dtype=torch.float32)
    ptr = device_view if host_out else _p
    ng = 0 if f.glt is None else f.glt.shape[0]
    o = GlsOut(betas=torch.empty(V, K, **f32), tstats=torch.empty(V, K, **f32), sigma2=torch.empty(V, **f32),
               fstats=torch.empty(V, **f32), r2=torch.empty(V, **f32), lam=torch.empty(V, **f32),
               cbeta=torch.empty(V, ng, **f32) if ng else None, ct=torch.empty(V, ng, **f32) if ng else None,
               resid=torch.empty(V, T, **f32) if want_residuals else None,
               resid_w=torch.empty(V, T, **f32) if want_residuals else None,
               pred=torch.empty(V, T, **f32) if want_predicted else None)
    nt = 0 if f.task_idx is None else f.task_idx.numel()
    ga = _lib.GlsArgs(V=V, T=T, K=K, dof=max(1, T - K), center=0, Gsum=_p(f.Gsum), Y=_p(Y),
                      scale=_p(scale), Xt=_p(Xt), best=_p(best),
                      order=_p(order), coef=_p(f.coef), G=_p(f.G), Adiag=_p(f.Adiag), XtX=_p(f.XtX),
                      a=_p(f.a), b=_p(f.b), lambda_fp32=int(f.grid.lambda_fp32), n_task=nt,
                      task_idx=_p(f.task_idx), Ftask=_p(f.Ftask), n_glt=ng, glt=_p(f.glt),
                      glt_var=_p(f.glt_var), betas=ptr(o.betas), tstats=ptr(o.tstats), sigma2=ptr(o.sigma2),
                      fstats=ptr(o.fstats), r2=ptr(o.r2), lam=ptr(o.lam), cbeta=_view(ptr, o.cbeta),
                      ct=_view(ptr, o.ct), resid=_view(ptr, o.resid), resid_w=_view(ptr, o.resid_w),
                      pred=_view(ptr, o.pred), center_dev=_p(f.center_flag), n_pairs=n_pairs,
                      band_coef=_p(f.band_coef), band_w=f.band_w, band=_p(f.band))
    h, ptau_d, w_d = 0, None, None
    if lj is not None and lj[0] > 0:
        h, ptau, w, _ = lj
        ptau_d = None if ptau is None else const_dev(ptau, dev)
        w_d = const_dev(w, dev)
        o.ljung_box = torch.empty(V, **f32)
    tiles = torch.empty(P + 1, dtype=torch.int32, device=dev)
    _run("ffs_reml_gls_grouped", lib.ffs_reml_gls_grouped, C.byref(ga), h, _p(ptau_d), _p(w_d),
         _view(ptr, o.ljung_box), P, _p(work), _p(tiles), st)
    o._keep = (ptau_d, w_d, tiles)
    o._keep2 = (Y, order, work, Xt, best)
    return o


@dataclass
class DsortOut:
    betas: torch.Tensor
    tstats: torch.Tensor
    dbetas: torch.Tensor
    dtstats: torch.Tensor
    sigma2: torch.Tensor
    fstats: torch.Tensor
    r2: torch.Tensor
    cbeta: torch.Tensor | None = None
    ct: torch.Tensor | None = None
    resid: torch.Tensor | None = None
    resid_w: torch.Tensor | None = None
    pred: torch.Tensor | None = None
    ljung_box: torch.Tensor | None = None
    set_fstats: torch.Tensor | None = None
    set_sd: torch.Tensor | None = None
    set_coef: torch.Tensor | None = None
    status: torch.Tensor | None = None


def dsort_sets_plan(column_sets, K: int, q: int):
    """(set_ptr, set_idx, set_col, n_out) of column sets over [X | D] (indices
    >= K name D columns): the sets with every index < K + q, repeats removed;
    the others stay NaN (fastfuncstuff/glm/arma.py:3461-3479)."""
    ptr, idx, col = [0], [], []
    for g, cols in enumerate(column_sets):
        cols = list(dict.fromkeys(int(c) for c in cols))
        if any(c < 0 for c in cols):
            raise IndexError(f"column_sets[{g}] has a negative column index: {cols}")
        if not cols or any(c >= K + q for c in cols):
            continue
        idx.extend(cols)
        ptr.append(len(idx))
        col.append(g)
    return np.asarray(ptr, np.int32), np.asarray(idx, np.int32), np.asarray(col, np.int32), len(column_sets)


def gls_dsort(Y: torch.Tensor, scale: torch.Tensor, best: torch.Tensor, f: GridFactors, X: torch.Tensor,
              D: torch.Tensor, *, want_residuals: bool = False, want_predicted: bool = False, lj=None,
              design: torch.Tensor | None = None, column_sets=None) -> DsortOut:
    """The -dsort GLS of every voxel with [X | D_v] at its pair (``ffs_reml_gls_dsort``).

    ``D`` (V, q, T) holds each voxel's regressors after the constant guard and
    any per-run expansion; grouped fits pass X as (D, T, K) and ``design``."""
    lib = _lib.load()
    dev = Y.device
    V, T = Y.shape
    K, P = f.K, f.P
    q = D.shape[1]
    st = _stream()
    Y = Y.to(dtype=torch.float32).contiguous()
    D = D.to(device=dev, dtype=torch.float32).contiguous()
    n_pairs = 0
    key = best.to(torch.int32)
    if design is not None:
        key = design.to(torch.int32) * P + key
        n_pairs = P
    key = key.contiguous()
    X = X.to(device=dev, dtype=torch.float32)
    Xt = padded_design_t(X) if X.ndim == 2 else torch.stack([padded_design_t(x) for x in X])
    xmean = (X.double().mean(-2) if X.ndim == 3 else X.double().mean(0, keepdim=True)).float().contiguous()
    f32 = dict(device=dev, dtype=torch.float32)
    ng = 0 if f.glt is None else f.glt.shape[0]
    o = DsortOut(betas=torch.empty(V, K, **f32), tstats=torch.empty(V, K, **f32), dbetas=torch.empty(V, q, **f32),
                 dtstats=torch.empty(V, q, **f32), sigma2=torch.empty(V, **f32), fstats=torch.empty(V, **f32),
                 r2=torch.empty(V, **f32), cbeta=torch.empty(V, ng, **f32) if ng else None,
                 ct=torch.empty(V, ng, **f32) if ng else None,
                 resid=torch.empty(V, T, **f32) if want_residuals else None,
                 resid_w=torch.empty(V, T, **f32) if want_residuals else None,
                 pred=torch.empty(V, T, **f32) if want_predicted else None,
                 status=torch.zeros(1, dtype=torch.int32, device=dev))
    sp = si = sc_ = None
    n_sets = n_out = 0
    if column_sets:
        ptr, idx, col, n_out = dsort_sets_plan(column_sets, K, q)
        n_sets = len(col)
        o.set_fstats = torch.full((V, n_out), float("nan"), **f32)
        o.set_sd = torch.full((V, n_out), float("nan"), **f32)
        o.set_coef = torch.full((V, n_out), float("nan"), **f32)
        if n_sets:
            if f.Afull is None:
                raise ValueError("gls_dsort: column sets need the factors' Afull (build_factors(afull=True))")
            sp, si, sc_ = const_dev(ptr, dev), const_dev(idx, dev), const_dev(col, dev)
    h, ptau_d, w_d = 0, None, None
    if lj is not None and lj[0] > 0:
        h, ptau, w, _ = lj
        ptau_d = None if ptau is None else const_dev(ptau, dev)
        w_d = const_dev(w, dev)
        o.ljung_box = torch.empty(V, **f32)
    nt = 0 if f.task_idx is None else f.task_idx.numel()
    a = _lib.DsortArgs(V=V, T=T, K=K, q=q, dof=max(1, T - K - q), Y=_p(Y), scale=_p(scale), D=_p(D), Xt=_p(Xt),
                       xmean=_p(xmean), best=_p(key), n_pairs=n_pairs, coef=_p(f.coef), G=_p(f.G), U=_p(f.U),
                       Adiag=_p(f.Adiag), XtX=_p(f.XtX), Afull=_p(f.Afull), n_task=nt, task_idx=_p(f.task_idx),
                       Ftask=_p(f.Ftask), n_glt=ng, glt=_p(f.glt), glt_var=_p(f.glt_var), n_sets=n_sets,
                       set_ptr=_p(sp), set_idx=_p(si), set_col=_p(sc_), n_set_out=n_out, lj_h=h, lj_tau=_p(ptau_d),
                       lj_w=_p(w_d), betas=_p(o.betas), tstats=_p(o.tstats), dbetas=_p(o.dbetas),
                       dtstats=_p(o.dtstats), sigma2=_p(o.sigma2), fstats=_p(o.fstats), r2=_p(o.r2),
                       cbeta=_p(o.cbeta), ct=_p(o.ct), resid=_p(o.resid), resid_w=_p(o.resid_w), pred=_p(o.pred),
                       ljung_box=_p(o.ljung_box), set_fstats=_p(o.set_fstats), set_sd=_p(o.set_sd),
                       set_coef=_p(o.set_coef), status=_p(o.status), band_coef=_p(f.band_coef), band_w=f.band_w,
                       band=_p(f.band))
    _run("ffs_reml_gls_dsort", lib.ffs_reml_gls_dsort, C.byref(a), st)
    o._keep = (Y, D, key, Xt, xmean, sp, si, sc_, ptau_d, w_d)
    return o


def dsort_prepare(dsort, V: int, T: int, run_bounds=None, dev=None) -> torch.Tensor:
    """The -dsort regressors as the kernel reads them, (V, q, T) float32 on the
    device: (V, T) taken as one dataset, the shape checked as the reference
    does (ValueError), a series constant and nonzero through time replaced by
    its dataset's mean over the other voxels (with a warning), then one column
    per set and run when ``run_bounds`` [t0, ..., T] is given
    (fastfuncstuff/glm/arma.py:3207-3245, :3931-3945, :3385-3397)."""
    import warnings

    Dt = dsort if isinstance(dsort, torch.Tensor) else torch.as_tensor(np.asarray(dsort))
    Dt = Dt.to(device=dev, dtype=torch.float32)
    if Dt.ndim == 2:
        Dt = Dt.unsqueeze(1)
    if Dt.ndim != 3 or Dt.shape[0] != V or Dt.shape[2] != T:
        raise ValueError(f"dsort must be (n_voxels={V}, n_dsort, n_timepoints={T}); got {tuple(Dt.shape)}")
    sd = Dt.double().std(dim=2)
    mabs = Dt.double().abs().mean(dim=2)
    bad = (sd < 1e-8) & (mabs > 1e-8)
    n_bad = int(bad.sum().item())
    if n_bad:
        Dt = Dt.clone()
        for d in range(Dt.shape[1]):
            bd = bad[:, d]
            if bool(bd.any()):
                good = ~bd
                src = Dt[good, d] if bool(good.any()) else Dt[:, d]
                Dt[bd, d] = src.double().mean(0).float()
        warnings.warn(f"-dsort: {n_bad} voxel timeseries were ~constant through time and were replaced by "
                      "their dataset mean (matches 3dREMLfit).", stacklevel=3)
    if run_bounds is not None:
        rb = [int(x) for x in run_bounds]
        n_runs = len(rb) - 1
        n_sets = Dt.shape[1]
        out = torch.zeros(V, n_sets * n_runs, T, device=Dt.device, dtype=torch.float32)
        for si in range(n_sets):
            for r in range(n_runs):
                out[:, si * n_runs + r, rb[r]:rb[r + 1]] = Dt[:, si, rb[r]:rb[r + 1]]
        Dt = out
    return Dt.contiguous()


class GroupedFitGraph:
    """The grouped full-grid fit of one shape (one design per voxel group) as
    one CUDA graph: the FP64 grid build of every design, the residualisation
    of every voxel against its design, the tcgen05 projection work list, the
    criterion, the selection and the GLS, replayed as one unit. The data and
    the designs are copied into the graph's static buffers; the centring test
    of the designs (torch linear algebra) runs before the replay and its
    result is copied in too. Results are returned as new tensors."""

    def __init__(self, Y: torch.Tensor, Xs: torch.Tensor, grid: RemlGrid, layout: RunLayout, slots: DesignSlots, *,
                 hierarchical: bool, do_scale: bool, gls_kw: dict, factor_kw: dict):
        dev = Xs.device
        self.Y = torch.empty(tuple(Y.shape), dtype=torch.float32, device=dev)
        self.Xs = Xs.float().contiguous().clone()
        self.grid, self.layout, self.slots = grid, layout, slots
        self.hierarchical, self.do_scale, self.gls_kw, self.factor_kw = hierarchical, do_scale, gls_kw, factor_kw
        self.cflag, self.ccoef = constant_flag(self.Xs)
        self.Y.copy_(Y, non_blocking=True)
        self._body()  # fills the host-side caches a capture must not create
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="thread_local"):
            self._body()

    def _body(self):
        self.f = build_factors(self.Xs, self.grid, self.layout, center=(self.cflag, self.ccoef), **self.factor_kw)
        self.so = search_designs(self.Y, self.f, self.slots, hierarchical=self.hierarchical, do_scale=self.do_scale)
        self.go = gls(self.Y, self.so.scale, self.so.best, self.f, self.Xs, design=self.slots.design, **self.gls_kw)

    def run(self, Y: torch.Tensor, Xs: torch.Tensor):
        """(SearchOut, GlsOut) of data Y (V, T) and designs Xs (D, T, K)."""
        self.Y.copy_(Y, non_blocking=True)
        if not torch.equal(Xs, self.Xs):
            self.Xs.copy_(Xs)
            flag, coef = constant_flag(self.Xs)
            self.cflag.copy_(flag)
            self.ccoef.copy_(coef)
        self.graph.replay()
        so = SearchOut(best=self.so.best.clone(), best_crit=self.so.best_crit.clone(), scale=self.so.scale.clone())
        go = GlsOut(**{k: (None if v is None else v.clone()) for k, v in vars(self.go).items()
                       if not k.startswith("_")})
        return so, go


_GROUPED_GRAPHS: dict = {}


def grouped_graph_for(Y, Xs, grid, layout, gid, *, hierarchical, do_scale, gls_kw, factor_kw) -> GroupedFitGraph:
    """The cached GroupedFitGraph of this shape, grouping and options (built on first use)."""
    gid = np.asarray(gid, dtype=np.int32)
    fk = tuple((k, None if v is None else v.key() if hasattr(v, "key") else np.asarray(v).tobytes())
               for k, v in sorted(factor_kw.items()))
    key = (tuple(Y.shape), tuple(Xs.shape), str(Xs.device), grid.a.tobytes(), grid.b.tobytes(), grid.lambda_fp32,
           grid.ltop, None if grid.band is None else grid.band.tobytes(),
           layout.run_start.tobytes(), layout.tau.tobytes(), gid.tobytes(), hierarchical, do_scale,
           tuple(sorted(gls_kw.items())), fk)
    gr = _GROUPED_GRAPHS.get(key)
    if gr is None:
        while len(_GROUPED_GRAPHS) >= 2:  # a plan holds a few GB of static buffers
            _GROUPED_GRAPHS.pop(next(iter(_GROUPED_GRAPHS)))
        slots = design_slots(gid, Xs.shape[0], Xs.shape[2], grid.P, Xs.device)
        gr = GroupedFitGraph(Y, Xs, grid, layout, slots, hierarchical=hierarchical, do_scale=do_scale,
                             gls_kw=gls_kw, factor_kw=factor_kw)
        _GROUPED_GRAPHS[key] = gr
    return gr
