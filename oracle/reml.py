"""CPU oracle for the ARMA(1,1) REML voxelwise GLM -- TEST INFRASTRUCTURE ONLY.

This module is a NumPy restatement of the reference algorithm (fastfuncstuff's
``fit_glm_arma11`` path). It exists to check the CUDA product path and to time the
reference's CPU algorithm as the CPU baseline. Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of
``bench.py`` may import it, and there only as the checker or the timed CPU
baseline -- never as a fallback for the product path.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against golden vectors produced by running the reference itself
(``tests/golden/make_golden.py``), and against the reference's own known-answer
tests (Ljung-Box AFNI goldens, whitener-equals-dense, float32-vs-float64
selection).

Every function follows the dense algorithm of the reference (dense R, dense
Cholesky, dense L^-1 GEMMs), so it is an independent check of the product path,
which uses an O(N) banded factorisation instead.

Arithmetic: ``dtype=np.float64`` is the FP64 oracle (the reference's
``use_double=True``); ``dtype=np.float32`` mirrors the reference's default float32
CPU run and is what the CPU baseline times. Grid validity and lambda are always
evaluated in float32, element by element, exactly as the reference does on its
float32 grid tensors.

Reference citations are ``path:line`` inside the fastfuncstuff project.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

F32 = np.float32
F64 = np.float64


class _AfniMode:
    """Run-wide AFNI-faithful switch, as the reference keeps it
    (fastfuncstuff/glm/arma.py:59-92): banded R, near-white pairs dropped from
    the grid, AFNI's hierarchical ltop."""

    on: bool = False
    corcut: float = 1e-4


AFNI_MODE = _AfniMode()


def set_afni_mode(enabled: bool, corcut: float = 1e-4) -> None:
    """Follows fastfuncstuff/glm/arma.py:85-92."""
    AFNI_MODE.on = bool(enabled)
    AFNI_MODE.corcut = float(corcut)


def afni_bmax(a: float, lam: float, corcut: float) -> int:
    """Off-diagonals AFNI keeps in R: the lag at which lam * rho^(k-1) has
    fallen to corcut, rho = a clamped to [-0.9, 0.9]; 0 (R = I) below corcut,
    1 for a pure MA(1). Follows fastfuncstuff/glm/arma.py:95-109."""
    if abs(lam) < corcut:
        return 0
    rho = min(0.9, max(-0.9, a))
    if rho == 0.0:
        return 1
    return 1 + int(math.ceil(math.log(corcut / abs(lam)) / math.log(abs(rho))))

_LJ_RUN_SEPARATION = 66666  # fastfuncstuff/glm/arma.py:5968


# --------------------------------------------------------------------------- grid


def ensure_zero_in_grid(a_grid, b_grid, tolerance: float = 1e-6):
    """Snap a near-zero grid value to 0.0, or insert 0.0 and sort.

    Follows fastfuncstuff/glm/arma.py:516-582.
    """

    def _one(g):
        g = np.asarray(g, dtype=F32).copy()
        near = np.abs(g) < tolerance
        if near.any():
            g[near] = 0.0
        else:
            g = np.sort(np.concatenate([np.zeros(1, F32), g]))
        return g

    return _one(a_grid), _one(b_grid)


def arma_lambda_f32(a, b, dtype=F32):
    """lambda = (a+b)(1+ab)/(1+b^2+2ab), evaluated op by op in ``dtype``.

    Follows fastfuncstuff/glm/arma.py:695-729 (the expression order of
    ``_compute_arma11_lambda``). The reference evaluates it in the grid's dtype,
    which is the fit's dtype (float32, or float64 under ``use_double``;
    fastfuncstuff/glm/arma.py:1341-1342).
    """
    a = np.asarray(a, dtype=F32).astype(dtype)
    b = np.asarray(b, dtype=F32).astype(dtype)
    one, two = dtype(1), dtype(2)
    num = (a + b) * (one + a * b)
    den = (one + b * b) + (two * a) * b
    return num / den


def arma_lambda_output_f32(a, b):
    """The per-voxel lambda stored in results: (b+a)(1+ab)/(1+2ab+b^2+1e-10).

    Follows fastfuncstuff/glm/arma.py:4769-4777 and :4931-4936 (a different
    expression order from the grid filter's lambda, kept as written there).
    """
    a = np.asarray(a, dtype=F32)
    b = np.asarray(b, dtype=F32)
    one, two = F32(1), F32(2)
    num = (b + a) * (one + a * b)
    den = ((one + (two * a) * b) + b * b) + F32(1e-10)
    return num / den


@dataclass
class Grid:
    """The filtered (a, b) grid in the reference's ``param_list`` order."""

    a_axis: np.ndarray  # sorted unique a values (float32), after ensure_zero_in_grid
    b_axis: np.ndarray
    a: np.ndarray  # (P,) float32, meshgrid 'ij' order (a-major), filtered
    b: np.ndarray
    lam: np.ndarray  # (P,) float32 lambda of each kept pair
    ai: np.ndarray  # (P,) index of a in a_axis
    bi: np.ndarray

    @property
    def n(self) -> int:
        return int(self.a.shape[0])

    def param_list(self):
        return [(float(x), float(y)) for x, y in zip(self.a, self.b)]


def valid_grid(a_grid, b_grid, dtype=F32) -> Grid:
    """The valid (a, b) pairs of a grid.

    Follows the filter of fastfuncstuff/glm/arma.py:989-1040
    (``build_arma11_covariance_batch``): |a|<1, |b|<1, |1-a^2|>=1e-6, gamma0>0,
    lambda>=0, evaluated in ``dtype`` (the fit's dtype: the grid is cast to it at
    fastfuncstuff/glm/arma.py:1341-1342). Pairs are enumerated by
    ``meshgrid(a, b, 'ij')``. ``ensure_zero_in_grid`` is applied first, on the
    float32 grid, as ``precompute_autocorr_grid`` does (arma.py:1339).
    """
    a_g, b_g = ensure_zero_in_grid(a_grid, b_grid)
    am, bm = np.meshgrid(a_g, b_g, indexing="ij")
    a32 = am.reshape(-1).astype(F32)
    b32 = bm.reshape(-1).astype(F32)
    a, b = a32.astype(dtype), b32.astype(dtype)
    one, two = dtype(1), dtype(2)
    ok = (np.abs(a) < 1.0) & (np.abs(b) < 1.0)
    denom = one - a * a
    ok &= np.abs(denom) >= dtype(1e-6)
    gamma0 = ((one + b * b) + (two * a) * b) / (denom + dtype(1e-10))
    ok &= gamma0 > 0
    lam = arma_lambda_f32(a32, b32, dtype)
    ok &= lam >= 0
    if AFNI_MODE.on:  # near-white pairs fold into (0, 0) (arma.py:1031-1036)
        ok &= (lam == 0) | (lam >= AFNI_MODE.corcut)
    a, b, lam = a32[ok], b32[ok], lam[ok]
    a_axis = np.array(sorted(set(a.tolist())), dtype=F32)
    b_axis = np.array(sorted(set(b.tolist())), dtype=F32)
    ai = np.searchsorted(a_axis, a)
    bi = np.searchsorted(b_axis, b)
    return Grid(a_axis, b_axis, a, b, lam, ai, bi)


# ----------------------------------------------------------------- runs / censor


def run_bounds(n: int, run_starts=None):
    """[(start, stop), ...] of each run. Follows fastfuncstuff/glm/whiten.py:27-38."""
    if run_starts is None:
        return [(0, n)]
    starts = sorted({int(s) for s in np.asarray(run_starts).reshape(-1).tolist()})
    if not starts or starts[0] != 0:
        starts = [0, *starts]
    stops = [*starts[1:], n]
    return [(s, e) for s, e in zip(starts, stops) if e > s]


def build_censor_run_info(run_starts, n_total: int, good_list=None):
    """Run starts in retained-index space and the within-run time index tau.

    Follows fastfuncstuff/glm/arma.py:752-820.
    """
    starts = [int(s) for s in np.asarray(run_starts).reshape(-1).tolist()]
    if good_list is None:
        return starts, None
    retained = np.asarray(good_list, dtype=np.int64).reshape(-1)
    st = np.asarray(starts, dtype=np.int64)
    run_id = np.searchsorted(st, retained, side="right") - 1
    tau = retained - st[run_id]
    out = []
    for r in range(len(starts)):
        pos = np.nonzero(run_id == r)[0]
        if pos.size:
            out.append(int(pos[0]))
    return (out or [0]), tau


# --------------------------------------------------------- correlation / whitener


def corr_block(a: float, lam: float, taus: np.ndarray, dtype=F64, band: int | None = None) -> np.ndarray:
    """Dense ARMA(1,1) correlation of one run block: R_ij = corr[|tau_i - tau_j|].

    corr = [1, lam, lam*a, lam*a^2, ...]. Follows
    fastfuncstuff/glm/arma.py:1057-1073 (lambda is the float32 value, the powers
    of a are taken in ``dtype`` as the reference's type promotion does). With
    ``band`` the correlations at |tau_i - tau_j| > band are zero (AFNI's banded
    R, arma.py:1075-1089; band 0 is the identity).
    """
    taus = np.asarray(taus, dtype=np.int64)
    dist = np.abs(taus[:, None] - taus[None, :])
    max_lag = int(dist.max()) if taus.size else 0
    corr = np.zeros(max_lag + 1, dtype=dtype)
    corr[0] = 1.0
    if max_lag >= 1:
        corr[1] = dtype(lam)
        if max_lag >= 2:
            ex = np.arange(1, max_lag, dtype=dtype)
            corr[2:] = dtype(lam) * (dtype(a) ** ex)
    if band is not None:
        corr[band + 1:] = 0.0
    return corr[dist]


@dataclass
class Whitener:
    """L^-1 of a run-block-diagonal correlation, one dense block per run.

    Follows fastfuncstuff/glm/whiten.py:64-148 (``RunWhitener``).
    """

    blocks: list  # [(start, stop, Linv (m, m))]
    n: int

    def cols(self, M: np.ndarray) -> np.ndarray:
        """L^-1 @ M for M (T, k). Follows whiten.py:111-131."""
        out = np.empty_like(M)
        for s, e, Li in self.blocks:
            out[s:e] = Li.astype(M.dtype, copy=False) @ M[s:e]
        return out

    def rows(self, Y: np.ndarray) -> np.ndarray:
        """Y @ L^-T for Y (V, T). Follows whiten.py:133-148."""
        out = np.empty_like(Y)
        for s, e, Li in self.blocks:
            out[:, s:e] = Y[:, s:e] @ Li.astype(Y.dtype, copy=False).T
        return out

    def dense(self) -> np.ndarray:
        return self.cols(np.eye(self.n))


def _chol_inv(R: np.ndarray):
    """Cholesky factor's inverse (LAPACK trtri) and log(diag L + 1e-10)."""
    from scipy.linalg import lapack

    L = np.linalg.cholesky(R)
    logdiag = np.log(np.diagonal(L) + 1e-10)
    trtri = lapack.dtrtri if L.dtype == F64 else lapack.strtri
    Linv, info = trtri(L, lower=1)
    if info != 0:
        raise np.linalg.LinAlgError("singular Cholesky factor")
    return np.tril(Linv), logdiag


def _solve_lower(L: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Solve L X = B for lower-triangular L (LAPACK trtrs via scipy)."""
    from scipy.linalg import solve_triangular

    return solve_triangular(L, B, lower=True, check_finite=False)


def arma11_whiteners(grid: Grid, n: int, run_starts=None, tau=None, dtype=F64):
    """One whitener per valid pair plus logdet(R).

    Follows fastfuncstuff/glm/whiten.py:197-271: without censoring one max-length
    Toeplitz factor whose leading blocks serve every run; with ``tau`` one block
    per run. logdet(R) = 2 sum log(diag L + 1e-10) over the runs.
    """
    bounds = run_bounds(n, run_starts)
    lens = [e - s for s, e in bounds]
    whs, logdet = [], np.zeros(grid.n, dtype=dtype)

    def band(g):
        return afni_bmax(float(grid.a[g]), float(grid.lam[g]), AFNI_MODE.corcut) if AFNI_MODE.on else None

    if tau is None:
        m_max = max(lens)
        taus = np.arange(m_max)
        for g in range(grid.n):
            R = corr_block(float(grid.a[g]), float(grid.lam[g]), taus, dtype, band(g))
            Linv, logdiag = _chol_inv(R)
            cum = np.cumsum(logdiag)
            logdet[g] = 2 * sum(cum[m - 1] for m in lens)
            whs.append(Whitener([(s, e, Linv[: e - s, : e - s]) for s, e in bounds], n))
        return whs, logdet
    tau = np.asarray(tau, dtype=np.int64).reshape(-1)
    for g in range(grid.n):
        blocks, ld = [], 0.0
        for s, e in bounds:
            R = corr_block(float(grid.a[g]), float(grid.lam[g]), tau[s:e], dtype, band(g))
            Linv, logdiag = _chol_inv(R)
            ld = ld + 2 * logdiag.sum()
            blocks.append((s, e, Linv))
        logdet[g] = ld
        whs.append(Whitener(blocks, n))
    return whs, logdet


@dataclass
class PrecomputedGrid:
    grid: Grid
    whiteners: list
    X_w: np.ndarray  # (P, T, K)
    Q: np.ndarray  # (P, T, K)
    logdet_R: np.ndarray  # (P,)
    logdet_XtX: np.ndarray  # (P,)
    used_qr: bool = False


def precompute_reml_grid(X, grid: Grid, run_starts=None, tau=None, dtype=F64, autocorr=None):
    """Per-pair whitened design, Q and log det(X_w'X_w).

    Follows fastfuncstuff/glm/arma.py:1371-1531: Cholesky of X_w'X_w and
    Q = X_w L^-T, falling back to QR for the whole batch when any Cholesky fails
    (:1490-1500); logdet = 2 sum log(|diag| + 1e-10) (:1501-1503).
    """
    X = np.asarray(X, dtype=dtype)
    n = X.shape[0]
    if autocorr is None:
        whs, logdet_R = arma11_whiteners(grid, n, run_starts, tau, dtype)
    else:
        whs, logdet_R = autocorr
    Xw = np.stack([w.cols(X) for w in whs]) if whs else np.zeros((0,) + X.shape, dtype)
    used_qr = False
    try:
        XtX = np.einsum("gti,gtj->gij", Xw, Xw)
        L = np.linalg.cholesky(XtX)
        Q = np.stack([_solve_lower(L[g], Xw[g].T).T for g in range(Xw.shape[0])])
        diag = np.diagonal(L, axis1=1, axis2=2)
    except np.linalg.LinAlgError:
        used_qr = True
        Q, Rq = np.linalg.qr(Xw)
        diag = np.diagonal(Rq, axis1=1, axis2=2)
    logdet_XtX = 2 * np.log(np.abs(diag) + 1e-10).sum(axis=1)
    return PrecomputedGrid(grid, whs, Xw, Q, logdet_R.astype(dtype), logdet_XtX.astype(dtype), used_qr)


# ------------------------------------------------------------------------ search


def design_pinv(X: np.ndarray) -> np.ndarray:
    """Rank-truncated pseudo-inverse, SVD in float64.

    Follows fastfuncstuff/glm/core.py:248-273 (tolerance uses the design dtype).
    """
    Xd = np.asarray(X, dtype=F64)
    U, S, Vh = np.linalg.svd(Xd, full_matrices=False)
    tol = max(Xd.shape) * np.finfo(np.asarray(X).dtype).eps * S[0]
    r = int((S > tol).sum())
    return ((Vh[:r].T / S[:r]) @ U[:, :r].T).astype(np.asarray(X).dtype)


def residualize(X: np.ndarray, Y: np.ndarray) -> np.ndarray:
    """Y - (Y pinv(X)^T) X^T, skipped for float64 data.

    Follows fastfuncstuff/glm/arma.py:1554-1571.
    """
    if Y.dtype == F64 or X.shape[1] == 0:
        return Y
    X = X.astype(Y.dtype)
    pinv = design_pinv(X)
    return Y - (Y @ pinv.T) @ X.T


def search_exhaustive(X, Y, pre: PrecomputedGrid, return_surface: bool = False):
    """Global argmin of the REML criterion over every grid point.

    Follows fastfuncstuff/glm/arma.py:1886-2018: per pair Y_w = Y L^-T,
    RSS = sum Y_w^2 - sum (Y_w Q)^2 accumulated in float64,
    crit = logdet_R + logdet_XtX + (T-K) log(RSS + 1e-10) cast to Y's dtype, and
    a running minimum with strict '<' (the first pair wins ties).
    Returns (best_index (V,), best_crit (V,)[, surface (V, P)]).
    """
    T, K = X.shape
    dt = Y.dtype.type
    Yr = residualize(np.asarray(X, dtype=dt), Y)
    V = Y.shape[0]
    best = np.full(V, np.inf, dtype=dt)
    best_i = np.zeros(V, dtype=np.int64)
    surface = np.empty((V, pre.grid.n), dtype=dt) if return_surface else None
    for g, w in enumerate(pre.whiteners):
        Yw = w.rows(Yr)
        QtY = Yw @ pre.Q[g].astype(dt)
        rss = (Yw.astype(F64) ** 2).sum(1) - (QtY.astype(F64) ** 2).sum(1)
        const = dt(pre.logdet_R[g]) + dt(pre.logdet_XtX[g])
        lik = (F64(const) + (T - K) * np.log(rss + 1e-10)).astype(dt)
        imp = lik < best
        best[imp] = lik[imp]
        best_i[imp] = g
        if surface is not None:
            surface[:, g] = lik
    if return_surface:
        return best_i, best, surface
    return best_i, best


def _ltop(n_a: int, n_b: int, afni_faithful: bool = False) -> int:
    """Top level of the power-of-2 descent. Follows fastfuncstuff/glm/arma.py:2109-2115."""
    if afni_faithful:
        pna = (n_a - 1).bit_length() - 1
        pnb = (n_b - 1).bit_length() - 1
        return max(0, min(pna, pnb) - 2)
    return max(0, min(n_a, n_b).bit_length() - 2)


def select_hierarchical_from_surface(surface: np.ndarray, grid: Grid, afni_faithful=False):
    """AFNI's power-of-2 descent from (0, 0) as indexing on the full surface.

    Follows fastfuncstuff/glm/arma.py:2224-2322: lattice (V, n_a, n_b) with +inf
    at filtered pairs; coarsest level = fixed lattice; finer levels = 3x3 windows
    of +-step clamped to the lattice, flattened b-outer / a-inner; first minimum
    wins; a level only moves the voxel on a strict improvement.
    Returns (best_index into the grid (V,), best_crit (V,)).
    """
    V = surface.shape[0]
    n_a, n_b = len(grid.a_axis), len(grid.b_axis)
    lat = np.full((V, n_a, n_b), np.inf, dtype=surface.dtype)
    lat[:, grid.ai, grid.bi] = surface
    ltop = _ltop(n_a, n_b, afni_faithful)
    za = int(np.nonzero(np.abs(grid.a_axis) < 1e-6)[0][0])
    zb = int(np.nonzero(np.abs(grid.b_axis) < 1e-6)[0][0])
    vr = np.arange(V)
    ba = np.full(V, za, dtype=np.int64)
    bb = np.full(V, zb, dtype=np.int64)
    bl = lat[vr, ba, bb].copy()
    for lev in range(ltop, -1, -1):
        step = 1 << lev
        if lev == ltop:
            ac = np.arange(0, n_a, step)
            bc = np.arange(0, n_b, step)
            sub = lat[:, ac][:, :, bc].transpose(0, 2, 1).reshape(V, -1)  # b outer, a inner
            am = np.argmin(sub, axis=1)
            mn = sub[vr, am]
            a_sel = ac[am % len(ac)]
            b_sel = bc[am // len(ac)]
        else:
            offs = np.array([-step, 0, step])
            ac = np.clip(ba[:, None] + offs, 0, n_a - 1)
            bc = np.clip(bb[:, None] + offs, 0, n_b - 1)
            sub = lat[vr[:, None, None], ac[:, None, :], bc[:, :, None]].reshape(V, 9)
            am = np.argmin(sub, axis=1)
            mn = sub[vr, am]
            a_sel = ac[vr, am % 3]
            b_sel = bc[vr, am // 3]
        imp = mn < bl
        bl = np.where(imp, mn, bl)
        ba = np.where(imp, a_sel, ba)
        bb = np.where(imp, b_sel, bb)
    index = _lattice_to_index(grid)
    return index[ba, bb], bl


def _lattice_to_index(grid: Grid) -> np.ndarray:
    idx = np.full((len(grid.a_axis), len(grid.b_axis)), -1, dtype=np.int64)
    idx[grid.ai, grid.bi] = np.arange(grid.n)
    return idx


def search_hierarchical_subset(X, Y, pre: PrecomputedGrid, afni_faithful=False):
    """The reference's CPU default: the descent with one subset GEMM per grid point.

    Follows fastfuncstuff/glm/arma.py:2021-2221 (``_eval_subset`` at :2130-2168,
    levels at :2179-2213). Identical selections to
    :func:`select_hierarchical_from_surface` on the same criterion values; it is
    the algorithm the CPU baseline times.
    """
    T, K = X.shape
    dt = Y.dtype.type
    Yr = residualize(np.asarray(X, dtype=dt), Y)
    grid = pre.grid
    V = Y.shape[0]
    n_a, n_b = len(grid.a_axis), len(grid.b_axis)
    table = _lattice_to_index(grid)
    za = int(np.nonzero(np.abs(grid.a_axis) < 1e-6)[0][0])
    zb = int(np.nonzero(np.abs(grid.b_axis) < 1e-6)[0][0])
    ba = np.full(V, za, dtype=np.int64)
    bb = np.full(V, zb, dtype=np.int64)
    bl = np.full(V, np.inf, dtype=dt)

    def ev(ai, bi, act):
        g = table[ai, bi]
        if g < 0:
            return
        Ys = Yr[act]
        Yw = pre.whiteners[g].rows(Ys)
        QtY = Yw @ pre.Q[g].astype(dt)
        rss = (Yw.astype(F64) ** 2).sum(1) - (QtY.astype(F64) ** 2).sum(1)
        const = dt(pre.logdet_R[g]) + dt(pre.logdet_XtX[g])
        lik = (F64(const) + (T - K) * np.log(rss + 1e-10)).astype(dt)
        imp = lik < bl[act]
        if imp.any():
            gi = act[imp]
            bl[gi] = lik[imp]
            ba[gi] = ai
            bb[gi] = bi

    ev(za, zb, np.arange(V))
    ltop = _ltop(n_a, n_b, afni_faithful)
    for lev in range(ltop, -1, -1):
        step = 1 << lev
        if lev == ltop:
            a_lo, a_hi = np.zeros(V, np.int64), np.full(V, n_a - 1)
            b_lo, b_hi = np.zeros(V, np.int64), np.full(V, n_b - 1)
        else:
            a_lo, a_hi = np.clip(ba - step, 0, n_a - 1), np.clip(ba + step, 0, n_a - 1)
            b_lo, b_hi = np.clip(bb - step, 0, n_b - 1), np.clip(bb + step, 0, n_b - 1)
        for bi in range(0, n_b, step):
            in_b = (bi >= b_lo) & (bi <= b_hi)
            if not in_b.any():
                continue
            for ai in range(0, n_a, step):
                if table[ai, bi] < 0:
                    continue
                win = in_b & (ai >= a_lo) & (ai <= a_hi)
                if not win.any():
                    continue
                ev(ai, bi, np.nonzero(win)[0])
    return table[ba, bb], bl


# ------------------------------------------------------------------- Ljung-Box


def ljung_box_max_lag(n_time: int, n_regressors: int = 0, min_run: int | None = None) -> int:
    """AFNI's max lag h. Follows fastfuncstuff/glm/arma.py:5971-5999."""
    if min_run is None:
        min_run = n_time
    if min_run < 2:
        return 0
    h1 = min_run // 8
    h2 = int(round(3.0 * math.log(min_run)))
    return min(n_regressors + 2 + min(h1, h2), min_run // 2)


def resolve_ljung_box_lag(n_time: int, max_lag) -> int:
    """ljung_box_uneven's own clamp. Follows fastfuncstuff/glm/arma.py:6002-6014."""
    hh = int(max_lag) if max_lag else 0
    if hh < 2 or hh > n_time // 2:
        hh = 2 + min(n_time // 8, int(round(3.0 * math.log(n_time))))
        hh = min(hh, n_time // 2)
    return hh


def build_ljung_box_tau(n_time: int, run_starts=None, tau=None):
    """Pseudo-time for lag binning. Follows fastfuncstuff/glm/arma.py:6017-6049."""
    starts = [] if run_starts is None else [int(s) for s in np.asarray(run_starts).reshape(-1)]
    starts = sorted({s for s in starts if 0 <= s < n_time}) or [0]
    if tau is None and len(starts) == 1 and starts[0] == 0:
        return None
    st = np.asarray(starts, dtype=np.int64)
    idx = np.arange(n_time, dtype=np.int64)
    run_id = np.searchsorted(st, idx, side="right") - 1
    within = np.asarray(tau, dtype=np.int64).reshape(-1) if tau is not None else idx - st[run_id]
    return within + _LJ_RUN_SEPARATION * run_id


def ljung_box(resid: np.ndarray, max_lag=None, tau=None) -> np.ndarray:
    """Ljung-Box of each row, AFNI ljung_box_uneven semantics, float64.

    Follows fastfuncstuff/glm/arma.py:6058-6141: c_k = sum r_j r_{j+k} / sum r^2
    binned by time lag (pairs with 0 < dj <= h), bins need n_k > 1,
    LB = n(n+2) sum c_k^2 / n_k clamped at 1e10; 0 when n < 10 or sum r^2 < 1e-10.
    """
    r = np.asarray(resid, dtype=F64)
    if r.ndim == 1:
        r = r[None]
    V, n = r.shape
    out = np.zeros(V)
    if n < 10:
        return out
    hh = resolve_ljung_box_lag(n, max_lag)
    if hh < 1:
        return out
    s0 = (r * r).sum(1)
    ok = s0 >= 1e-10
    s0 = np.where(ok, s0, 1.0)
    sumk = np.zeros((V, hh + 1))
    nj = np.zeros(hh + 1, dtype=np.int64)
    if tau is None:
        for k in range(1, hh + 1):
            nj[k] = n - k
            sumk[:, k] = (r[:, : n - k] * r[:, k:]).sum(1)
    else:
        t = np.asarray(tau, dtype=np.int64).reshape(-1)
        for k in range(1, hh + 1):
            dj = t[k:] - t[: n - k]
            keep = np.nonzero((dj > 0) & (dj <= hh))[0]
            if keep.size:
                np.add.at(nj, dj[keep], 1)
                prod = r[:, : n - k][:, keep] * r[:, k:][:, keep]
                for col, d in enumerate(dj[keep]):
                    sumk[:, d] += prod[:, col]
    good = nj > 1
    good[0] = False
    if not good.any():
        return out
    gi = np.nonzero(good)[0]
    ck = sumk[:, gi] / s0[:, None]
    g = (ck**2 / nj[gi].astype(F64)).sum(1) * (n * (n + 2.0))
    return np.where(ok, np.minimum(g, 1.0e10), 0.0)


# ------------------------------------------------------------------------- GLS


def _cod(y: np.ndarray, pred: np.ndarray) -> np.ndarray:
    """Coefficient of determination. Follows fastfuncstuff/glm/xval.py:564-593."""
    ss_res = ((y - pred) ** 2).sum(1)
    ss_tot = ((y - y.mean(1, keepdims=True)) ** 2).sum(1)
    deg = ss_tot <= 1e-10
    r2 = 1.0 - ss_res / np.maximum(ss_tot, 1e-10)
    return np.where(deg, 0.0, np.minimum(r2, 1.0))


@dataclass
class Results:
    """The per-voxel outputs of ``ARMA11Results`` this oracle produces.

    Field meanings follow fastfuncstuff/glm/arma.py:585-692.
    """

    betas: np.ndarray = None
    tstats: np.ndarray = None
    r2: np.ndarray = None
    arma_params: np.ndarray = None
    arma_index: np.ndarray = None
    arma_lambda: np.ndarray = None
    reml_likelihood: np.ndarray = None
    sigma2: np.ndarray = None
    fstats: np.ndarray = None
    dof: int = None
    residuals: np.ndarray = None
    residuals_whitened: np.ndarray = None
    predicted: np.ndarray = None
    ljung_box: np.ndarray = None
    ljung_box_dof: int = None
    contrast_betas: np.ndarray = None
    contrast_tstats: np.ndarray = None
    r2_partial: np.ndarray = None
    set_fstats: np.ndarray = None
    set_sd: np.ndarray = None
    set_coef: np.ndarray = None
    dsort_betas: np.ndarray = None
    dsort_tstats: np.ndarray = None
    reml_lklhd_surface: np.ndarray = None
    extra: dict = field(default_factory=dict)


def column_set_matrices(A: np.ndarray, X: np.ndarray, column_sets):
    """Per column set: (indices, inv(A_SS + 1e-8 I), Xc_S' Xc_S / T) with A =
    (X_w'X_w)^-1 of one (a, b) and Xc the column-centred unwhitened design;
    None for a set naming a column outside the design (or an empty set).
    Follows fastfuncstuff/glm/arma.py:3542-3561."""
    K, T = X.shape[1], X.shape[0]
    Xc = X - X.mean(0, keepdims=True)
    out = []
    for cols in column_sets:
        keep = [c for c in cols if c < K]
        if len(keep) != len(cols) or not keep:
            out.append(None)
            continue
        ix = np.asarray(keep)
        M = np.linalg.inv(A[np.ix_(ix, ix)] + 1e-8 * np.eye(len(ix), dtype=A.dtype))
        Xs = Xc[:, ix]
        out.append((ix, M, Xs.T @ Xs / T))
    return out


def column_set_stats(beta: np.ndarray, sigma2: np.ndarray, mats):
    """(F, SD, coef) per voxel and set of the betas and sigma2 of the scaled
    data: F = b_S' M b_S / (q sigma2 + 1e-30), SD = sqrt(max(b_S' C b_S, 0)),
    coef = b for a one-column set; NaN where a set is absent (coef: or wider).
    Follows fastfuncstuff/glm/arma.py:3564-3586."""
    V, G = beta.shape[0], len(mats)
    F = np.full((V, G), np.nan, beta.dtype)
    sd = np.full((V, G), np.nan, beta.dtype)
    coef = np.full((V, G), np.nan, beta.dtype)
    for g, m in enumerate(mats):
        if m is None:
            continue
        ix, M, C = m
        b = beta[:, ix]
        F[:, g] = np.einsum("vi,ij,vj->v", b, M, b) / (len(ix) * sigma2 + 1e-30)
        sd[:, g] = np.sqrt(np.maximum(np.einsum("vi,ij,vj->v", b, C, b), 0.0))
        if len(ix) == 1:
            coef[:, g] = b[:, 0]
    return F, sd, coef


def gls_at(Xd, Y, whitener: Whitener, dof: int, task_indices=None, glt=None, want_resid=False,
           lj=None, column_sets=None):
    """GLS refit of voxels that share one (a, b).

    Follows fastfuncstuff/glm/arma.py:4853-4905 (group constants: X_w'X_w,
    Cholesky, cholesky_inverse A, the F matrices) and :5227-5363, :5421-5472
    (betas = (Y_w X_w) A^T, sigma2 = sum r_w^2 / dof with float64 accumulation,
    t = b/(sqrt(sigma2 diag A)+1e-10), F = b'Mb/(sigma2 p + 1e-10), R^2 on the
    unwhitened data, GLT c'b and its t).
    """
    dt = Y.dtype
    K = Xd.shape[1]
    Xw = whitener.cols(Xd)
    XtX = Xw.T @ Xw
    try:
        Lg = np.linalg.cholesky(XtX)
        Li = _solve_lower(Lg, np.eye(K, dtype=dt))
        A = Li.T @ Li
    except np.linalg.LinAlgError:
        A = np.linalg.inv(XtX)
    Yw = whitener.rows(Y)
    beta = (Yw @ Xw) @ A.T
    rw = Yw - beta @ Xw.T
    pred = beta @ Xd.T
    sigma2 = ((rw.astype(F64) ** 2).sum(1) / dof).astype(dt)
    se = np.sqrt(sigma2[:, None] * np.diagonal(A)[None, :])
    t = beta / (se + 1e-10)
    if task_indices is not None:
        ti = list(task_indices)
        At = A[np.ix_(ti, ti)]
        M = np.linalg.inv(At + 1e-8 * np.eye(len(ti), dtype=dt))
        bt = beta[:, ti]
        quad = np.einsum("vi,ij,vj->v", bt, M, bt)
        F = quad / (sigma2 * len(ti) + 1e-10)
    else:
        quad = np.einsum("vi,ij,vj->v", beta, XtX, beta)
        F = quad / (sigma2 * K + 1e-10)
    r2 = _cod(Y.astype(dt), pred)
    out = dict(beta=beta, t=t, sigma2=sigma2, F=F, r2=r2)
    if glt is not None:
        C = np.asarray(glt, dtype=dt)
        cb = beta @ C.T
        cvar = np.einsum("cr,rs,cs->c", C, A, C)[None, :] * sigma2[:, None]
        out["cb"] = cb
        out["ct"] = cb / (np.sqrt(np.maximum(cvar, 0.0)) + 1e-10)
        out["ct_r2p"] = out["ct"] ** 2 / (out["ct"] ** 2 + dof)
    out["r2_partial"] = t**2 / (t**2 + dof)
    if want_resid:
        out["resid"] = Y - pred
        out["resid_w"] = rw
        out["pred"] = pred
    if lj is not None:
        out["lb"] = ljung_box(rw, lj[0], lj[1])
    if column_sets:
        out["sets"] = column_set_stats(beta, sigma2, column_set_matrices(A, Xd, column_sets))
    return out


def global_arma(X, y, a_grid, b_grid, run_starts=None, tau=None):
    """((a, b), criterion) of one series over the raw grid, a outer and b
    inner, the first strict minimum (fastfuncstuff/glm/arma.py:1189-1294 with
    :1106-1186): pairs with |a| or |b| >= 1 or lambda < 0 are skipped; the
    criterion is 2 sum log(diag L + 1e-10) + logdet(X_w'X_w + 1e-6 I) + (n - p)
    log(||y_w - X_w b||^2 + 1e-10), b from the regularised normal equations.
    FP64."""
    X = np.asarray(X, F64)
    y = np.asarray(y, F64)
    n, p = X.shape
    best, best_ab = np.inf, (0.5, 0.0)
    for a in np.asarray(a_grid, F32):
        for b in np.asarray(b_grid, F32):
            af, bf = float(a), float(b)
            if abs(af) >= 1 or abs(bf) >= 1:
                continue
            if (bf + af) * (1 + af * bf) / (1 + 2 * af * bf + bf * bf) < 0:
                continue
            one = Grid(np.array([a], F32), np.array([b], F32), np.array([a], F32), np.array([b], F32),
                       np.array([(bf + af) * (1 + af * bf) / (1 + 2 * af * bf + bf * bf)]),
                       np.zeros(1, np.int64), np.zeros(1, np.int64))
            whs, logdets = arma11_whiteners(one, n, run_starts, tau, F64)[:2]
            wh = whs[0]
            Xw = wh.cols(X)
            yw = wh.cols(y[:, None])[:, 0]
            M = Xw.T @ Xw + 1e-6 * np.eye(p)
            sign, ld = np.linalg.slogdet(M)
            beta = np.linalg.solve(M, Xw.T @ yw)
            rss = ((yw - Xw @ beta) ** 2).sum()
            lik = float(logdets[0]) + (ld if sign > 0 else 1e10) + (n - p) * np.log(rss + 1e-10)
            if lik < best:
                best, best_ab = lik, (af, bf)
    return best_ab, best


def dsort_constant_guard(D: np.ndarray) -> np.ndarray:
    """A -dsort series that is constant and nonzero through time is replaced by
    its dataset's mean series over the other voxels (all-zero, run-padded
    columns are left alone). Follows fastfuncstuff/glm/arma.py:3207-3245."""
    D = np.array(D, copy=True)
    sd = D.astype(F64).std(2, ddof=1)
    mean_abs = np.abs(D).astype(F64).mean(2)
    bad = (sd < 1e-8) & (mean_abs > 1e-8)
    for d in range(D.shape[1]):
        if bad[:, d].any():
            good = ~bad[:, d]
            src = D[good, d] if good.any() else D[:, d]
            D[bad[:, d], d] = src.mean(0)
    return D


def dsort_expand(D: np.ndarray, run_bounds=None) -> np.ndarray:
    """(V, n_sets, T) -> (V, n_sets * n_runs, T) with one zero-padded column per
    set and run when run_bounds [t0, t1, ..., T] is given (set-major, then
    run). Follows fastfuncstuff/glm/arma.py:3385-3397."""
    if run_bounds is None:
        return D
    V, n_sets, T = D.shape
    n_runs = len(run_bounds) - 1
    out = np.zeros((V, n_sets * n_runs, T), D.dtype)
    for si in range(n_sets):
        for r in range(n_runs):
            t0, t1 = run_bounds[r], run_bounds[r + 1]
            out[:, si * n_runs + r, t0:t1] = D[:, si, t0:t1]
    return out


def gls_dsort_at(Xd, Ys, D, whitener: Whitener, dof: int, task_indices=None, glt=None, lj=None,
                 column_sets=None):
    """The per-voxel GLS with the extended design [X | D_v] at one (a, b).

    Follows fastfuncstuff/glm/arma.py:3367-3539: X_ext = [X_w | D_w]; betas
    from the Cholesky factor of X_ext'X_ext + 1e-8 I, its inverse for the
    standard errors; sigma2 = sum r_w^2 / dof (float64 sum); t = b/(se+1e-10);
    R^2 of the unwhitened fit; F over the task (or all base) columns with
    inv(A_task + 1e-8 I) and 1e-30; GLT on the base block; Ljung-Box of r_w;
    column sets over [X | D] with the voxel's own inverse block.
    """
    dt = Ys.dtype
    V, q, T = D.shape
    K = Xd.shape[1]
    Xw = whitener.cols(Xd)
    Yw = whitener.rows(Ys)
    out = {k: [] for k in ("beta", "t", "sigma2", "F", "r2", "resid", "resid_w", "pred", "cb", "ct", "lb",
                           "sets")}
    Xc_all = None
    for v in range(V):
        Dw = whitener.cols(D[v].T.astype(dt))
        Xe = np.concatenate([Xw, Dw], 1)
        M = Xe.T @ Xe + 1e-8 * np.eye(K + q, dtype=dt)
        L = np.linalg.cholesky(M)
        Li = _solve_lower(L, np.eye(K + q, dtype=dt))
        Minv = Li.T @ Li
        b = Minv @ (Xe.T @ Yw[v])
        rw = Yw[v] - Xe @ b
        s2 = dt.type((rw.astype(F64) ** 2).sum() / dof)
        t = b / (np.sqrt(s2 * np.diagonal(Minv)) + 1e-10)
        pred = Xd @ b[:K] + b[K:] @ D[v]
        ti = list(task_indices) if task_indices is not None else list(range(K))
        A = Minv[np.ix_(ti, ti)]
        Ai = np.linalg.inv(A + 1e-8 * np.eye(len(ti), dtype=dt))
        bt = b[ti]
        out["F"].append(bt @ Ai @ bt / (s2 * len(ti) + 1e-30))
        out["beta"].append(b)
        out["t"].append(t)
        out["sigma2"].append(s2)
        out["r2"].append(_cod(Ys[v][None], pred[None])[0])
        out["resid"].append(Ys[v] - pred)
        out["resid_w"].append(rw)
        out["pred"].append(pred)
        if glt is not None:
            C = np.asarray(glt, dtype=dt)
            cb = C @ b[:K]
            var = np.einsum("cr,rs,cs->c", C, s2 * Minv[:K, :K], C)
            out["cb"].append(cb)
            out["ct"].append(cb / (np.sqrt(np.maximum(var, 0.0)) + 1e-10))
        if column_sets:
            if Xc_all is None:
                Xc_all = Xd - Xd.mean(0, keepdims=True)
            Xo = np.concatenate([Xc_all, (D[v] - D[v].mean(1, keepdims=True)).T], 1)
            F_, sd_, co_ = [], [], []
            for cols in column_sets:
                ix = np.asarray(cols)
                if len(ix) == 0 or ix.max() >= K + q:
                    F_.append(np.nan), sd_.append(np.nan), co_.append(np.nan)
                    continue
                bs = b[ix]
                As = Minv[np.ix_(ix, ix)] + 1e-8 * np.eye(len(ix), dtype=dt)
                F_.append(bs @ np.linalg.solve(As, bs) / (len(ix) * s2 + 1e-30))
                sd_.append((Xo[:, ix] @ bs).std())
                co_.append(bs[0] if len(ix) == 1 else np.nan)
            out["sets"].append((F_, sd_, co_))
    res = {k: np.asarray(v) for k, v in out.items() if v and k not in ("sets",)}
    if lj is not None:
        res["lb"] = ljung_box(res["resid_w"], lj[0], lj[1])
    if column_sets:
        res["sets"] = tuple(np.asarray([s[i] for s in out["sets"]], dt) for i in range(3))
    return res


def fit_glm_arma11(data, design, tr=2.0, a_grid=None, b_grid=None, *, use_double=True,
                   force_exhaustive_search=False, run_starts=None, tau=None,
                   task_indices=None, glt_matrices=None, want_residuals=False,
                   want_ljung_box=False, save_profile_likelihoods=False,
                   precomputed_arma_params=None, fp64_scaled=False, afni_faithful=False,
                   autocorr=None, subset_descent=False, column_sets=None, dsort=None, dsort_run_bounds=None,
                   estimate_per_voxel=True):
    """The reference's ``fit_glm_arma11`` for the options this path covers.

    Follows fastfuncstuff/glm/arma.py:3650-5878 on ``device=cpu``:

    - ``use_double=True``: float64 throughout, no per-voxel scaling, no
      residualisation (the reference's FP64 mode).
    - ``use_double=False``: the reference's float32 mode (Y / std(Y), float32
      GEMMs with float64 RSS accumulation, unscale at the end).
    - ``fp64_scaled=True`` (with ``use_double=True``): float64 arithmetic on the
      float32 mode's semantics -- the data divided by the float32 std, the
      likelihood reported on the scaled data, betas and sigma2 unscaled. This is
      the FP64 oracle the float32 product path is compared with.

    The selector is the hierarchical descent unless ``force_exhaustive_search``;
    the descent runs on the full surface, which selects the same points as the
    reference's subset-GEMM descent (fastfuncstuff/glm/arma.py:4688-4743). With
    ``subset_descent`` the descent instead evaluates only the pairs it visits,
    one subset GEMM per pair, which is the algorithm (and the cost) of the
    reference's default CPU run (arma.py:4699-4709).
    """
    dt = F64 if use_double else F32
    afni_faithful = afni_faithful or AFNI_MODE.on
    Y = np.asarray(data)
    if Y.ndim == 4:
        Y = Y.reshape(-1, Y.shape[-1])
    if Y.ndim != 2:
        raise ValueError(f"Data must be 2D or 4D, got {Y.ndim}D")
    Y = Y.astype(dt)
    X = np.asarray(design).astype(dt)
    V, T = Y.shape
    if X.shape[0] != T:
        raise ValueError(f"Timepoints mismatch: Data has {T}, Design has {X.shape[0]}")
    K = X.shape[1]
    scale = None
    if not use_double or fp64_scaled:
        # torch's CPU std of a float32 tensor accumulates in double and rounds to
        # float32 (fastfuncstuff/glm/arma.py:3952-3954)
        src = np.asarray(data).reshape(V, T).astype(F64)
        scale = np.maximum(np.std(src, axis=1, ddof=1).astype(F32), F32(1e-8))
    Ys = Y / scale[:, None].astype(dt) if scale is not None else Y
    dof = max(1, T - K)
    res = Results(dof=dof)
    if a_grid is None:
        a_grid = np.linspace(0.0, 0.8, 9).astype(F32)
    if b_grid is None:
        b_grid = np.linspace(-0.8, 0.8, 17).astype(F32)
    grid = valid_grid(a_grid, b_grid, dt)
    global_lik = None
    if not estimate_per_voxel and precomputed_arma_params is None:
        (a_opt, b_opt), global_lik = global_arma(X, Y.mean(0), a_grid, b_grid, run_starts, tau)
        precomputed_arma_params = np.tile(np.array([[a_opt, b_opt]], F32), (V, 1))
    if precomputed_arma_params is not None:
        pa = np.asarray(precomputed_arma_params, dtype=F32).reshape(V, 2)
        pairs, inv = np.unique(pa, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        res.arma_params = pa.astype(dt)
        idx = None
    else:
        pre = precompute_reml_grid(X, grid, run_starts, tau, dt, autocorr)
        if force_exhaustive_search:
            out = search_exhaustive(X, Ys, pre, return_surface=save_profile_likelihoods)
            if save_profile_likelihoods:
                idx, lik, surf = out
                res.reml_lklhd_surface = surf
            else:
                idx, lik = out
        elif subset_descent and not save_profile_likelihoods:
            idx, lik = search_hierarchical_subset(X, Ys, pre, afni_faithful)
        else:
            _, _, surf = search_exhaustive(X, Ys, pre, return_surface=True)
            idx, lik = select_hierarchical_from_surface(surf, grid, afni_faithful)
            if save_profile_likelihoods:
                res.reml_lklhd_surface = surf
        res.arma_index = idx
        res.reml_likelihood = lik
        res.arma_params = np.stack([grid.a[idx], grid.b[idx]], 1).astype(dt)
        pairs, inv = np.unique(res.arma_params.astype(F32), axis=0, return_inverse=True)
        inv = inv.reshape(-1)
    if global_lik is not None:
        res.reml_likelihood = np.full(V, global_lik, dt)
    lam = arma_lambda_output_f32(res.arma_params[:, 0], res.arma_params[:, 1]).astype(dt)
    if use_double:
        a64 = res.arma_params[:, 0].astype(F64)
        b64 = res.arma_params[:, 1].astype(F64)
        lam = (b64 + a64) * (1 + a64 * b64) / (1 + 2 * a64 * b64 + b64**2 + 1e-10)
    res.arma_lambda = lam
    n_out = len(task_indices) if task_indices else K
    res.betas = np.zeros((V, n_out), dt)
    res.tstats = np.zeros((V, n_out), dt)
    res.sigma2 = np.zeros(V, dt)
    res.fstats = np.zeros(V, dt)
    res.r2 = np.zeros(V, F32)
    res.r2_partial = np.zeros((V, n_out), dt)
    if want_residuals:
        res.residuals = np.zeros((V, T), dt)
        res.residuals_whitened = np.zeros((V, T), dt)
        res.predicted = np.zeros((V, T), dt)
    lj = None
    if want_ljung_box:
        starts = sorted({int(s) for s in np.asarray(run_starts).reshape(-1)}) if run_starts is not None else [0]
        mins = min(b - a for a, b in zip(starts, starts[1:] + [T])) if len(starts) > 1 else T
        h = ljung_box_max_lag(T, K, mins)
        lj = (h, build_ljung_box_tau(T, run_starts, tau))
        res.ljung_box = np.zeros(V, F32)
        res.ljung_box_dof = max(1, resolve_ljung_box_lag(T, h) - 2)
    if column_sets:
        res.set_fstats = np.full((V, len(column_sets)), np.nan, dt)
        res.set_sd = np.full((V, len(column_sets)), np.nan, dt)
        res.set_coef = np.full((V, len(column_sets)), np.nan, dt)
    if glt_matrices is not None:
        C = np.stack([np.asarray(c, dtype=dt).reshape(-1) for c in glt_matrices])
        res.contrast_betas = np.zeros((V, C.shape[0]), dt)
        res.contrast_tstats = np.zeros((V, C.shape[0]), dt)
    else:
        C = None
    for gi in range(pairs.shape[0]):
        members = np.nonzero(inv == gi)[0]
        a_opt, b_opt = float(pairs[gi, 0]), float(pairs[gi, 1])
        one = Grid(np.array([a_opt], F32), np.array([b_opt], F32), np.array([a_opt], F32),
                   np.array([b_opt], F32),
                   arma_lambda_f32(np.array([a_opt], F32), np.array([b_opt], F32), dt),
                   np.zeros(1, np.int64), np.zeros(1, np.int64))
        if one.lam[0] < 0 or abs(a_opt) >= 1 or abs(b_opt) >= 1:
            raise ValueError(f"Invalid ARMA(1,1) parameters: a={a_opt}, b={b_opt}")
        if precomputed_arma_params is None:
            # the search grid already holds this pair's whitener (arma.py:4837-4841)
            wh = pre.whiteners[int(idx[members[0]])]
        else:
            wh = arma11_whiteners(one, T, run_starts, tau, dt)[0][0]
        o = gls_at(X, Ys[members], wh, dof, task_indices, C, want_residuals, lj, column_sets)
        ti = list(task_indices) if task_indices else slice(None)
        res.betas[members] = o["beta"][:, ti]
        res.tstats[members] = o["t"][:, ti]
        res.sigma2[members] = o["sigma2"]
        res.fstats[members] = o["F"]
        res.r2[members] = o["r2"]
        res.r2_partial[members] = o["r2_partial"][:, ti]
        if C is not None:
            res.contrast_betas[members] = o["cb"]
            res.contrast_tstats[members] = o["ct"]
        if want_residuals:
            res.residuals[members] = o["resid"]
            res.residuals_whitened[members] = o["resid_w"]
            res.predicted[members] = o["pred"]
        if lj is not None:
            res.ljung_box[members] = o["lb"]
        if column_sets:
            res.set_fstats[members], res.set_sd[members], res.set_coef[members] = o["sets"]
    if dsort is not None:
        # the per-voxel GLS with [X | D_v] at the pairs estimated without D
        # (fastfuncstuff/glm/arma.py:3248-3539); dof drops by the D columns
        D = np.asarray(dsort, dtype=dt)
        if D.ndim == 2:
            D = D[:, None, :]
        D = dsort_expand(dsort_constant_guard(D), dsort_run_bounds)
        q = D.shape[1]
        dof = max(1, T - K - q)
        res.dof = dof
        res.dsort_betas = np.zeros((V, q), dt)
        res.dsort_tstats = np.zeros((V, q), dt)
        for gi in range(pairs.shape[0]):
            members = np.nonzero(inv == gi)[0]
            if precomputed_arma_params is None:
                wh = pre.whiteners[int(idx[members[0]])]
            else:
                one = Grid(np.array([pairs[gi, 0]], F32), np.array([pairs[gi, 1]], F32),
                           np.array([pairs[gi, 0]], F32), np.array([pairs[gi, 1]], F32),
                           arma_lambda_f32(np.array([pairs[gi, 0]], F32), np.array([pairs[gi, 1]], F32), dt),
                           np.zeros(1, np.int64), np.zeros(1, np.int64))
                wh = arma11_whiteners(one, T, run_starts, tau, dt)[0][0]
            o = gls_dsort_at(X, Ys[members], D[members], wh, dof, task_indices, C, lj, column_sets)
            ti = list(task_indices) if task_indices else slice(None)
            res.betas[members] = o["beta"][:, :K][:, ti]
            res.tstats[members] = o["t"][:, :K][:, ti]
            res.dsort_betas[members] = o["beta"][:, K:]
            res.dsort_tstats[members] = o["t"][:, K:]
            res.sigma2[members] = o["sigma2"]
            res.fstats[members] = o["F"]
            res.r2[members] = o["r2"]
            t2 = o["t"][:, :K] ** 2
            res.r2_partial[members] = (t2 / (t2 + dof))[:, ti]
            if C is not None:
                res.contrast_betas[members] = o["cb"]
                res.contrast_tstats[members] = o["ct"]
            if want_residuals:
                res.residuals[members] = o["resid"]
                res.residuals_whitened[members] = o["resid_w"]
                res.predicted[members] = o["pred"]
            if lj is not None:
                res.ljung_box[members] = o["lb"]
            if column_sets:
                res.set_fstats[members], res.set_sd[members], res.set_coef[members] = o["sets"]
    if scale is not None:
        s = scale.astype(dt)
        res.betas *= s[:, None]
        res.sigma2 *= s**2
        if res.dsort_betas is not None:
            res.dsort_betas *= s[:, None]
        if res.contrast_betas is not None:
            res.contrast_betas *= s[:, None]
        if column_sets:  # fastfuncstuff/glm/arma.py:5845-5848
            res.set_sd *= s[:, None]
            res.set_coef *= s[:, None]
        if want_residuals:
            res.residuals *= s[:, None]
            res.residuals_whitened *= s[:, None]
            res.predicted *= s[:, None]
        res.extra["scale"] = scale
    res.extra["grid"] = grid
    return res


def fit_glm_arma11_grouped(data, designs_by_group, group_indices, tr=2.0, **kw):
    """Per-group designs sharing one autocorrelation grid, scattered back.

    Follows fastfuncstuff/glm/arma.py:2836-3183: every group's design must have the
    same shape (ValueError otherwise), a missing group design raises KeyError, the
    design-independent whiteners are built once, and each group's voxels are fit
    with that group's design.
    """
    Y = np.asarray(data)
    gid = np.asarray(group_indices).astype(np.int64).reshape(-1)
    if gid.shape[0] != Y.shape[0]:
        raise ValueError(f"group_indices length {gid.shape[0]} != data n_voxels {Y.shape[0]}")
    groups = sorted(set(gid.tolist()))
    missing = [h for h in groups if h not in designs_by_group]
    if missing:
        raise KeyError(f"group ids {missing} missing from designs_by_group")
    shape0 = np.asarray(designs_by_group[groups[0]]).shape
    for h in groups[1:]:
        if np.asarray(designs_by_group[h]).shape != shape0:
            raise ValueError("per-group designs must share dims")
    use_double = kw.get("use_double", True)
    dt = F64 if use_double else F32
    a_grid = kw.get("a_grid")
    b_grid = kw.get("b_grid")
    if a_grid is None:
        a_grid = np.linspace(0.0, 0.8, 9).astype(F32)
    if b_grid is None:
        b_grid = np.linspace(-0.8, 0.8, 17).astype(F32)
    kw = dict(kw, a_grid=a_grid, b_grid=b_grid)
    grid = valid_grid(a_grid, b_grid, dt)
    autocorr = arma11_whiteners(grid, shape0[0], kw.get("run_starts"), kw.get("tau"), dt)
    per = {}
    for h in groups:
        m = gid == h
        per[h] = (m, fit_glm_arma11(Y[m], designs_by_group[h], tr, autocorr=autocorr, **kw))
    merged = Results(dof=per[groups[0]][1].dof)
    for attr in ("betas", "tstats", "r2", "arma_params", "arma_index", "arma_lambda",
                 "reml_likelihood", "sigma2", "fstats", "ljung_box", "r2_partial",
                 "contrast_betas", "contrast_tstats", "residuals", "residuals_whitened",
                 "predicted", "reml_lklhd_surface"):
        ref = getattr(per[groups[0]][1], attr)
        if ref is None:
            continue
        full = np.zeros((Y.shape[0],) + ref.shape[1:], dtype=ref.dtype)
        for h in groups:
            m, r = per[h]
            full[m] = getattr(r, attr)
        setattr(merged, attr, full)
    merged.ljung_box_dof = per[groups[0]][1].ljung_box_dof
    merged.extra["grid"] = grid
    return merged


# ------------------------------------------------------------------ criterion


def criterion_surface(X, Y, grid: Grid, run_starts=None, tau=None, scaled=True):
    """FP64 criterion surface (V, P) of float32 data, for gap checks on disagreements.

    With ``scaled`` the data are divided by their float32 std first, which is the
    float32 mode's likelihood scale (fastfuncstuff/glm/arma.py:4685-4686).
    """
    Y = np.asarray(Y)
    Yd = Y.astype(F64)
    if scaled:
        s = np.maximum(np.std(Yd, axis=1, ddof=1).astype(F32), F32(1e-8)).astype(F64)
        Yd = Yd / s[:, None]
    grid = valid_grid(grid.a_axis, grid.b_axis, F64) if grid.lam.dtype != F64 else grid
    pre = precompute_reml_grid(np.asarray(X, F64), grid, run_starts, tau, F64)
    _, _, surf = search_exhaustive(np.asarray(X, F64), Yd, pre, return_surface=True)
    return surf
