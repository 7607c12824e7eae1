"""NumPy model of the search kernels' arithmetic, driven by the host structures.

Restates, in float32 where the kernels use float32, what ``grid_build.cu`` (the
tridiagonal LDL' coefficients, with the identity for lambda == 0),
``search.cu`` (the surface recurrence per chunk with the chunk's shared AR
filter, the criterion relative to the pair (0, 0), the selectors) compute, using
the product's own ``RemlGrid`` (chunks, lattice, p0). CPU tests run it against
the FP64 oracle, so a contract bug between host and kernels shows up without a
GPU.
"""

from __future__ import annotations

import numpy as np

F32 = np.float32


def coefficients(a: float, b: float, tau: np.ndarray, run_start: np.ndarray) -> np.ndarray:
    """(T, 4) float32 (c, m, 1/D, 1/sqrt(D)) as grid_build.cu phase 1 computes them."""
    a64, b64 = float(np.float32(a)), float(np.float32(b))
    lam = (a64 + b64) * (1 + a64 * b64) / ((1 + b64 * b64) + (2 * a64) * b64)
    T = tau.shape[0]
    out = np.zeros((T, 4))
    for r in range(run_start.shape[0] - 1):
        t0, t1 = int(run_start[r]), int(run_start[r + 1])
        Dp = 1.0
        for t in range(t0, t1):
            c = m = 0.0
            D = 1.0
            if t > t0 and lam != 0.0:
                gap = int(tau[t] - tau[t - 1])
                c = a64**gap
                rho = lam * a64 ** (gap - 1)
                Ttt = 1.0 + c * c - 2.0 * c * rho
                Toff = rho - c
                m = Toff / Dp
                D = Ttt - m * Toff
            out[t] = (c, m, 1.0 / D, 1.0 / np.sqrt(D))
            Dp = D
    return out.astype(F32)


def surface(yr: np.ndarray, grid, coef: np.ndarray, proj: np.ndarray, const: np.ndarray, K: int):
    """d[p][v] and crit0[v] as surface_kernel computes them (float32 recurrences)."""
    V, T = yr.shape
    P = grid.P
    d = np.zeros((P, V), F32)
    yy = np.zeros(V, F32)
    st_all = np.zeros((P, V), F32)
    TB = 16  # steps per sample block (SURF_TB)
    for c in range(len(grid.chunk_start) - 1):
        slots = grid.chunk_pairs[grid.chunk_start[c] : grid.chunk_start[c + 1]]
        members = slots[slots >= 0]
        cs = coef[members, :, 0][:, :, None]  # each pair's own AR filter (shared per quarter)
        v = np.zeros((len(members), V), F32)
        sb = np.zeros((len(members), V), F32)
        st = np.zeros((len(members), V), F32)
        yp = np.zeros(V, F32)
        yyb = np.zeros(V, F32)
        yyt = np.zeros(V, F32)
        # steady[t]: every member's coefficients equal step t-1's; a block of
        # TB steady steps sums v^2 alone and scales the block sum by 1/D once
        cm = coef[members]
        steady = np.zeros(T, bool)
        steady[1:] = (cm[:, 1:, :3] == cm[:, :-1, :3]).all(axis=(0, 2))
        for t0 in range(0, T, TB):
            block_steady = t0 + TB <= T and bool(steady[t0 : t0 + TB].all())
            iD = coef[members, t0, 2][:, None]
            for t in range(t0, min(T, t0 + TB)):
                y = yr[:, t]
                z = (y[None, :] - cs[:, t] * yp[None, :]).astype(F32)
                yp = y
                yyb = (yyb + y * y).astype(F32)
                m = coef[members, t, 1][:, None]
                v = (z - m * v).astype(F32)
                if block_steady:
                    sb = (sb + v * v).astype(F32)
                else:
                    iD = coef[members, t, 2][:, None]
                    sb = (sb + (v * iD).astype(F32) * v).astype(F32)
            st = (st + sb * iD).astype(F32) if block_steady else (st + sb).astype(F32)
            sb[:] = 0
            yyt = (yyt + yyb).astype(F32)
            yyb[:] = 0
        st_all[members] = st
        yy = yyt
    Tk = T - K
    c0 = const[grid.p0]
    rss0 = np.maximum(yy - proj[grid.p0], 0).astype(F32)
    den = (rss0 + F32(1e-10)).astype(F32)
    for p in range(P):
        rss = np.maximum(st_all[p] - proj[p], 0).astype(F32)
        dc = F32(const[p] - c0)
        d[p] = (dc + F32(Tk) * np.log1p(((rss - rss0) / den).astype(F32))).astype(F32)
    crit0 = c0 + Tk * np.log(rss0.astype(np.float64) + 1e-10)
    return d, crit0


def select_exhaustive(d: np.ndarray, grid) -> np.ndarray:
    """First strict minimum in pair order (select_kernel, exhaustive mode)."""
    best = np.full(d.shape[1], grid.p0)
    bl = np.full(d.shape[1], np.inf, F32)
    for p in range(d.shape[0]):
        imp = d[p] < bl
        bl[imp] = d[p][imp]
        best[imp] = p
    return best
