"""Seeded synthetic fMRI workloads for the benchmark configurations.

No public dataset is used; these stand in for it with the shapes and value
distributions of the five workloads:

  0  N=200 (1 run), V=20,000, p=8: 2 task + intercept + Legendre 1-3 + 2 N(0,1)
  1  N=400 (2 x 200), V=200,000, p=20: 4 task + 2 x Legendre 0-4 + 6 motion
     random walks (step sd 0.05); (a, b) maps spatially smoothed on a
     64 x 64 x 49 grid inside a 200,000-voxel mask
  2  4 runs of 180/220/240/260 TRs, 5% of frames censored per run (855 kept),
     V=150,000, p=18: 2 task + 4 x Legendre 0-3; 20 HRF groups (gamma shape
     4-7 s, undershoot ratio 0.1-0.4), voxels assigned by Zipf(1.2) truncated
     to 20
  3  N=600 (3 x 200), V=150,000, p=130: 120 single-event columns (1 s events,
     ISI U(3, 8) s) + 3 x Legendre 0-2 + 1 N(0,1)
  4  the workload-1 design family at V=500,000 (inference of the learned
     proposal)

Conventions restated from the reference: TR 2 s; double-gamma HRF as a
difference of gamma densities (shape 6 and 16, scale 1, undershoot ratio 1/6 by
default) on a 0.1 s grid, normalised to unit area (fastfuncstuff/design/
hrf.py:1302-1386); 1 s boxcar events convolved at 0.1 s and sampled at TR;
Legendre drift per run on [-1, 1] (fastfuncstuff/glm/core.py:140-176);
ARMA(1,1) noise y_t = a y_{t-1} + e_t + b e_{t-1} with 200 burn-in samples,
then standardised (fastfuncstuff/simulation/noise.py:650-762); Y = X beta +
sigma * noise, beta ~ N(0,1), a ~ U(0.1, 0.8), b ~ U(-0.5, 0.3),
sigma ~ U(0.5, 2). The generator is numpy PCG64 seeded with 1000 + workload id.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

TR = 2.0


def double_gamma_hrf(tr: float = TR, shape1: float = 6.0, shape2: float = 16.0, ratio: float = 1.0 / 6.0,
                     dt: float = 0.1, duration: float = 32.0) -> np.ndarray:
    """Difference of two unit-scale gamma densities on a dt grid, unit area."""
    from scipy.stats import gamma

    t = np.arange(0.0, duration, dt)
    h = gamma.pdf(t, shape1) - ratio * gamma.pdf(t, shape2)
    s = h.sum() * dt
    return h / s if s > 0 else h


def event_regressor(n_time: int, onsets_s: np.ndarray, hrf: np.ndarray, tr: float = TR, dt: float = 0.1,
                    dur: float = 1.0) -> np.ndarray:
    """1 s boxcars at ``onsets_s`` convolved with ``hrf`` at dt, sampled every TR."""
    n_fine = int(round(n_time * tr / dt))
    box = np.zeros(n_fine)
    w = int(round(dur / dt))
    for o in onsets_s:
        i = int(round(o / dt))
        box[i : min(n_fine, i + w)] = 1.0
    conv = np.convolve(box, hrf)[:n_fine] * dt
    step = int(round(tr / dt))
    return conv[::step][:n_time]


def legendre(n: int, deg: int, lo: int = 0) -> np.ndarray:
    x = np.linspace(-1.0, 1.0, n)
    return np.stack([np.polynomial.legendre.Legendre.basis(d)(x) for d in range(lo, deg + 1)], 1)


def block_drift(lens: list[int], deg: int) -> np.ndarray:
    n = sum(lens)
    out = np.zeros((n, len(lens) * (deg + 1)))
    s = 0
    for r, m in enumerate(lens):
        out[s : s + m, r * (deg + 1) : (r + 1) * (deg + 1)] = legendre(m, deg)
        s += m
    return out


def arma_noise(rng: np.random.Generator, n: int, a: np.ndarray, b: np.ndarray, burn: int = 200,
               chunk: int = 65536) -> np.ndarray:
    """(V, n) float32 ARMA(1,1) noise, standardised per voxel (burn >= 1)."""
    V = a.shape[0]
    out = np.empty((V, n), dtype=np.float32)
    for v0 in range(0, V, chunk):
        v1 = min(V, v0 + chunk)
        av, bv = a[v0:v1], b[v0:v1]
        e_prev = rng.standard_normal(v1 - v0)
        y = e_prev.copy()
        blk = np.empty((n, v1 - v0))
        for t in range(1, n + burn):
            e = rng.standard_normal(v1 - v0)
            y = av * y + e + bv * e_prev
            e_prev = e
            if t >= burn:
                blk[t - burn] = y
        blk = (blk - blk.mean(0)) / blk.std(0, ddof=1)
        out[v0:v1] = blk.T
    return out


def _random_onsets(rng, n_time, n_events, tr=TR):
    total = n_time * tr
    return np.sort(rng.uniform(0.0, total - 30.0, n_events))


def _smooth_maps(rng, shape, n_keep, lo_hi_list, sigma=2.0):
    """Spatially smooth uniform maps on ``shape``, kept inside a centred mask."""
    from scipy.ndimage import gaussian_filter
    from scipy.special import ndtr

    zz, yy, xx = np.meshgrid(*[np.arange(s) - (s - 1) / 2 for s in shape], indexing="ij")
    r = (zz / shape[0]) ** 2 + (yy / shape[1]) ** 2 + (xx / shape[2]) ** 2
    mask_idx = np.argsort(r.reshape(-1), kind="stable")[:n_keep]
    maps = []
    for lo, hi in lo_hi_list:
        f = gaussian_filter(rng.standard_normal(shape), sigma)
        f = (f - f.mean()) / f.std()
        maps.append((lo + (hi - lo) * ndtr(f)).reshape(-1)[mask_idx])
    return maps, mask_idx


def workload1_design(seed: int) -> np.ndarray:
    """A fresh design of the 200k-voxel workload's kind, (400, 20) float32:
    2 runs x 200 TRs, 4 task regressors (20-30 random 1 s events each,
    double-gamma HRF), a Legendre 0-4 drift per run and 6 motion random walks
    (step sigma 0.05), from its own seeded generator (a family of such designs
    trains a proposal that serves designs it has not seen)."""
    rng = np.random.default_rng(np.random.PCG64(seed))
    hrf = double_gamma_hrf()
    n, lens = 400, [200, 200]
    task = [event_regressor(n, _random_onsets(rng, n, rng.integers(20, 31)), hrf) for _ in range(4)]
    motion = np.cumsum(rng.normal(0.0, 0.05, (n, 6)), axis=0)
    return np.column_stack(task + [block_drift(lens, 4), motion]).astype(np.float32)


@dataclass
class Workload:
    X: np.ndarray                # (T, K) float32 design (one group) or None
    Y: np.ndarray                # (V, T) float32
    a_true: np.ndarray
    b_true: np.ndarray
    run_starts: list[int] | None
    tau: np.ndarray | None
    designs: dict | None = None  # grouped designs (workload 2)
    groups: np.ndarray | None = None
    name: str = ""

    @property
    def V(self) -> int:
        return self.Y.shape[0]

    @property
    def T(self) -> int:
        return self.Y.shape[1]


def workload(cid: int, V: int | None = None, seed: int | None = None) -> Workload:
    """The seeded synthetic workload ``cid`` (0-4), optionally with fewer voxels."""
    rng = np.random.default_rng(np.random.PCG64(1000 + cid if seed is None else seed))
    hrf = double_gamma_hrf()
    if cid == 0:
        V = V or 20_000
        n = 200
        task = [event_regressor(n, _random_onsets(rng, n, rng.integers(20, 31)), hrf) for _ in range(2)]
        X = np.column_stack(task + [np.ones(n), legendre(n, 3, lo=1), rng.standard_normal((n, 2))])
        a = rng.uniform(0.1, 0.8, V)
        b = rng.uniform(-0.5, 0.3, V)
        noise = arma_noise(rng, n, a, b)
        runs, tau, name = None, None, "N=200 V=20k p=8 (1 run)"
    elif cid in (1, 4):
        V = V or (200_000 if cid == 1 else 500_000)
        lens = [200, 200]
        n = 400
        task = [event_regressor(n, _random_onsets(rng, n, rng.integers(20, 31)), hrf) for _ in range(4)]
        motion = np.cumsum(rng.normal(0.0, 0.05, (n, 6)), axis=0)
        X = np.column_stack(task + [block_drift(lens, 4), motion])
        n_vol = 64 * 64 * 49
        if V <= n_vol:
            (a, b), _ = _smooth_maps(rng, (49, 64, 64), V, [(0.1, 0.8), (-0.5, 0.3)])
        else:
            reps = -(-V // 200_000)
            parts = [_smooth_maps(rng, (49, 64, 64), 200_000, [(0.1, 0.8), (-0.5, 0.3)])[0] for _ in range(reps)]
            a = np.concatenate([p[0] for p in parts])[:V]
            b = np.concatenate([p[1] for p in parts])[:V]
        noise = np.concatenate([arma_noise(rng, 200, a, b), arma_noise(rng, 200, a, b)], axis=1)
        runs, tau = [0, 200], None
        name = f"N=400 (2x200) V={V // 1000}k p=20"
    elif cid == 2:
        V = V or 150_000
        lens = [180, 220, 240, 260]
        cens = [9, 11, 12, 13]
        n_full = sum(lens)
        a = rng.uniform(0.1, 0.8, V)
        b = rng.uniform(-0.5, 0.3, V)
        noise_full = np.concatenate([arma_noise(rng, m, a, b) for m in lens], axis=1)
        keep, s = [], 0
        for m, c in zip(lens, cens):
            drop = set(rng.choice(m, c, replace=False).tolist())
            keep += [s + i for i in range(m) if i not in drop]
            s += m
        keep = np.asarray(keep)
        from .glm.grid import build_censor_run_info

        run_starts_full = np.cumsum([0] + lens[:-1]).tolist()
        runs, tau_t = build_censor_run_info(run_starts_full, n_full, keep.tolist())
        tau = tau_t.numpy()
        onsets = [_random_onsets(rng, n_full, rng.integers(40, 61)) for _ in range(2)]
        drift = block_drift(lens, 3)
        designs = {}
        for h in range(20):
            hh = double_gamma_hrf(shape1=rng.uniform(4.0, 7.0), ratio=rng.uniform(0.1, 0.4))
            task = [event_regressor(n_full, o, hh) for o in onsets]
            designs[h] = np.column_stack(task + [drift])[keep].astype(np.float32)
        zipf = 1.0 / np.arange(1, 21) ** 1.2
        groups = rng.choice(20, V, p=zipf / zipf.sum())
        beta = rng.standard_normal((V, 18))
        sig = rng.uniform(0.5, 2.0, V)
        Y = np.empty((V, keep.size), dtype=np.float32)
        for h in range(20):
            m = groups == h
            Y[m] = beta[m] @ designs[h].T + sig[m, None] * noise_full[m][:, keep]
        return Workload(None, Y, a, b, runs, tau, designs, groups.astype(np.int64),
                        "N=855 (4 runs, censored) V=150k p=18, 20 HRF groups")
    elif cid == 3:
        V = V or 150_000
        lens = [200, 200, 200]
        n = 600
        t_ev, onsets = 10.0, []
        while len(onsets) < 120:
            onsets.append(t_ev)
            t_ev += 1.0 + rng.uniform(3.0, 8.0)
        scale = (n * TR - 40.0) / onsets[-1]
        onsets = np.asarray(onsets) * min(1.0, scale)
        single = [event_regressor(n, [o], hrf) for o in onsets]
        X = np.column_stack(single + [block_drift(lens, 2), rng.standard_normal(n)])
        a = rng.uniform(0.1, 0.8, V)
        b = rng.uniform(-0.5, 0.3, V)
        noise = np.concatenate([arma_noise(rng, 200, a, b) for _ in lens], axis=1)
        runs, tau, name = [0, 200, 400], None, "N=600 (3x200) V=150k p=130 single-trial"
    else:
        raise ValueError(f"unknown workload {cid}")
    X = X.astype(np.float32)
    beta = rng.standard_normal((V, X.shape[1]))
    sig = rng.uniform(0.5, 2.0, (V, 1))
    Y = (beta @ X.T.astype(np.float64) + sig * noise).astype(np.float32)
    return Workload(X, Y, a, b, runs, tau, name=name)
