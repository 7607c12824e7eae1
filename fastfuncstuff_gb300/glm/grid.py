"""Host-side description of the REML (a, b) grid and the run structure.

These are the small pieces of setup the kernels need: which pairs are valid, in
what order, where each pair sits on the (a, b) lattice, and how the runs and
censoring gaps lay out the time axis. They follow the reference's semantics
exactly (same float32 / float64 arithmetic for the validity filter and lambda),
so the pair list -- and therefore every index the kernels return -- is the
reference's ``param_list``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

# AFNI 3dREMLfit defaults (-MAXa 0.8 -MAXb 0.8 -Grid 3): a in [0, 0.8] step 0.1,
# b in [-0.8, 0.8] step 0.1 (fastfuncstuff/glm/arma.py:234-243).
DEFAULT_ARMA_A_GRID = (0.0, 0.8, 9)
DEFAULT_ARMA_B_GRID = (-0.8, 0.8, 17)

SURFACE_CHUNK = 16  # pair slots per surface-kernel chunk (csrc/search.cu SURF_G)
SURFACE_QUARTER = 4  # slots per quarter: pairs of one quarter share one AR filter


class _RemlMode:
    """Run-wide REML mode (AFNI-faithful switches), as in fastfuncstuff/glm/arma.py:59-92."""

    afni_faithful: bool = False
    corcut: float = 1e-4


_REML_MODE = _RemlMode()


def set_afni_mode(enabled: bool, corcut: float = 1e-4) -> None:
    """Toggle AFNI-faithful REML behaviour (fastfuncstuff/glm/arma.py:85-92)."""
    _REML_MODE.afni_faithful = bool(enabled)
    _REML_MODE.corcut = float(corcut)


def get_default_arma_grids(device=None) -> tuple[torch.Tensor, torch.Tensor]:
    """AFNI's default grids. Follows fastfuncstuff/glm/arma.py:484-513."""
    return (torch.linspace(*DEFAULT_ARMA_A_GRID, device=device),
            torch.linspace(*DEFAULT_ARMA_B_GRID, device=device))


def parse_grid_arg(grid_str: str) -> torch.Tensor:
    """A -a_grid / -b_grid argument as a 1-D float32 tensor, read as
    fastfuncstuff/cli/reml.py:115-160 reads it:

    * ``start:stop:num``  linspace (num >= 2), e.g. ``-0.9:0.9:65``;
    * ``start,stop,num``  linspace, when there are exactly three values and the
      last is a whole number >= 2 (the legacy form);
    * ``v1,v2,...``       the values themselves.

    A malformed argument prints ``ERROR: ...`` and exits with status 1, as the
    reference's command line does.
    """
    import sys

    def fail(msg: str):
        print(f"ERROR: {msg}")
        sys.exit(1)

    s = grid_str.strip()
    if ":" in s:
        parts = s.split(":")
        if len(parts) != 3:
            fail(f"colon range must be start:stop:num, got '{s}'")
        try:
            start, stop, num = float(parts[0]), float(parts[1]), int(parts[2])
        except ValueError:
            fail(f"could not parse the range '{s}'")
        if num < 2:
            fail(f"num_points must be >= 2 in '{s}'")
        return torch.linspace(start, stop, num)
    try:
        values = [float(p) for p in s.split(",")]
    except ValueError:
        fail(f"could not parse grid values '{s}'")
    if len(values) == 3 and values[2].is_integer() and values[2] >= 2:
        return torch.linspace(values[0], values[1], int(values[2]))
    return torch.tensor(values, dtype=torch.float32)


def _as_f32_cpu(g) -> torch.Tensor:
    if isinstance(g, torch.Tensor):
        return g.detach().to(device="cpu", dtype=torch.float32).reshape(-1)
    return torch.as_tensor(np.asarray(g), dtype=torch.float32).reshape(-1)


def ensure_zero_in_grid(a_grid, b_grid, tolerance: float = 1e-6):
    """Snap a near-zero value to 0.0 or insert 0.0. Follows fastfuncstuff/glm/arma.py:516-582."""

    def one(g):
        g = _as_f32_cpu(g)
        near = torch.abs(g) < tolerance
        if bool(near.any()):
            g = g.clone()
            g[near] = 0.0
        else:
            g = torch.sort(torch.cat([torch.zeros(1), g]))[0]
        return g

    return one(a_grid), one(b_grid)


def compute_arma_lambda(a, b):
    """lambda = (a+b)(1+ab)/(1+b^2+2ab). Follows fastfuncstuff/glm/arma.py:695-729."""
    return (a + b) * (1 + a * b) / (1 + b**2 + 2 * a * b)


def _valid_mask(a: torch.Tensor, b: torch.Tensor, afni: bool, corcut: float):
    # the filter of fastfuncstuff/glm/arma.py:989-1040, evaluated in a's dtype
    ok = (torch.abs(a) < 1.0) & (torch.abs(b) < 1.0)
    denom = 1 - a**2
    ok &= torch.abs(denom) >= 1e-6
    gamma0 = (1 + b**2 + 2 * a * b) / (denom + 1e-10)
    ok &= gamma0 > 0
    lam = compute_arma_lambda(a, b)
    ok &= lam >= 0
    if afni:
        ok &= (lam == 0) | (lam >= corcut)
    return ok


def afni_band(a: float, lam: float, corcut: float) -> int:
    """The off-diagonals AFNI keeps in R (its rcmat_arma11): the lag at which
    lam rho^(k-1), rho = a clamped to [-0.9, 0.9], has fallen to corcut; 0
    (R = I) when |lam| < corcut, 1 for a pure MA(1) (a = 0). Follows
    fastfuncstuff/glm/arma.py:95-109 in Python floats, as the reference
    evaluates it."""
    mag = abs(lam)
    if mag < corcut:
        return 0
    rho = max(-0.9, min(0.9, a))
    if rho == 0.0:
        return 1
    return 1 + int(math.ceil(math.log(corcut / mag) / math.log(abs(rho))))


def estimate_valid_grid_pairs(a_grid, b_grid) -> int:
    """Number of valid pairs. Follows fastfuncstuff/glm/arma.py:291-338."""
    a, b = torch.meshgrid(_as_f32_cpu(a_grid), _as_f32_cpu(b_grid), indexing="ij")
    return int(_valid_mask(a.reshape(-1), b.reshape(-1), False, 0.0).sum())


@dataclass
class RemlGrid:
    """The valid pairs in ``param_list`` order and their lattice."""

    a: np.ndarray          # (P,) float32
    b: np.ndarray          # (P,) float32
    a_axis: np.ndarray     # sorted unique a of the valid pairs
    b_axis: np.ndarray
    lattice: np.ndarray    # (n_a, n_b) int32 pair index, -1 where filtered
    p0: int                # index of (0, 0)
    za: int
    zb: int
    ltop: int
    chunk_start: np.ndarray  # (n_chunks + 1,) int32
    chunk_pairs: np.ndarray  # int32 pair slots of each chunk (-1: empty), one AR filter per quarter
    lambda_fp32: bool
    band: np.ndarray | None = None  # AFNI-faithful mode: int32 band of R per pair (afni_band)

    @property
    def P(self) -> int:
        return int(self.a.shape[0])

    def param_list(self) -> list[tuple[float, float]]:
        return [(float(x), float(y)) for x, y in zip(self.a, self.b)]

    def index_of(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        """Pair index of each (a, b) (exact float32 match), -1 if absent."""
        ai = np.searchsorted(self.a_axis, np.asarray(a, np.float32))
        bi = np.searchsorted(self.b_axis, np.asarray(b, np.float32))
        ai_c = np.clip(ai, 0, len(self.a_axis) - 1)
        bi_c = np.clip(bi, 0, len(self.b_axis) - 1)
        hit = (self.a_axis[ai_c] == a) & (self.b_axis[bi_c] == b)
        return np.where(hit, self.lattice[ai_c, bi_c], -1)


def lambda_is_zero(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """lambda == 0 exactly in float64 (a + b of two float32 values is exact)."""
    return (np.asarray(a, np.float64) + np.asarray(b, np.float64)) == 0.0


def coefficient_chunks(a: np.ndarray, b: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Chunks of SURFACE_CHUNK pair slots for the surface kernel.

    Pairs sharing a share the AR filter c_t = a^gap; pairs with lambda == 0
    (R = I) use the identity (c = 0) whatever their a, so they form one class
    of their own. Each class is cut into quarters of at most SURFACE_QUARTER
    pairs (padded with -1, an empty slot) and a chunk takes up to four
    quarters, in class order; identity quarters fill chunks of their own, which
    the kernel evaluates as one sum of squares.
    Returns (chunk_start, chunk_pairs): the slots of chunk c are
    chunk_pairs[chunk_start[c] : chunk_start[c + 1]].
    """
    ident = lambda_is_zero(a, b)
    classes: dict = {}
    for p in range(a.size):
        key = "identity" if ident[p] else float(a[p])
        classes.setdefault(key, []).append(p)
    q = SURFACE_QUARTER
    per = SURFACE_CHUNK // q

    def quarters(members):
        out = []
        for i in range(0, len(members), q):
            part = members[i : i + q]
            out.append(part + [-1] * (q - len(part)))
        return out

    idq = quarters(classes.pop("identity", []))
    otherq = [qq for members in classes.values() for qq in quarters(members)]
    starts, slots = [0], []
    for group in (idq, otherq):
        for i in range(0, len(group), per):
            for qq in group[i : i + per]:
                slots.extend(qq)
            starts.append(len(slots))
    return np.asarray(starts, np.int32), np.asarray(slots, np.int32)


def hierarchical_ltop(n_a: int, n_b: int, afni_faithful: bool) -> int:
    """Top level of the power-of-2 descent. Follows fastfuncstuff/glm/arma.py:2109-2115."""
    if afni_faithful:
        pna = (n_a - 1).bit_length() - 1
        pnb = (n_b - 1).bit_length() - 1
        return max(0, min(pna, pnb) - 2)
    return max(0, min(n_a, n_b).bit_length() - 2)


def make_grid(a_grid, b_grid, use_double: bool = False) -> RemlGrid:
    """Valid pairs of the grids, in the reference's order.

    ``ensure_zero_in_grid`` runs on the float32 grids, then the validity filter
    runs in the fit's dtype (float64 under ``use_double``), as
    fastfuncstuff/glm/arma.py:1339-1342 does before ``build_arma11_covariance_batch``.
    """
    ag, bg = ensure_zero_in_grid(a_grid, b_grid)
    key = (ag.numpy().tobytes(), bg.numpy().tobytes(), bool(use_double), _REML_MODE.afni_faithful,
           float(_REML_MODE.corcut))
    hit = _GRID_CACHE.get(key)
    if hit is not None:
        return hit
    dt = torch.float64 if use_double else torch.float32
    am, bm = torch.meshgrid(ag.to(dt), bg.to(dt), indexing="ij")
    a, b = am.reshape(-1), bm.reshape(-1)
    ok = _valid_mask(a, b, _REML_MODE.afni_faithful, _REML_MODE.corcut)
    band = None
    if _REML_MODE.afni_faithful:
        # the band from a and lambda in the fit's dtype (arma.py:1077-1084)
        lam = compute_arma_lambda(a[ok], b[ok])
        band = np.array([afni_band(float(x), float(y), _REML_MODE.corcut)
                         for x, y in zip(a[ok].tolist(), lam.tolist())], dtype=np.int32)
    a = a[ok].to(torch.float32).numpy()
    b = b[ok].to(torch.float32).numpy()
    if a.size == 0:
        raise ValueError("no valid (a, b) pair in the grid")
    a_axis = np.array(sorted(set(a.tolist())), dtype=np.float32)
    b_axis = np.array(sorted(set(b.tolist())), dtype=np.float32)
    lattice = np.full((len(a_axis), len(b_axis)), -1, dtype=np.int32)
    ai = np.searchsorted(a_axis, a)
    bi = np.searchsorted(b_axis, b)
    lattice[ai, bi] = np.arange(a.size, dtype=np.int32)
    za = int(np.nonzero(np.abs(a_axis) < 1e-6)[0][0])
    zb = int(np.nonzero(np.abs(b_axis) < 1e-6)[0][0])
    p0 = int(lattice[za, zb])
    if p0 < 0:
        raise ValueError("the (0, 0) pair is missing from the valid grid")
    chunk_start, chunk_pairs = coefficient_chunks(a, b)
    g = RemlGrid(a=a, b=b, a_axis=a_axis, b_axis=b_axis, lattice=lattice, p0=p0, za=za, zb=zb,
                 ltop=hierarchical_ltop(len(a_axis), len(b_axis), _REML_MODE.afni_faithful),
                 chunk_start=chunk_start, chunk_pairs=chunk_pairs, lambda_fp32=not use_double, band=band)
    if len(_GRID_CACHE) > 64:
        _GRID_CACHE.clear()
    _GRID_CACHE[key] = g
    return g


# grids by (axes, dtype, AFNI mode): the host-side setup of repeated fits
_GRID_CACHE: dict = {}


def grid_of_pairs(a: np.ndarray, b: np.ndarray, use_double: bool = False) -> RemlGrid:
    """A grid holding exactly the given pairs (the GLS of precomputed (a, b))."""
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    dt = torch.float64 if use_double else torch.float32
    lam = compute_arma_lambda(torch.from_numpy(a).to(dt), torch.from_numpy(b).to(dt))
    bad = (np.abs(a) >= 1) | (np.abs(b) >= 1) | (lam < 0).numpy()
    if bad.any():
        i = int(np.nonzero(bad)[0][0])
        raise ValueError(f"Invalid ARMA(1,1) parameters: a={a[i]}, b={b[i]}")
    P = a.size
    lattice = np.arange(P, dtype=np.int32).reshape(P, 1)
    chunk_start, chunk_pairs = coefficient_chunks(a, b)
    return RemlGrid(a=a, b=b, a_axis=a.copy(), b_axis=b.copy(), lattice=lattice, p0=0, za=0, zb=0,
                    ltop=0, chunk_start=chunk_start, chunk_pairs=chunk_pairs, lambda_fp32=not use_double)


# ---------------------------------------------------------------- runs / censor


def run_bounds(n: int, run_starts=None) -> list[tuple[int, int]]:
    """[(start, stop), ...] for each run. Follows fastfuncstuff/glm/whiten.py:27-38."""
    if run_starts is None:
        return [(0, n)]
    vals = run_starts.tolist() if isinstance(run_starts, torch.Tensor) else list(np.asarray(run_starts).reshape(-1))
    starts = sorted({int(s) for s in vals})
    if not starts or starts[0] != 0:
        starts = [0, *starts]
    stops = [*starts[1:], n]
    return [(s, e) for s, e in zip(starts, stops) if e > s]


def build_censor_run_info(run_starts, n_total: int, good_list=None):
    """Retained-space run starts and the within-run time index tau.

    Follows fastfuncstuff/glm/arma.py:752-820.
    """
    starts = run_starts.tolist() if isinstance(run_starts, torch.Tensor) else list(run_starts)
    if good_list is None:
        return [int(s) for s in starts], None
    retained = torch.as_tensor(np.asarray(good_list), dtype=torch.long).flatten()
    st = torch.tensor(starts, dtype=torch.long)
    run_id = torch.bucketize(retained, st, right=True) - 1
    tau = retained - st[run_id]
    out = []
    for r in range(len(starts)):
        pos = (run_id == r).nonzero(as_tuple=False)
        if pos.numel() > 0:
            out.append(int(pos[0].item()))
    return (out or [0]), tau


@dataclass
class RunLayout:
    """Run starts (n_runs + 1 entries, last = T) and the within-run time index."""

    run_start: np.ndarray
    tau: np.ndarray

    @property
    def n_runs(self) -> int:
        return int(self.run_start.shape[0] - 1)


def run_layout(T: int, run_starts=None, tau=None) -> RunLayout:
    bounds = run_bounds(T, run_starts)
    rs = np.asarray([s for s, _ in bounds] + [T], dtype=np.int32)
    if tau is None:
        tt = np.concatenate([np.arange(e - s) for s, e in bounds]).astype(np.int32)
    else:
        tt = np.asarray(tau.cpu().numpy() if isinstance(tau, torch.Tensor) else tau).reshape(-1).astype(np.int64)
        if tt.shape[0] != T:
            raise ValueError(f"tau has {tt.shape[0]} entries for {T} timepoints")
        for s, e in bounds:
            if e - s > 1 and np.any(np.diff(tt[s:e]) < 1):
                raise ValueError("tau must increase strictly within each run")
        tt = tt.astype(np.int32)
    return RunLayout(rs, tt)


# ------------------------------------------------------------------ Ljung-Box

LJ_RUN_SEPARATION = 66666  # fastfuncstuff/glm/arma.py:5968


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
    """ljung_box_uneven's clamp. Follows fastfuncstuff/glm/arma.py:6002-6014."""
    hh = int(max_lag) if max_lag else 0
    if hh < 2 or hh > n_time // 2:
        hh = 2 + min(n_time // 8, int(round(3.0 * math.log(n_time))))
        hh = min(hh, n_time // 2)
    return hh


def build_ljung_box_tau(n_time: int, run_starts=None, tau=None):
    """Pseudo-time with runs pushed far apart. Follows fastfuncstuff/glm/arma.py:6017-6049."""
    vals = [] if run_starts is None else (
        run_starts.tolist() if isinstance(run_starts, torch.Tensor) else list(np.asarray(run_starts).reshape(-1)))
    starts = sorted({int(s) for s in vals if 0 <= int(s) < n_time}) or [0]
    if tau is None and len(starts) == 1 and starts[0] == 0:
        return None
    st = np.asarray(starts, dtype=np.int64)
    idx = np.arange(n_time, dtype=np.int64)
    run_id = np.searchsorted(st, idx, side="right") - 1
    if tau is not None:
        within = np.asarray(tau.cpu().numpy() if isinstance(tau, torch.Tensor) else tau).reshape(-1).astype(np.int64)
    else:
        within = idx - st[run_id]
    return within + LJ_RUN_SEPARATION * run_id


def ljung_box_plan(n_time: int, n_regressors: int, run_starts=None, tau=None):
    """(h, pseudo-time or None, 1/n_k weights, dof) for the GLS kernel's Ljung-Box.

    The bin counts n_k depend only on the time layout, so they are counted here
    once (fastfuncstuff/glm/arma.py:6088-6114); bins with n_k <= 1 get weight 0.
    """
    starts = sorted({int(s) for s in (run_starts.tolist() if isinstance(run_starts, torch.Tensor)
                                     else list(np.asarray(run_starts).reshape(-1)))}) if run_starts is not None else [0]
    mins = min(b - a for a, b in zip(starts, starts[1:] + [n_time])) if len(starts) > 1 else n_time
    h_req = ljung_box_max_lag(n_time, n_regressors, mins)
    dof = max(1, resolve_ljung_box_lag(n_time, h_req) - 2)
    if n_time < 10:
        return 0, None, None, dof
    hh = resolve_ljung_box_lag(n_time, h_req)
    ptau = build_ljung_box_tau(n_time, run_starts, tau)
    nj = np.zeros(hh + 1, dtype=np.int64)
    if ptau is None:
        for k in range(1, hh + 1):
            nj[k] = n_time - k
    else:
        for k in range(1, hh + 1):
            dj = ptau[k:] - ptau[: n_time - k]
            keep = (dj > 0) & (dj <= hh)
            np.add.at(nj, dj[keep], 1)
    w = np.zeros(hh + 1, dtype=np.float32)
    good = nj > 1
    good[0] = False
    w[good] = 1.0 / nj[good]
    ptau32 = None if ptau is None else (ptau - ptau.min()).astype(np.int32)
    return hh, ptau32, w, dof
