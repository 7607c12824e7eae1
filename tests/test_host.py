"""Host-side logic of the product path, checked on the CPU against the oracle."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from fastfuncstuff_gb300 import synth
from fastfuncstuff_gb300.glm import grid as G
from fastfuncstuff_gb300.glm.arma import fit_glm_arma11, fit_glm_arma11_grouped
from oracle import reml as o
from tests.conftest import load_golden


@pytest.mark.parametrize("use_double", [False, True])
@pytest.mark.parametrize(
    "grids",
    [
        (torch.linspace(-0.8, 0.8, 33), torch.linspace(-0.8, 0.8, 33)),
        (torch.linspace(0.0, 0.8, 9), torch.linspace(-0.8, 0.8, 17)),
        (torch.linspace(-0.8, 0.8, 17), torch.linspace(-0.8, 0.8, 17)),
        (torch.tensor([0.1, 0.3, 0.5]), torch.tensor([-0.2, 0.2])),  # zero inserted
        (torch.linspace(-0.95, 0.95, 39), torch.linspace(-0.95, 0.95, 39)),
    ],
)
def test_grid_matches_oracle(grids, use_double):
    a, b = grids
    g = G.make_grid(a, b, use_double=use_double)
    og = o.valid_grid(a.numpy(), b.numpy(), np.float64 if use_double else np.float32)
    np.testing.assert_array_equal(g.a, og.a)
    np.testing.assert_array_equal(g.b, og.b)
    np.testing.assert_array_equal(g.a_axis, og.a_axis)
    assert g.a[g.p0] == 0 and g.b[g.p0] == 0
    assert g.ltop == o._ltop(len(og.a_axis), len(og.b_axis))
    # lattice round trip and chunks that share a
    for p in range(g.P):
        ai = np.searchsorted(g.a_axis, g.a[p])
        bi = np.searchsorted(g.b_axis, g.b[p])
        assert g.lattice[ai, bi] == p
    # every quarter shares one AR filter: one a, or only lambda == 0 pairs
    # (identity); identity quarters never share a chunk with other quarters
    ident = G.lambda_is_zero(g.a, g.b)
    Q = G.SURFACE_QUARTER
    for c in range(len(g.chunk_start) - 1):
        s, e = g.chunk_start[c], g.chunk_start[c + 1]
        assert 0 < e - s <= G.SURFACE_CHUNK and (e - s) % Q == 0
        slots = g.chunk_pairs[s:e]
        filled = slots[slots >= 0]
        assert filled.size > 0
        assert ident[filled].all() or not ident[filled].any()
        for q0 in range(0, e - s, Q):
            members = slots[q0 : q0 + Q]
            members = members[members >= 0]
            assert members.size > 0
            if not ident[members].any():
                assert len(set(g.a[members].tolist())) == 1
    filled = g.chunk_pairs[g.chunk_pairs >= 0]
    assert sorted(filled.tolist()) == list(range(g.P))
    assert ident[g.p0]


def test_grid_counts_and_default():
    assert G.estimate_valid_grid_pairs(torch.linspace(-0.8, 0.8, 33), torch.linspace(-0.8, 0.8, 33)) == 561
    a, b = G.get_default_arma_grids()
    assert G.make_grid(a, b).P == G.estimate_valid_grid_pairs(a, b)
    assert 100 < G.make_grid(a, b).P < 153


def test_index_of_pairs():
    g = G.make_grid(torch.linspace(-0.8, 0.8, 17), torch.linspace(-0.8, 0.8, 17))
    idx = g.index_of(g.a, g.b)
    np.testing.assert_array_equal(idx, np.arange(g.P))
    assert g.index_of(np.array([0.05], np.float32), np.array([0.0], np.float32))[0] == -1


def test_grid_of_pairs_rejects_invalid():
    with pytest.raises(ValueError, match="Invalid ARMA"):
        G.grid_of_pairs(np.array([0.5], np.float32), np.array([-0.7], np.float32))  # lambda < 0
    with pytest.raises(ValueError):
        G.grid_of_pairs(np.array([1.0], np.float32), np.array([0.0], np.float32))


def test_run_layout_and_censoring():
    lay = G.run_layout(10, [0, 5])
    assert lay.run_start.tolist() == [0, 5, 10]
    assert lay.tau.tolist() == [0, 1, 2, 3, 4, 0, 1, 2, 3, 4]
    starts, tau = G.build_censor_run_info([0, 5], 10, [0, 1, 3, 4, 5, 6, 8, 9])
    assert starts == [0, 4] and tau.tolist() == [0, 1, 3, 4, 0, 1, 3, 4]
    lay = G.run_layout(8, starts, tau)
    assert lay.run_start.tolist() == [0, 4, 8] and lay.tau.tolist() == [0, 1, 3, 4, 0, 1, 3, 4]
    with pytest.raises(ValueError):
        G.run_layout(4, None, np.array([0, 2, 2, 3]))
    assert G.run_bounds(10, [4]) == [(0, 4), (4, 10)]


@pytest.mark.parametrize("case", ["multirun", "censored", "single"])
def test_ljung_box_plan_matches_oracle_binning(case):
    d = load_golden(case)
    T, K = d["X"].shape
    rs = d["run_starts"] if "run_starts" in d else None
    tau = d["tau"] if "tau" in d else None
    h, ptau, w, dof = G.ljung_box_plan(T, K, rs, tau)
    starts = sorted(set(np.asarray(rs).tolist())) if rs is not None else [0]
    mins = min(b - a for a, b in zip(starts, starts[1:] + [T])) if len(starts) > 1 else T
    assert h == o.resolve_ljung_box_lag(T, o.ljung_box_max_lag(T, K, mins))
    assert dof == max(1, h - 2)
    # the weighted statistic from the plan equals the oracle's on random residuals
    r = np.random.default_rng(0).standard_normal((3, T))
    want = o.ljung_box(r, o.ljung_box_max_lag(T, K, mins), o.build_ljung_box_tau(T, rs, tau))
    got = []
    for row in r:
        s0 = (row**2).sum()
        bins = np.zeros(h + 1)
        for k in range(1, h + 1):
            for t in range(T - k):
                dj = (ptau[t + k] - ptau[t]) if ptau is not None else k
                if 0 < dj <= h:
                    bins[dj] += row[t] * row[t + k]
        got.append(T * (T + 2.0) * ((bins / s0) ** 2 * w).sum())
    np.testing.assert_allclose(got, want, rtol=1e-6)  # float32 1/n_k weights


def test_fit_argument_errors_raise_before_gpu():
    with pytest.raises(ValueError, match="2D or 4D"):
        fit_glm_arma11(np.zeros((2, 3, 10), np.float32), np.ones((10, 2)), tr=2.0)
    with pytest.raises(ValueError, match="Timepoints mismatch"):
        fit_glm_arma11(np.zeros((2, 10), np.float32), np.ones((9, 2)), tr=2.0)
    with pytest.raises(NotImplementedError):
        fit_glm_arma11(np.zeros((2, 10), np.float32), np.ones((10, 2)), tr=2.0, want_ols=True)


def test_grouped_argument_errors():
    Y = np.zeros((4, 10), np.float32)
    with pytest.raises(KeyError):
        fit_glm_arma11_grouped(Y, {0: np.ones((10, 2))}, [0, 0, 1, 1], tr=2.0)
    with pytest.raises(ValueError):
        fit_glm_arma11_grouped(Y, {0: np.ones((10, 2)), 1: np.ones((10, 3))}, [0, 0, 1, 1], tr=2.0)


def test_synthetic_workloads_are_seeded_and_shaped():
    w0 = synth.workload(0, V=300)
    w0b = synth.workload(0, V=300)
    np.testing.assert_array_equal(w0.Y, w0b.Y)
    assert w0.Y.shape == (300, 200) and w0.X.shape == (200, 8)
    w1 = synth.workload(1, V=500)
    assert w1.Y.shape == (500, 400) and w1.X.shape == (400, 20) and w1.run_starts == [0, 200]
    w2 = synth.workload(2, V=400)
    assert w2.Y.shape == (400, 855) and len(w2.designs) == 20
    assert all(d.shape == (855, 18) for d in w2.designs.values())
    assert w2.run_starts == [0, 171, 380, 608] and w2.tau.shape == (855,)
    w3 = synth.workload(3, V=200)
    assert w3.Y.shape == (200, 600) and w3.X.shape == (600, 130)
    assert np.linalg.matrix_rank(w3.X.astype(np.float64)) == 130
    # the noise follows y_t = a y_{t-1} + e_t + b e_{t-1}: lag-1 autocorrelation ~ lambda
    rng = np.random.default_rng(5)
    n = synth.arma_noise(rng, 4000, np.full(4, 0.6), np.full(4, 0.2))
    r1 = (n[:, 1:] * n[:, :-1]).mean(1)
    lam = (0.6 + 0.2) * (1 + 0.12) / (1 + 0.04 + 0.24)
    np.testing.assert_allclose(r1, lam, atol=0.06)


@pytest.mark.parametrize("case", ["single", "multirun", "censored"])
def test_kernel_model_with_host_structures_matches_oracle(case):
    """The kernels' float32 arithmetic, driven by the product's grid/chunks/runs,
    selects what the FP64 oracle selects (exact ties included)."""
    from tests import kernel_model as km

    d = load_golden(case)
    X, Y = d["X"].astype(np.float64), d["Y"].astype(np.float64)
    T, K = X.shape
    rs = d["run_starts"] if "run_starts" in d else None
    tau = d["tau"] if "tau" in d else None
    g = G.make_grid(d["a_grid"], d["b_grid"])
    lay = G.run_layout(T, rs, tau)
    og = o.valid_grid(d["a_grid"], d["b_grid"], np.float64)
    pre = o.precompute_reml_grid(X, og, rs, tau)
    s = np.maximum(np.std(Y, axis=1, ddof=1).astype(np.float32), np.float32(1e-8)).astype(np.float64)
    Ys = Y / s[:, None]
    _, _, surf64 = o.search_exhaustive(X, Ys, pre, return_surface=True)
    Q0, _ = np.linalg.qr(X)
    yr = (Ys - (Ys @ Q0) @ Q0.T).astype(np.float32)
    coef = np.stack([km.coefficients(g.a[p], g.b[p], lay.tau, lay.run_start) for p in range(g.P)])
    proj = np.stack([((yr.astype(np.float64) @ (pre.whiteners[p].dense().T @ pre.Q[p])) ** 2).sum(1)
                     for p in range(g.P)]).astype(np.float32)
    const = pre.logdet_R + pre.logdet_XtX
    dd, crit0 = km.surface(yr, g, coef, proj, const, K)
    best = km.select_exhaustive(dd, g)
    ref = np.argmin(surf64, axis=1)
    agree = (best == ref).mean()
    assert agree >= 0.99, agree
    bad = best != ref
    gap = np.abs(surf64[bad, best[bad]] - surf64[bad, ref[bad]]) / np.abs(surf64[bad, ref[bad]])
    assert gap.size == 0 or gap.max() <= 1e-6


def test_design_slots_layout():
    """Grouped-fit slots: each design's voxels contiguous and padded to 256
    slots, every voxel in exactly one slot, the projection work list covering
    every (slot tile of 128, pair) once with the design's U rows."""
    from fastfuncstuff_gb300.glm import engine

    rng = np.random.default_rng(3)
    D, K, P = 5, 18, 561
    gid = rng.choice(D, 3001, p=[0.5, 0.2, 0.15, 0.1, 0.05])
    gid[gid == 3] = 4  # one design without voxels
    s = engine.design_slots(gid, D, K, P, "cpu")
    idx = s.idx.numpy()
    assert s.Vp % 256 == 0 and s.Vp == idx.size
    real = idx >= 0
    assert np.array_equal(np.sort(idx[real]), np.arange(gid.size))
    assert np.array_equal(idx[s.real.numpy()], np.arange(gid.size))
    design_of_slot = np.repeat(s.tile32.numpy(), 32)
    assert np.array_equal(design_of_slot[s.real.numpy()], gid)
    assert np.array_equal(np.repeat(s.tile256.numpy(), 256), design_of_slot)
    items = s.items.numpy()
    assert int(s.n_items[0]) == items.shape[0] and s.max_pairs * K <= 256
    cover = np.zeros((s.Vp // 128, P), np.int32)
    for v0, nv, row_b, npr, out0, slot0 in items:
        assert nv == 128 and out0 == v0 and 1 <= npr <= s.max_pairs
        d = design_of_slot[v0]
        assert row_b == (d * P + slot0) * K
        cover[v0 // 128, slot0:slot0 + npr] += 1
    assert (cover == 1).all()



def test_column_sets_plan_layout_and_blocks():
    """column_sets as the kernels read them: sets inside the design packed
    (offsets, indices, output columns), sets naming a column >= K or empty left
    out (their statistics stay NaN), each set's Xc_S' Xc_S / T block per
    design; a negative index is an error, as index_select makes it in the
    reference (fastfuncstuff/glm/arma.py:3542-3561)."""
    from fastfuncstuff_gb300.glm import engine

    d = load_golden("sets")
    X = d["X"].astype(np.float64)
    sets = [[0], [0, 1], [2, 3, 4], [1, 99], [5], []]
    cs = engine.column_sets_plan(sets, d["X"])
    assert cs.n_out == 6 and cs.n_sets == 4
    np.testing.assert_array_equal(cs.set_col, [0, 1, 2, 4])
    np.testing.assert_array_equal(cs.set_ptr, [0, 1, 3, 6, 7])
    np.testing.assert_array_equal(cs.set_idx, [0, 0, 1, 2, 3, 4, 5])
    assert cs.msum == 1 + 4 + 9 + 1
    Xc = X - X.mean(0)
    mats = o.column_set_matrices(np.eye(X.shape[1]), X, [s for s in sets if s and max(s) < X.shape[1]])
    ref = np.concatenate([m[2].reshape(-1) for m in mats])
    np.testing.assert_allclose(cs.C[0], ref, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(cs.C[0][:1], [(Xc[:, 0] ** 2).mean()], rtol=1e-6)
    two = engine.column_sets_plan(sets, np.stack([d["X"], 2 * d["X"]]))
    np.testing.assert_allclose(two.C[1], 4 * two.C[0], rtol=1e-6)
    with pytest.raises(IndexError):
        engine.column_sets_plan([[0, -1]], d["X"])


def test_dsort_prepare_guard_expansion_and_errors():
    """-dsort inputs as the kernel reads them (fastfuncstuff/glm/arma.py:3207-3245,
    :3385-3397, :3931-3945): (V, T) is one dataset; a constant nonzero series is
    replaced by its dataset's mean over the other voxels (all-zero columns stay);
    dsort_run_bounds expands each set into one zero-padded column per run; a
    wrong shape is a ValueError. Checked against the oracle's restatement."""
    from fastfuncstuff_gb300.glm import engine

    rng = np.random.default_rng(8)
    V, T = 12, 30
    D = rng.standard_normal((V, 2, T)).astype(np.float32)
    D[1, 0] = 3.0          # constant: replaced
    D[2, 1] = 0.0          # all zero: kept
    with pytest.warns(UserWarning, match="constant"):
        got = engine.dsort_prepare(D, V, T, None, torch.device("cpu")).numpy()
    ref = o.dsort_constant_guard(D)
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-7)
    assert not got[2, 1].any()
    one = engine.dsort_prepare(D[:, 1], V, T, None, torch.device("cpu"))
    assert one.shape == (V, 1, T)
    rb = [0, 12, 30]
    exp = engine.dsort_prepare(D[3:5], 2, T, rb, torch.device("cpu")).numpy()
    np.testing.assert_allclose(exp, o.dsort_expand(D[3:5], rb), rtol=0, atol=0)
    assert exp.shape == (2, 4, T) and not exp[:, 0, 12:].any() and not exp[:, 1, :12].any()
    with pytest.raises(ValueError, match="dsort must be"):
        engine.dsort_prepare(D[:, :, :T - 1], V, T, None, torch.device("cpu"))


def test_parse_grid_arg_formats_and_errors(capsys):
    """The three -a_grid / -b_grid formats of fastfuncstuff/cli/reml.py:115-160."""
    from fastfuncstuff_gb300 import parse_grid_arg

    g = parse_grid_arg("-0.9:0.9:65")
    assert g.dtype == torch.float32 and torch.equal(g, torch.linspace(-0.9, 0.9, 65))
    assert torch.equal(parse_grid_arg(" 0.025:0.9:32 "), torch.linspace(0.025, 0.9, 32))
    # three comma-separated values whose last is a whole number >= 2: legacy linspace
    assert torch.equal(parse_grid_arg("-0.8,0.8,33"), torch.linspace(-0.8, 0.8, 33))
    assert torch.equal(parse_grid_arg("0,0.8,9.0"), torch.linspace(0.0, 0.8, 9))
    # anything else separated by commas is the list itself
    assert torch.equal(parse_grid_arg("0.1,0.2,0.3,0.5,0.7,0.9"),
                       torch.tensor([0.1, 0.2, 0.3, 0.5, 0.7, 0.9], dtype=torch.float32))
    assert torch.equal(parse_grid_arg("0.1,0.2,0.5"), torch.tensor([0.1, 0.2, 0.5]))  # last not whole
    assert torch.equal(parse_grid_arg("0.1,0.2,1"), torch.tensor([0.1, 0.2, 1.0]))   # whole but < 2
    assert torch.equal(parse_grid_arg("0.4"), torch.tensor([0.4]))
    for bad in ("0:1", "0:1:2:3", "a:1:5", "0:1:1", "0:1:2.5", "0.1,x", ""):
        with pytest.raises(SystemExit) as e:
            parse_grid_arg(bad)
        assert e.value.code == 1
        assert "ERROR" in capsys.readouterr().out


@pytest.mark.parametrize("corcut", [1e-4, 1e-2])
def test_afni_mode_grid_and_band_match_oracle(corcut):
    """set_afni_mode(True, corcut): the near-white pairs (0 < lambda < corcut)
    filtered out of the grid as the oracle filters them, AFNI's ltop, and each
    pair's band of R
    (the last lag with lam a^(g-1) above corcut) equal to the oracle's
    afni_bmax; the exact R's grid comes back when the mode is switched off."""
    a = b = torch.linspace(-0.8, 0.8, 17)
    exact = G.make_grid(a, b)
    G.set_afni_mode(True, corcut)
    o.set_afni_mode(True, corcut)
    try:
        g = G.make_grid(a, b)
        og = o.valid_grid(a.numpy(), b.numpy(), np.float32)
        np.testing.assert_array_equal(g.a, og.a)
        np.testing.assert_array_equal(g.b, og.b)
        assert g.ltop == o._ltop(len(og.a_axis), len(og.b_axis), True)
        want = np.array([o.afni_bmax(float(og.a[p]), float(og.lam[p]), corcut) for p in range(og.n)])
        np.testing.assert_array_equal(g.band, want)
        assert g.P <= exact.P and (g.band > 0).any()
    finally:
        G.set_afni_mode(False)
        o.set_afni_mode(False)
    again = G.make_grid(a, b)
    assert again.band is None and again.P == exact.P
