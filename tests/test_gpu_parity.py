"""CUDA path against the FP64 oracle and the reference's golden fixtures (GB300 only).

Parity bars (written where they are used):
* selected pair: identical to the FP64 oracle on >= 99.9% of voxels, and every
  disagreement within 1e-6 (relative) of the optimal criterion on the oracle's
  FP64 surface;
* betas and t: within 1e-4 relative (per voxel, max-norm) of the FP64 oracle;
* grid factors (FP64 on the GPU): logdets within 1e-9 relative of the reference.
"""

from __future__ import annotations

import os

import numpy as np
import pytest
import torch

from fastfuncstuff_gb300 import synth
from fastfuncstuff_gb300.glm import engine
from fastfuncstuff_gb300.glm import grid as G
from fastfuncstuff_gb300.glm.arma import fit_glm_arma11, fit_glm_arma11_grouped, precompute_reml_grid
from oracle import reml as o
from tests.conftest import load_golden
from tests.test_oracle_golden import case_kwargs

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")

# tolerances (see module docstring)
ARGMIN_AGREE = 0.999
CRIT_GAP_REL = 1e-6
BETA_REL = 1e-4


def rel_maxnorm(got, want):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    num = np.abs(got - want).max(axis=-1)
    den = np.maximum(np.abs(want).max(axis=-1), 1e-12)
    return num / den


def check_selection(idx_gpu, idx_ref, surf64):
    """>= 99.9% identical; the rest within CRIT_GAP_REL of the optimum on the FP64 surface."""
    idx_gpu = np.asarray(idx_gpu)
    idx_ref = np.asarray(idx_ref)
    agree = float((idx_gpu == idx_ref).mean())
    bad = np.nonzero(idx_gpu != idx_ref)[0]
    if bad.size:
        v = bad
        c_gpu = surf64[v, idx_gpu[v]]
        c_ref = surf64[v, idx_ref[v]]
        gap = np.abs(c_gpu - c_ref) / np.maximum(np.abs(c_ref), 1.0)
        assert gap.max() <= CRIT_GAP_REL, (agree, gap.max())
    assert agree >= ARGMIN_AGREE or bad.size <= 1, agree
    return agree


def _index(params, grid):
    return grid.index_of(np.asarray(params[:, 0], np.float32), np.asarray(params[:, 1], np.float32))


# ------------------------------------------------------------------ grid build


def test_grid_factors_match_reference_precompute():
    d = load_golden("grid")
    X = torch.from_numpy(d["X"])
    T = X.shape[0]
    f = precompute_reml_grid(X, T, d["a_grid"], d["b_grid"], DEV, run_starts=d["run_starts"], use_double=True)
    torch.cuda.synchronize()
    pairs = np.stack([f.grid.a, f.grid.b], 1).astype(np.float64)
    np.testing.assert_array_equal(pairs, d["pairs"])
    np.testing.assert_allclose(f.logdet_R.cpu().numpy(), d["logdet_R"], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(f.logdet_XtX.cpu().numpy(), d["logdet_XtX"], rtol=1e-9, atol=1e-9)
    assert int(f.info.cpu().abs().sum()) == 0
    # the recurrence coefficients whiten exactly like the dense L^-1
    coef = f.coef.cpu().numpy().astype(np.float64)
    Xd = d["X"].astype(np.float64)
    for p in range(f.P):
        c, m, _, rs = coef[p, :, 0], coef[p, :, 1], coef[p, :, 2], coef[p, :, 3]
        xw = np.zeros_like(Xd)
        xp = np.zeros(Xd.shape[1])
        vp = np.zeros(Xd.shape[1])
        for t in range(T):
            z = Xd[t] - c[t] * xp
            v = z - m[t] * vp
            xw[t] = v * rs[t]
            xp, vp = Xd[t], v
        np.testing.assert_allclose(xw, d["X_w"][p], rtol=2e-6, atol=2e-6)
    # U = L^-T Q and G = R^-1 X (X'R^-1 X)^-1 against the dense FP64 restatement
    og = o.valid_grid(d["a_grid"], d["b_grid"], np.float64)
    pre = o.precompute_reml_grid(Xd, og, run_starts=d["run_starts"])
    T = Xd.shape[0]
    assert f.U.shape[2] == (T + 3) // 4 * 4 and not f.U[:, :, T:].any() and not f.G[:, :, T:].any()
    U = f.U[:, :, :T].cpu().numpy()
    Gm = f.G[:, :, :T].cpu().numpy()
    for p in range(0, f.P, 5):
        Li = pre.whiteners[p].dense()
        U_ref = Li.T @ pre.Q[p]
        np.testing.assert_allclose(U[p].T, U_ref, rtol=1e-5, atol=1e-6)
        A = np.linalg.inv(pre.X_w[p].T @ pre.X_w[p])
        G_ref = Li.T @ pre.X_w[p] @ A
        np.testing.assert_allclose(Gm[p].T, G_ref, rtol=1e-4, atol=1e-5)


# --------------------------------------------------------- projection kernels


@pytest.mark.parametrize("K,T,V", [(20, 400, 1000), (8, 200, 777), (18, 855, 300), (130, 600, 260)])
def test_tensor_core_projection_matches_simt(K, T, V):
    rng = np.random.default_rng(K)
    X = rng.standard_normal((T, K)).astype(np.float32)
    Y = rng.standard_normal((V, T)).astype(np.float32)
    g = torch.linspace(-0.8, 0.8, 9)
    f = precompute_reml_grid(torch.from_numpy(X), T, g, g, DEV, run_starts=[0, T // 2])
    Yd = torch.from_numpy(Y).to(DEV)
    outs = {}
    for proj in ("tc", "simt"):
        so = engine.search(Yd, f, hierarchical=False, projector=proj, keep_surface=True)
        torch.cuda.synchronize()
        assert int(so._flag.item()) == 0
        outs[proj] = so
    s_tc = outs["tc"].surf.cpu().numpy()
    s_si = outs["simt"].surf.cpu().numpy()
    # the two projections agree to float32 level: criterion differences within
    # 2e-6 of the criterion's size (fp16 hi/lo split: ~2^-22 per product)
    c0 = np.abs(outs["simt"].crit0.cpu().numpy())[None, :]
    assert (np.abs(s_tc - s_si) / np.maximum(c0, 1.0)).max() < 2e-6, np.abs(s_tc - s_si).max()
    np.testing.assert_array_equal(outs["tc"].best.cpu().numpy(), outs["simt"].best.cpu().numpy())


# ------------------------------------------------------------- full fits


@pytest.mark.parametrize("case", ["single", "multirun", "censored", "baseline"])
@pytest.mark.parametrize("exhaustive", [True, False])
def test_fit_matches_fp64_oracle(case, exhaustive):
    d = load_golden(case)
    kw = case_kwargs(d)
    ref = o.fit_glm_arma11(d["Y"], d["X"], use_double=True, fp64_scaled=True,
                           force_exhaustive_search=exhaustive, save_profile_likelihoods=True, **kw)
    gkw = dict(kw)
    if "glt_matrices" in gkw:
        gkw["glt_labels"] = ["c0"]
    got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, force_exhaustive_search=exhaustive, want_r2_partial=True, **gkw)
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    idx = _index(got.arma_params.numpy(), grid)
    check_selection(idx, ref.arma_index, ref.reml_lklhd_surface)
    same = idx == ref.arma_index
    assert rel_maxnorm(got.betas.numpy()[same], ref.betas[same]).max() <= BETA_REL
    assert rel_maxnorm(got.tstats.numpy()[same], ref.tstats[same]).max() <= BETA_REL
    np.testing.assert_allclose(got.sigma2.numpy()[same], ref.sigma2[same], rtol=1e-4)
    np.testing.assert_allclose(got.fstats.numpy()[same], ref.fstats[same], rtol=2e-4, atol=1e-4)
    np.testing.assert_allclose(got.r2.numpy()[same], ref.r2[same], atol=2e-5)
    np.testing.assert_allclose(got.reml_likelihood.numpy()[same], ref.reml_likelihood[same], rtol=1e-5,
                               atol=2e-3)
    lam = o.arma_lambda_output_f32(got.arma_params[:, 0].numpy(), got.arma_params[:, 1].numpy())
    np.testing.assert_array_equal(got.arma_lambda.numpy(), lam)
    if kw.get("want_ljung_box"):
        np.testing.assert_allclose(got.ljung_box.numpy()[same], ref.ljung_box[same], rtol=2e-3, atol=1e-3)
        assert got.ljung_box_dof == ref.ljung_box_dof
    if "glt_matrices" in kw:
        assert rel_maxnorm(got.contrast_betas.numpy()[same], ref.contrast_betas[same]).max() <= BETA_REL
        assert rel_maxnorm(got.contrast_tstats.numpy()[same], ref.contrast_tstats[same]).max() <= BETA_REL
    if kw.get("want_residuals"):
        np.testing.assert_allclose(got.residuals.numpy()[same], ref.residuals[same], rtol=1e-4, atol=2e-4)
        np.testing.assert_allclose(got.residuals_whitened.numpy()[same], ref.residuals_whitened[same],
                                   rtol=1e-4, atol=2e-4)
    np.testing.assert_allclose(got.r2_partial.numpy()[same], ref.r2_partial[same], atol=1e-4)


@pytest.mark.parametrize("T", [96, 94, 93])
def test_fit_any_series_length_matches_fp64_oracle(T):
    """The 32-voxel tile kernels of prep and GLS read 16-byte words of Y when
    T % 4 == 0 and single samples otherwise (the K x T matrices are padded to
    a multiple of 4 either way). Both against the FP64 oracle, with the
    residual, whitened-residual, fitted-value and Ljung-Box outputs."""
    d = load_golden("single")
    Y = np.ascontiguousarray(d["Y"][:, :T])
    X = np.ascontiguousarray(d["X"][:T])
    kw = dict(a_grid=d["a_grid"], b_grid=d["b_grid"], want_residuals=True, want_ljung_box=True)
    ref = o.fit_glm_arma11(Y, X, use_double=True, fp64_scaled=True, force_exhaustive_search=True,
                           save_profile_likelihoods=True, **kw)
    got = fit_glm_arma11(Y, X, tr=2.0, device=DEV, verbose=False, force_exhaustive_search=True,
                         want_predicted=True, **kw)
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    idx = _index(got.arma_params.numpy(), grid)
    check_selection(idx, ref.arma_index, ref.reml_lklhd_surface)
    same = idx == ref.arma_index
    assert rel_maxnorm(got.betas.numpy()[same], ref.betas[same]).max() <= BETA_REL
    assert rel_maxnorm(got.tstats.numpy()[same], ref.tstats[same]).max() <= BETA_REL
    np.testing.assert_allclose(got.sigma2.numpy()[same], ref.sigma2[same], rtol=1e-4)
    np.testing.assert_allclose(got.r2.numpy()[same], ref.r2[same], atol=2e-5)
    np.testing.assert_allclose(got.residuals.numpy()[same], ref.residuals[same], rtol=1e-4, atol=2e-4)
    np.testing.assert_allclose(got.residuals_whitened.numpy()[same], ref.residuals_whitened[same],
                               rtol=1e-4, atol=2e-4)
    np.testing.assert_allclose(got.ljung_box.numpy()[same], ref.ljung_box[same], rtol=2e-3, atol=1e-3)
    # fitted values + residuals give back the data
    scale = np.abs(Y).max(axis=1, keepdims=True)
    np.testing.assert_allclose((got.predicted + got.residuals).numpy() / scale, Y / scale, atol=1e-5)


def test_reference_float32_selection_agrees():
    """The reference's own float32 run (golden) selects what the GPU selects."""
    for case in ("single", "multirun", "censored", "baseline"):
        d = load_golden(case)
        kw = case_kwargs(d)
        if "glt_matrices" in kw:
            kw["glt_labels"] = ["c0"]
        got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, force_exhaustive_search=True, **kw)
        agree = (got.arma_params.numpy() == d["f32_exh__arma_params"]).all(1).mean()
        assert agree >= 0.98, (case, agree)


def test_use_double_semantics_match_fp64_reference():
    d = load_golden("single")
    got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, a_grid=d["a_grid"], b_grid=d["b_grid"], device=DEV, verbose=False, use_double=True, force_exhaustive_search=True)
    assert got.betas.dtype == torch.float64
    np.testing.assert_array_equal(got.arma_params.numpy(), d["f64_exh__arma_params"])
    np.testing.assert_allclose(got.reml_likelihood.numpy(), d["f64_exh__reml_likelihood"], rtol=1e-5, atol=2e-3)
    assert rel_maxnorm(got.betas.numpy(), d["f64_exh__betas"]).max() <= BETA_REL


def test_grouped_matches_reference():
    d = load_golden("grouped")
    designs = {h: d[f"X{h}"] for h in range(3)}
    got = fit_glm_arma11_grouped(d["Y"], designs, d["gid"], tr=2.0, a_grid=d["a_grid"], b_grid=d["b_grid"],
                                 device=DEV, force_exhaustive_search=True)
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    ref_idx = _index(d["f64_exh__arma_params"], grid)
    idx = _index(got.arma_params.numpy(), grid)
    # the FP64 surface of the same fits decides the voxels that differ
    surf = o.fit_glm_arma11_grouped(d["Y"], designs, d["gid"], a_grid=d["a_grid"], b_grid=d["b_grid"],
                                    use_double=True, force_exhaustive_search=True,
                                    save_profile_likelihoods=True).reml_lklhd_surface
    check_selection(idx, ref_idx, surf)
    same = idx == ref_idx
    assert rel_maxnorm(got.betas.numpy()[same], d["f64_exh__betas"][same]).max() <= BETA_REL


def test_design_basis_centring_test_matches_normal_equations():
    """The design-basis kernel's centring test (FP64 Cholesky of X'X, c with
    X c = 1) agrees with the torch FP64 normal equations: constant in the span
    (intercept; per-run drift), not in the span, and a rank-deficient X'X."""
    rng = np.random.default_rng(7)
    T = 200
    t = np.linspace(-1, 1, T)
    cases = {
        "intercept": np.column_stack([rng.standard_normal((T, 3)), np.ones(T)]),
        "runs": np.column_stack([rng.standard_normal(T), (np.arange(T) < 90), (np.arange(T) >= 90), t]),
        "no_constant": np.column_stack([rng.standard_normal((T, 3)), t]),
        "rank_deficient": np.column_stack([t, 2 * t, t**2]),  # no constant, X'X singular
    }
    for name, X in cases.items():
        Xd = torch.from_numpy(X.astype(np.float32)).to(DEV)
        q0, flag, coef = engine.design_basis(Xd, with_constant=True)
        ref_flag, ref_coef = engine.constant_flag(Xd)
        torch.cuda.synchronize()
        assert int(flag[0]) == int(ref_flag[0]), name
        np.testing.assert_allclose(coef.cpu().numpy(), ref_coef.cpu().numpy(), rtol=1e-5, atol=1e-6, err_msg=name)
        if int(flag[0]):
            np.testing.assert_allclose(X @ coef.cpu().numpy().astype(np.float64), np.ones(T), atol=1e-5)
        # Q0 spans the design's columns, orthonormal (full-rank cases)
        if name != "rank_deficient":
            Q = q0[:, :T].cpu().numpy().astype(np.float64).T
            np.testing.assert_allclose(Q.T @ Q, np.eye(Q.shape[1]), atol=1e-5)


@pytest.mark.parametrize("exhaustive", [True, False])
def test_column_sets_match_oracle_and_reference(exhaustive):
    """column_sets on the device (per-pair inv(A_SS + 1e-8 I) from the grid
    build, per-voxel F / SD / coefficient after the GLS) against the FP64
    oracle on the float32 mode's semantics, and against the reference's own
    float32 outputs on the voxels whose pair agrees; the set naming a column
    outside the design stays NaN."""
    d = load_golden("sets")
    kw = case_kwargs(d)
    ref = o.fit_glm_arma11(d["Y"], d["X"], use_double=True, fp64_scaled=True, force_exhaustive_search=exhaustive,
                           save_profile_likelihoods=True, **kw)
    got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, force_exhaustive_search=exhaustive, **kw)
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    idx = _index(got.arma_params.numpy(), grid)
    check_selection(idx, ref.arma_index, ref.reml_lklhd_surface)
    same = idx == ref.arma_index

    def check_sets(g, r, betas_ref, bound):
        # the set statistics inherit the betas' error, which is bounded
        # relative to each voxel's largest beta (t's to its largest t): F
        # through sqrt(F) (a t-like scale), per voxel over the sets; SD and
        # coefficient against the voxel's largest |beta|
        for name in ("set_fstats", "set_sd", "set_coef"):
            np.testing.assert_array_equal(np.isnan(g[name]), np.isnan(r[name]), err_msg=name)
        ok = ~np.isnan(r["set_fstats"][0])
        assert rel_maxnorm(np.sqrt(g["set_fstats"][:, ok]), np.sqrt(r["set_fstats"][:, ok])).max() <= bound
        scale = np.abs(betas_ref).max(1)
        for name in ("set_sd", "set_coef"):
            col = ~np.isnan(r[name][0])
            err = np.abs(g[name][:, col] - r[name][:, col]).max(1) / scale
            assert err.max() <= bound, (name, err.max())

    fields = ("set_fstats", "set_sd", "set_coef")
    check_sets({k: getattr(got, k).numpy()[same] for k in fields}, {k: getattr(ref, k)[same] for k in fields},
               ref.betas[same], 2 * BETA_REL)
    # the reference's own float32 run, on the voxels whose pair agrees
    mode = "f32_exh" if exhaustive else "f32_def"
    agree = (got.arma_params.numpy() == d[mode + "__arma_params"]).all(1)
    assert agree.mean() >= 0.97
    check_sets({k: getattr(got, k).numpy()[agree] for k in fields}, {k: d[f"{mode}__{k}"][agree] for k in fields},
               d[mode + "__betas"][agree], 2e-3)


@pytest.mark.parametrize("T,K", [(400, 20), (201, 7), (300, 70), (300, 200)])
def test_design_basis_equals_grid_build_identity_pair(T, K):
    """Q0 of the design-basis kernels is U of the pair (0, 0) bit for bit (the
    grouped fit takes its basis from the grid build, the per-group fit from
    the design basis): the factor in shared memory (K <= 64), in global
    memory (K = 70), and a Gram formed over several staged passes of the
    samples (K = 200). It also spans X (orthonormal, X = Q0' R)."""
    rng = np.random.default_rng(K)
    t = np.linspace(-1, 1, T)
    X = np.column_stack([np.ones(T), t, rng.standard_normal((T, K - 2))]).astype(np.float32)
    Xd = torch.from_numpy(X).to(DEV)
    g = G.make_grid(torch.linspace(-0.6, 0.6, 3), torch.linspace(-0.6, 0.6, 3))
    lay = G.run_layout(T, [0])
    f = engine.build_factors(Xd, g, lay, with_tc=False)
    q0 = engine.design_basis(Xd)
    torch.cuda.synchronize()
    u00 = f.U[g.p0]
    assert torch.equal(q0, u00)
    Q = q0[:, :T].cpu().numpy().astype(np.float64).T
    np.testing.assert_allclose(Q.T @ Q, np.eye(K), atol=2e-5)
    R = Q.T @ X.astype(np.float64)
    np.testing.assert_allclose(Q @ R, X, atol=2e-4 * np.abs(X).max())


@pytest.mark.parametrize("selector", ["hierarchical", "exhaustive"])
def test_grouped_batched_fit_equals_per_group_fits(selector):
    """The grouped fit runs every design in one pass per stage (one grid build
    over designs x pairs, a (design, voxel tile, pair block) projection work
    list, per-tile designs in prep and the criterion, design x pair keys in
    the GLS). Each voxel's arithmetic is the per-group fit's, so the results
    are those of fitting every group on its own: workload-2 shapes (4 censored
    runs, N=855, Zipf group sizes), fewer voxels and 6 of the 20 designs."""
    w = synth.workload(2, V=6000)
    keep = np.isin(w.groups, np.arange(6))
    Y, gid = w.Y[keep], w.groups[keep]
    designs = {h: w.designs[h] for h in range(6)}
    kw = dict(a_grid=np.linspace(-0.8, 0.8, 17), b_grid=np.linspace(-0.8, 0.8, 17), run_starts=w.run_starts,
              tau=w.tau, device=DEV, verbose=False, force_exhaustive_search=selector == "exhaustive",
              want_residuals=True, glt_labels=["t0-t1"], glt_matrices=[np.eye(18)[0] - np.eye(18)[1]],
              column_sets=[[0], [0, 1], [2, 3, 4, 5], [17, 18]])
    got = fit_glm_arma11_grouped(Y, designs, gid, tr=2.0, **kw)
    for h in range(6):
        m = gid == h
        ref = fit_glm_arma11(Y[m], designs[h], tr=2.0, **kw)
        np.testing.assert_array_equal(got.arma_params.numpy()[m], ref.arma_params.numpy())
        np.testing.assert_array_equal(got.reml_likelihood.numpy()[m], ref.reml_likelihood.numpy())
        for name in ("betas", "tstats", "sigma2", "fstats", "r2", "arma_lambda", "contrast_betas",
                     "contrast_tstats", "residuals", "residuals_whitened", "set_fstats", "set_sd", "set_coef"):
            np.testing.assert_array_equal(getattr(got, name).numpy()[m], getattr(ref, name).numpy(), err_msg=name)


def test_grouped_fit_graph_equals_eager_fit():
    """fit_glm_arma11_grouped replays the whole grouped fit (grid build over
    designs x pairs, residualisation, projection work list, criterion,
    selection, GLS) from one CUDA graph: bit-identical to the eager fit, and a
    second replay with new data gives that data's eager results."""
    w = synth.workload(2, V=5000)
    keep = np.isin(w.groups, np.arange(5))
    Y, gid = w.Y[keep], w.groups[keep]
    designs = {h: w.designs[h] for h in range(5)}
    kw = dict(a_grid=np.linspace(-0.8, 0.8, 17), b_grid=np.linspace(-0.8, 0.8, 17), run_starts=w.run_starts,
              tau=w.tau, device=DEV, verbose=False, want_residuals=True, glt_labels=["t0-t1"],
              glt_matrices=[np.eye(18)[0] - np.eye(18)[1]])
    for data in (Y, Y[:, ::-1].copy()):  # the second call replays the graph on other data
        eager = fit_glm_arma11_grouped(data, designs, gid, tr=2.0, cuda_graphs=False, **kw)
        graph = fit_glm_arma11_grouped(data, designs, gid, tr=2.0, cuda_graphs=True, **kw)
        for name in ("arma_params", "reml_likelihood", "betas", "tstats", "sigma2", "fstats", "r2", "arma_lambda",
                     "contrast_betas", "contrast_tstats", "residuals", "residuals_whitened"):
            np.testing.assert_array_equal(getattr(graph, name).numpy(), getattr(eager, name).numpy(), err_msg=name)


def test_precomputed_params_path():
    d = load_golden("multirun")
    kw = case_kwargs(d)
    kw["glt_labels"] = ["c0"]
    first = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, **kw)
    again = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False,
                           precomputed_arma_params=first.arma_params, **kw)
    np.testing.assert_array_equal(again.arma_params.numpy(), first.arma_params.numpy())
    assert rel_maxnorm(again.betas.numpy(), first.betas.numpy()).max() <= 1e-5
    np.testing.assert_allclose(again.sigma2.numpy(), first.sigma2.numpy(), rtol=1e-5)


def test_edge_cases_constant_and_pure_signal_voxels():
    d = load_golden("single")
    Y = d["Y"][:40].copy()
    Y[0] = 0.0                                 # all-zero voxel
    Y[1] = 7.5                                 # constant voxel
    Y[2] = d["X"] @ np.arange(d["X"].shape[1], dtype=np.float32)  # exactly in the design span
    got = fit_glm_arma11(Y, d["X"], tr=2.0, a_grid=d["a_grid"], b_grid=d["b_grid"], device=DEV, verbose=False)
    for name in ("betas", "tstats", "sigma2", "fstats", "r2", "reml_likelihood"):
        assert torch.isfinite(getattr(got, name)).all(), name
    assert float(got.r2[0]) == 0.0


# ----------------------------------------------------- workload-size parity


def test_workload0_subset_parity_exhaustive_and_hierarchical():
    w = synth.workload(0, V=1500)
    g = torch.linspace(-0.8, 0.8, 33)
    og = o.valid_grid(g.numpy(), g.numpy(), np.float64)
    surf = o.criterion_surface(w.X, w.Y, og, scaled=True)
    for exhaustive in (True, False):
        got = fit_glm_arma11(w.Y, w.X, tr=2.0, a_grid=g, b_grid=g, device=DEV, verbose=False,
                             force_exhaustive_search=exhaustive)
        if exhaustive:
            ref_idx = np.argmin(surf, axis=1)
        else:
            ref_idx, _ = o.select_hierarchical_from_surface(surf, og)
        idx = _index(got.arma_params.numpy(), G.make_grid(g, g))
        agree = check_selection(idx, ref_idx, surf)
        print(f"workload0 exhaustive={exhaustive}: agreement {agree:.5f}")


def test_rvar_round_trip_reuses_the_fitted_pairs(tmp_path):
    """fit -> -Rvar file -> load_arma_params -> fit with precomputed_arma_params:
    the second fit reuses the first's (a, b) and reproduces its GLS; the file's
    StDev, -LogLik and LjungBox volumes are the first fit's."""
    from fastfuncstuff_gb300 import load_arma_params, save_arma_rvar

    d = load_golden("multirun")
    kw = case_kwargs(d)
    kw["glt_labels"] = ["c0"]
    first = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, **kw)
    V = d["Y"].shape[0]
    mask = np.zeros(V + 7, bool)
    mask[3:3 + V] = True
    path = save_arma_rvar(first, tmp_path / "rvar.nii.gz", volume_shape=(V + 7, 1, 1), voxel_mask=mask)
    ab = load_arma_params(path, mask)
    np.testing.assert_array_equal(ab, first.arma_params.numpy())
    again = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, precomputed_arma_params=ab, **kw)
    np.testing.assert_array_equal(again.arma_params.numpy(), first.arma_params.numpy())
    assert rel_maxnorm(again.betas.numpy(), first.betas.numpy()).max() <= 1e-5
    import gzip
    import struct
    raw = gzip.decompress(path.read_bytes())
    off = int(struct.unpack_from("<f", raw, 108)[0])
    vol = np.frombuffer(raw, np.float32, offset=off).reshape((V + 7, 1, 1, 6), order="F")[mask, 0, 0]
    np.testing.assert_allclose(vol[:, 3], np.sqrt(first.sigma2.numpy()), rtol=1e-6)
    np.testing.assert_array_equal(vol[:, 4], first.reml_likelihood.numpy())
    np.testing.assert_array_equal(vol[:, 5], first.ljung_box.numpy())


@pytest.mark.parametrize("tag", ["two", "runs"])
@pytest.mark.parametrize("exhaustive", [True, False])
def test_dsort_matches_oracle_and_reference(tag, exhaustive):
    """-dsort on the device (ffs_reml_gls_dsort: block elimination against the
    pair's G and U, a q x q solve per voxel) against the FP64 oracle on the
    float32 mode's semantics, and against the reference's own float32 run:
    base and voxelwise betas and t, sigma2, F, R^2, GLT, Ljung-Box, residuals
    and column sets over [X | D]; two datasets per voxel (one with constant
    series the guard replaces), and one dataset expanded per run."""
    d = load_golden("dsort")
    K = d["X"].shape[1]
    ptr, idx = d[f"{tag}__sets_ptr"], d[f"{tag}__sets_idx"]
    sets = [[int(c) for c in idx[ptr[g]:ptr[g + 1]]] for g in range(len(ptr) - 1)]
    kw = dict(a_grid=d["a_grid"], b_grid=d["b_grid"], run_starts=d["run_starts"], task_indices=[0, 1],
              glt_matrices=[d["glt"][0]], want_ljung_box=True, want_residuals=True, column_sets=sets)
    if tag == "two":
        kw["dsort"] = d["D"]
    else:
        kw.update(dsort=d["D"][:, :1], dsort_run_bounds=[0, 64, 128])
    with pytest.warns(UserWarning, match="constant") if tag == "two" else _no_warning():
        got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, force_exhaustive_search=exhaustive, glt_labels=["t0-t1"], **kw)
    ref = o.fit_glm_arma11(d["Y"], d["X"], use_double=True, fp64_scaled=True, force_exhaustive_search=exhaustive,
                           save_profile_likelihoods=True, **kw)
    assert got.dof == ref.dof == int(d[f"{tag}_f64_def__dof"])
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    idx_g = _index(got.arma_params.numpy(), grid)
    check_selection(idx_g, ref.arma_index, ref.reml_lklhd_surface)
    same = idx_g == ref.arma_index
    q = ref.dsort_betas.shape[1]
    assert got.dsort_betas.shape == (d["Y"].shape[0], q)
    full_got = np.concatenate([got.betas.numpy(), got.dsort_betas.numpy()], 1)[same]
    full_ref = np.concatenate([ref.betas, ref.dsort_betas], 1)[same]
    assert rel_maxnorm(full_got, full_ref).max() <= BETA_REL
    t_got = np.concatenate([got.tstats.numpy(), got.dsort_tstats.numpy()], 1)[same]
    t_ref = np.concatenate([ref.tstats, ref.dsort_tstats], 1)[same]
    assert rel_maxnorm(t_got, t_ref).max() <= BETA_REL
    np.testing.assert_allclose(got.sigma2.numpy()[same], ref.sigma2[same], rtol=1e-4)
    assert rel_maxnorm(np.sqrt(got.fstats.numpy()[same])[:, None], np.sqrt(ref.fstats[same])[:, None]).max() <= 2e-4
    np.testing.assert_allclose(got.r2.numpy()[same], ref.r2[same], atol=2e-5)
    assert rel_maxnorm(got.contrast_tstats.numpy()[same], ref.contrast_tstats[same]).max() <= 2e-4
    np.testing.assert_allclose(got.ljung_box.numpy()[same], ref.ljung_box[same], rtol=2e-3, atol=1e-3)
    scale = np.abs(ref.residuals[same]).max(1, keepdims=True)
    assert (np.abs(got.residuals.numpy()[same] - ref.residuals[same]) / scale).max() <= 2e-4
    for name in ("set_fstats", "set_sd", "set_coef"):
        np.testing.assert_array_equal(np.isnan(getattr(got, name).numpy()), np.isnan(getattr(ref, name)))
    ok = ~np.isnan(ref.set_fstats[0])
    assert rel_maxnorm(np.sqrt(got.set_fstats.numpy()[same][:, ok]), np.sqrt(ref.set_fstats[same][:, ok])).max() <= 2e-4
    col = ~np.isnan(ref.set_sd[0])
    err = np.abs(got.set_sd.numpy()[same][:, col] - ref.set_sd[same][:, col]).max(1) / np.abs(full_ref).max(1)
    assert err.max() <= 2e-4
    # the reference's own float32 run, on the voxels whose pair agrees
    mode = f"{tag}_{'f32_exh' if exhaustive else 'f32_def'}"
    agree = (got.arma_params.numpy() == d[mode + "__arma_params"]).all(1)
    assert agree.mean() >= 0.97
    for name in ("betas", "dsort_betas"):
        g, r = getattr(got, name).numpy()[agree], d[f"{mode}__{name}"][agree]
        assert rel_maxnorm(g, r).max() <= 5e-3, name


class _no_warning:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def test_autotuner_picks_a_tile_and_results_do_not_depend_on_it():
    """The projection's tile shape (pairs per B tile) is chosen by timing; every
    candidate gives the same surface bit for bit (each pair's sums are formed
    in the same order), so the choice only changes the speed."""
    from fastfuncstuff_gb300 import autotune_projection
    from fastfuncstuff_gb300 import _lib

    rng = np.random.default_rng(9)
    T, K, V = 300, 20, 3000
    X = rng.standard_normal((T, K)).astype(np.float32)
    Y = torch.from_numpy(rng.standard_normal((V, T)).astype(np.float32)).to(DEV)
    g = torch.linspace(-0.8, 0.8, 17)
    f = precompute_reml_grid(torch.from_numpy(X), T, g, g, DEV, run_starts=[0, 150])
    tuned = autotune_projection(T, K, f.P, DEV, V=8192, reps=2)
    assert tuned["pairs"] in (12, 6, 3) and set(tuned["ms"]) == {12, 6, 3}
    lib = _lib.load()
    surfs = []
    orig = engine.autotune_projection
    engine.autotune_projection = lambda *a, **k: None  # keep each forced tile shape
    try:
        for pairs in (12, 6, 3):
            _lib.check(lib.ffs_reml_tune_tc_pairs(K, pairs), "tune")
            so = engine.search(Y, f, hierarchical=False, projector="tc", keep_surface=True)
            torch.cuda.synchronize()
            surfs.append(so.surf.cpu())
    finally:
        engine.autotune_projection = orig
        _lib.check(lib.ffs_reml_tune_tc_pairs(K, tuned["pairs"]), "tune")
    assert torch.equal(surfs[0], surfs[1]) and torch.equal(surfs[0], surfs[2])


def test_global_arma_matches_oracle_and_reference():
    """estimate_per_voxel=False: one (a, b) from the unscaled mean series (the
    full grid's exhaustive argmin on the device), its criterion for every
    voxel, then the GLS of every voxel at that pair; against the reference's
    own outputs and the FP64 oracle."""
    d = load_golden("global")
    kw = dict(a_grid=d["a_grid"], b_grid=d["b_grid"], run_starts=d["run_starts"], estimate_per_voxel=False)
    got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, **kw)
    np.testing.assert_array_equal(got.arma_params.numpy(), d["f32__arma_params"])
    np.testing.assert_allclose(got.reml_likelihood.numpy(), d["f32__reml_likelihood"], rtol=1e-5)
    ref = o.fit_glm_arma11(d["Y"], d["X"], use_double=True, fp64_scaled=True, **kw)
    np.testing.assert_array_equal(got.arma_params.numpy(), ref.arma_params.astype(np.float32))
    assert rel_maxnorm(got.betas.numpy(), ref.betas).max() <= BETA_REL
    assert rel_maxnorm(got.tstats.numpy(), ref.tstats).max() <= BETA_REL
    np.testing.assert_allclose(got.sigma2.numpy(), ref.sigma2, rtol=1e-4)
    np.testing.assert_allclose(got.r2.numpy(), ref.r2, atol=2e-5)
    assert rel_maxnorm(got.betas.numpy(), d["f32__betas"]).max() <= 2e-3


def test_global_arma_use_double_matches_fp64_reference():
    """estimate_per_voxel=False under use_double: the mean series formed in
    float64 as the reference's data.mean(0) is, the pair and likelihood of the
    reference's own float64 run."""
    d = load_golden("global")
    kw = dict(a_grid=d["a_grid"], b_grid=d["b_grid"], run_starts=d["run_starts"], estimate_per_voxel=False)
    got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, use_double=True, **kw)
    assert got.betas.dtype == torch.float64
    np.testing.assert_array_equal(got.arma_params.numpy(), d["f64__arma_params"])
    np.testing.assert_allclose(got.reml_likelihood.numpy(), d["f64__reml_likelihood"], rtol=1e-5)
    assert rel_maxnorm(got.betas.numpy(), d["f64__betas"]).max() <= BETA_REL
    np.testing.assert_allclose(got.sigma2.numpy(), d["f64__sigma2"], rtol=1e-4)


# ------------------------------------------- the benchmark workloads' shapes


def _oracle_parity(got, ref, grid, label):
    """check_selection on the FP64 surface, then betas and t within BETA_REL of
    the FP64 oracle wherever the pair agrees; returns the agreement."""
    idx = _index(got.arma_params.numpy(), grid)
    agree = check_selection(idx, ref.arma_index, ref.reml_lklhd_surface)
    same = idx == ref.arma_index
    eb = rel_maxnorm(got.betas.numpy()[same], ref.betas[same]).max()
    et = rel_maxnorm(got.tstats.numpy()[same], ref.tstats[same]).max()
    print(f"{label}: agreement {agree:.5f}, beta rel err {eb:.2e}, t rel err {et:.2e}")
    assert eb <= BETA_REL and et <= BETA_REL
    return agree


@pytest.mark.parametrize("exhaustive", [True, False])
def test_workload1_shape_parity(exhaustive):
    """The headline shape: N=400 as 2 runs x 200, p=20 (4 task, 2 x Legendre
    0-4, 6 motion random walks), the 33 x 33 grid (561 valid pairs), 1,200
    voxels, against the FP64 oracle in both selector modes."""
    w = synth.workload(1, V=1200)
    g = torch.linspace(-0.8, 0.8, 33)
    ref = o.fit_glm_arma11(w.Y, w.X, a_grid=g.numpy(), b_grid=g.numpy(), run_starts=w.run_starts,
                           use_double=True, fp64_scaled=True, force_exhaustive_search=exhaustive,
                           save_profile_likelihoods=True)
    got = fit_glm_arma11(w.Y, w.X, tr=2.0, a_grid=g, b_grid=g, run_starts=w.run_starts, device=DEV,
                         verbose=False, force_exhaustive_search=exhaustive)
    _oracle_parity(got, ref, G.make_grid(g, g), f"workload1 exhaustive={exhaustive}")


def test_workload2_shape_grouped_parity():
    """Grouped designs at the workload-2 shape: 4 runs of 180/220/240/260 TRs
    with 5% of frames censored (N=855 kept, per-run tau), p=18, three of the
    HRF-group designs, against the FP64 oracle's per-group fits."""
    w = synth.workload(2, V=1500)
    keep = w.groups < 3
    Y, gid = w.Y[keep], w.groups[keep]
    designs = {h: w.designs[h] for h in range(3)}
    g = torch.linspace(-0.8, 0.8, 33)
    ref = o.fit_glm_arma11_grouped(Y, designs, gid, a_grid=g.numpy(), b_grid=g.numpy(), run_starts=w.run_starts,
                                   tau=w.tau, use_double=True, fp64_scaled=True, force_exhaustive_search=True,
                                   save_profile_likelihoods=True)
    got = fit_glm_arma11_grouped(Y, designs, gid, tr=2.0, a_grid=g, b_grid=g, run_starts=w.run_starts,
                                 tau=w.tau, device=DEV, force_exhaustive_search=True)
    _oracle_parity(got, ref, G.make_grid(g, g), "workload2 grouped")


def test_workload3_shape_parity():
    """The single-trial shape: N=600 as 3 runs x 200, p=130 (120 one-event
    columns + drift and a nuisance column), 33 x 33 grid, 300 voxels."""
    w = synth.workload(3, V=300)
    g = torch.linspace(-0.8, 0.8, 33)
    ref = o.fit_glm_arma11(w.Y, w.X, a_grid=g.numpy(), b_grid=g.numpy(), run_starts=w.run_starts,
                           use_double=True, fp64_scaled=True, force_exhaustive_search=True,
                           save_profile_likelihoods=True)
    got = fit_glm_arma11(w.Y, w.X, tr=2.0, a_grid=g, b_grid=g, run_starts=w.run_starts, device=DEV,
                         verbose=False, force_exhaustive_search=True)
    _oracle_parity(got, ref, G.make_grid(g, g), "workload3")
