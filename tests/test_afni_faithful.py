"""AFNI-faithful mode (``set_afni_mode(True)``) on the GPU: the banded R.

The reference truncates each pair's correlation to AFNI's band
(fastfuncstuff/glm/arma.py:95-109, :918-926, :1075-1089), drops the near-white
pairs from the grid (:1031-1036) and uses AFNI's hierarchical ltop. The grid
build factors the banded R as a band (``band_L``), and the surface and GLS
kernels whiten against it. Checked against the FP64 oracle (pinned to the
reference's own outputs in ``tests/golden/afni_faithful.npz``) and against the
reference's float32 outputs in that fixture.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from fastfuncstuff_gb300.glm import grid as G
from fastfuncstuff_gb300.glm.arma import fit_glm_arma11, precompute_reml_grid, set_afni_mode
from oracle import reml as o
from tests.conftest import load_golden
from tests.test_gpu_parity import BETA_REL, _index, check_selection, rel_maxnorm
from tests.test_oracle_golden import afni_faithful_case

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


@pytest.fixture
def afni_mode():
    set_afni_mode(True)
    o.set_afni_mode(True)
    yield
    set_afni_mode(False)
    o.set_afni_mode(False)


@pytest.mark.parametrize("tag", ["runs", "cens"])
def test_banded_factors_match_the_dense_oracle(tag, afni_mode):
    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, tag)
    T = X.shape[0]
    f = precompute_reml_grid(torch.from_numpy(X), T, d["a_grid"], d["b_grid"], DEV, run_starts=kw["run_starts"],
                             tau=kw.get("tau"), use_double=True)
    torch.cuda.synchronize()
    og = o.valid_grid(d["a_grid"], d["b_grid"], np.float64)
    np.testing.assert_array_equal(np.stack([f.grid.a, f.grid.b], 1), np.stack([og.a, og.b], 1))
    band = np.array([o.afni_bmax(float(og.a[p]), float(og.lam[p]), 1e-4) for p in range(og.n)])
    np.testing.assert_array_equal(f.grid.band, band)
    assert int(f.info.cpu().abs().sum()) == 0
    pre = o.precompute_reml_grid(X.astype(np.float64), og, run_starts=kw["run_starts"], tau=kw.get("tau"))
    np.testing.assert_allclose(f.logdet_R.cpu().numpy(), pre.logdet_R, rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(f.logdet_XtX.cpu().numpy(), pre.logdet_XtX, rtol=1e-9, atol=1e-9)
    L = f.band_L.cpu().numpy()
    coef = f.band_coef.cpu().numpy().astype(np.float64)
    U = f.U[:, :, :T].cpu().numpy()
    for p in range(0, f.P, 7):
        # the band rows are the dense Cholesky factor's, zero outside the band
        Li = pre.whiteners[p].dense()
        Ld = np.linalg.inv(Li)
        for t in range(T):
            for j in range(L.shape[2]):
                want = Ld[t, t - j] if j <= t else 0.0
                assert abs(L[p, t, j] - want) <= 1e-9 * max(1.0, abs(want)), (p, t, j)
        # the fp32 coefficients whiten like L^-1
        xw = np.zeros_like(X, dtype=np.float64)
        for t in range(T):
            acc = X[t].astype(np.float64) * coef[p, t, 0]
            for j in range(1, min(t, L.shape[2] - 1) + 1):
                acc -= coef[p, t, j] * xw[t - j]
            xw[t] = acc
        np.testing.assert_allclose(xw, pre.X_w[p], rtol=2e-5, atol=2e-5)
        np.testing.assert_allclose(U[p].T, Li.T @ pre.Q[p], rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("tag", ["runs", "cens"])
@pytest.mark.parametrize("exhaustive", [True, False])
def test_afni_faithful_fit_matches_fp64_oracle_and_reference(tag, exhaustive, afni_mode):
    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, tag)
    ref = o.fit_glm_arma11(Y, X, use_double=True, fp64_scaled=True, force_exhaustive_search=exhaustive,
                           save_profile_likelihoods=True, want_ljung_box=True, want_residuals=True, **kw)
    got = fit_glm_arma11(Y, X, tr=2.0, device=DEV, verbose=False, force_exhaustive_search=exhaustive,
                         want_ljung_box=True, want_residuals=True, **kw)
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    idx = _index(got.arma_params.numpy(), grid)
    check_selection(idx, ref.arma_index, ref.reml_lklhd_surface)
    same = idx == ref.arma_index
    assert rel_maxnorm(got.betas.numpy()[same], ref.betas[same]).max() <= BETA_REL
    assert rel_maxnorm(got.tstats.numpy()[same], ref.tstats[same]).max() <= BETA_REL
    np.testing.assert_allclose(got.sigma2.numpy()[same], ref.sigma2[same], rtol=1e-4)
    np.testing.assert_allclose(got.reml_likelihood.numpy()[same], ref.reml_likelihood[same], rtol=1e-5,
                               atol=2e-3)
    np.testing.assert_allclose(got.residuals_whitened.numpy()[same], ref.residuals_whitened[same],
                               rtol=1e-4, atol=2e-4)
    np.testing.assert_allclose(got.ljung_box.numpy()[same], ref.ljung_box[same], rtol=2e-3, atol=1e-3)
    # the reference's own float32 run of the same mode
    mode = f"{tag}_f32_{'exh' if exhaustive else 'def'}__"
    agree = (got.arma_params.numpy() == d[mode + "arma_params"]).all(1)
    assert agree.mean() >= 0.97, agree.mean()
    assert rel_maxnorm(got.betas.numpy()[agree], d[mode + "betas"][agree]).max() <= 2e-3


def test_afni_faithful_surface_differs_from_the_exact_r(afni_mode):
    """The banded criterion is not the exact one (so the mode is really in use)."""
    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, "runs")
    a = fit_glm_arma11(Y, X, tr=2.0, device=DEV, verbose=False, force_exhaustive_search=True, **kw)
    set_afni_mode(False)
    b = fit_glm_arma11(Y, X, tr=2.0, device=DEV, verbose=False, force_exhaustive_search=True, **kw)
    assert np.abs(a.reml_likelihood.numpy() - b.reml_likelihood.numpy()).max() > 1e-6


def test_band_sums_match_the_dense_oracle(afni_mode):
    """ffs_reml_band_sums (strip mode): y'R^-1 y of residualised rows at a
    set of pairs by the band's forward substitution, against ||L^-1 y||^2
    with the FP64 oracle's dense whitener."""
    from fastfuncstuff_gb300 import _lib
    from fastfuncstuff_gb300.glm import engine

    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, "runs")
    T = X.shape[0]
    f = precompute_reml_grid(torch.from_numpy(X), T, d["a_grid"], d["b_grid"], DEV, run_starts=kw["run_starts"],
                             use_double=True)
    pre = engine.prep(torch.from_numpy(Y).to(DEV), f, want_yr_t=False, want_rows=True)
    V = Y.shape[0]
    pairs = np.arange(1, f.P, 7, dtype=np.int32)
    ids = torch.arange(V, dtype=torch.int32, device=DEV)
    count = torch.tensor([V], dtype=torch.int32, device=DEV)
    pairs_d = torch.from_numpy(pairs).to(DEV)
    out = torch.empty(len(pairs), V, dtype=torch.float32, device=DEV)
    lib = _lib.load()
    _lib.check(lib.ffs_reml_band_sums(V, count.data_ptr(), T, ids.data_ptr(), pre.rows.data_ptr(),
                                      f.band_coef.data_ptr(), f.band_w, f.band.data_ptr(), None, None, 0, None, None,
                                      0, 0, None, pairs_d.data_ptr(), len(pairs), out.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream), "ffs_reml_band_sums")
    torch.cuda.synchronize()
    og = o.valid_grid(d["a_grid"], d["b_grid"], np.float64)
    po = o.precompute_reml_grid(X.astype(np.float64), og, run_starts=kw["run_starts"])
    rows = pre.rows.cpu().numpy().astype(np.float64)
    got = out.cpu().numpy()
    for q, p in enumerate(pairs):
        want = ((po.whiteners[int(p)].dense() @ rows.T) ** 2).sum(0)
        np.testing.assert_allclose(got[q], want, rtol=2e-5, err_msg=f"pair {p}")


def test_afni_faithful_learned_fit(afni_mode):
    """The learned-seeded refine under the banded R: the window and strip
    criteria read y'R^-1 y from ffs_reml_band_sums, the fallback and the GLS
    run the banded full grid. The graph-replayed fit equals the eager one bit
    for bit; its pairs agree with the exhaustive banded full grid, and where
    they agree the GLS outputs are the full grid's and the likelihood agrees
    to float32 rounding."""
    from fastfuncstuff_gb300.glm import learned

    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, "runs")
    lay = G.run_layout(X.shape[0], kw["run_starts"])
    prop, _ = learned.train_proposal(torch.from_numpy(X).to(DEV), lay, d["a_grid"], d["b_grid"],
                                     n_voxels=200_000, epochs=6)
    opts = dict(kw, device=DEV, verbose=False, want_residuals=True)
    eager = fit_glm_arma11(Y, X, tr=2.0, proposal=prop, proposal_recenter=1, cuda_graphs=False, **opts)
    graph = fit_glm_arma11(Y, X, tr=2.0, proposal=prop, proposal_recenter=1, cuda_graphs=True, **opts)
    for name in ("arma_params", "reml_likelihood", "betas", "tstats", "sigma2", "residuals_whitened"):
        np.testing.assert_array_equal(getattr(graph, name).numpy(), getattr(eager, name).numpy(), err_msg=name)
    full = fit_glm_arma11(Y, X, tr=2.0, force_exhaustive_search=True, **opts)
    same = (eager.arma_params == full.arma_params).all(1).numpy()
    assert same.mean() >= 0.95, same.mean()
    np.testing.assert_array_equal(eager.betas.numpy()[same], full.betas.numpy()[same])
    np.testing.assert_allclose(eager.reml_likelihood.numpy()[same], full.reml_likelihood.numpy()[same], rtol=1e-5)
    # the voxels the learned fit answers differently lie no lower than the
    # full grid's optimum (a window holds no pair the full grid does not)
    assert (eager.reml_likelihood.numpy() >= full.reml_likelihood.numpy() - 1e-5 *
            np.abs(full.reml_likelihood.numpy())).all()


@pytest.mark.parametrize("tag", ["two", "runs"])
@pytest.mark.parametrize("exhaustive", [True, False])
def test_afni_faithful_dsort_matches_fp64_oracle(tag, exhaustive, afni_mode):
    """-dsort under the banded R: the voxel's regressors, its series and the
    residual whitened by the pair's band in the dsort GLS (block elimination
    against the band-built G and U), against the FP64 oracle in the same mode
    on the dsort fixture's data (two datasets per voxel, and one expanded per
    run)."""
    import warnings

    d = load_golden("dsort")
    kw = dict(a_grid=d["a_grid"], b_grid=d["b_grid"], run_starts=d["run_starts"], task_indices=[0, 1],
              want_ljung_box=True, want_residuals=True)
    if tag == "two":
        kw["dsort"] = d["D"]
    else:
        kw.update(dsort=d["D"][:, :1], dsort_run_bounds=[0, 64, 128])
    with warnings.catch_warnings():
        warnings.filterwarnings("ignore", message=".*constant.*")
        got = fit_glm_arma11(d["Y"], d["X"], tr=2.0, device=DEV, verbose=False, force_exhaustive_search=exhaustive,
                             **kw)
        ref = o.fit_glm_arma11(d["Y"], d["X"], use_double=True, fp64_scaled=True,
                               force_exhaustive_search=exhaustive, save_profile_likelihoods=True, **kw)
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    idx = _index(got.arma_params.numpy(), grid)
    check_selection(idx, ref.arma_index, ref.reml_lklhd_surface)
    same = idx == ref.arma_index
    full_got = np.concatenate([got.betas.numpy(), got.dsort_betas.numpy()], 1)[same]
    full_ref = np.concatenate([ref.betas, ref.dsort_betas], 1)[same]
    assert rel_maxnorm(full_got, full_ref).max() <= BETA_REL
    t_got = np.concatenate([got.tstats.numpy(), got.dsort_tstats.numpy()], 1)[same]
    t_ref = np.concatenate([ref.tstats, ref.dsort_tstats], 1)[same]
    assert rel_maxnorm(t_got, t_ref).max() <= BETA_REL
    np.testing.assert_allclose(got.sigma2.numpy()[same], ref.sigma2[same], rtol=1e-4)
    np.testing.assert_allclose(got.ljung_box.numpy()[same], ref.ljung_box[same], rtol=2e-3, atol=1e-3)
    scale = np.abs(ref.residuals_whitened[same]).max(1, keepdims=True)
    np.testing.assert_allclose(got.residuals_whitened.numpy()[same] / scale, ref.residuals_whitened[same] / scale,
                               atol=2e-4)


def _afni_designs(X):
    """Three designs of one shape: the case's own, its first column delayed by
    two samples, its second column with a slow ramp added."""
    X1 = X.copy()
    X1[:, 0] = np.roll(X[:, 0], 2)
    X2 = X.copy()
    X2[:, 1] = X[:, 1] + np.linspace(-0.5, 0.5, X.shape[0], dtype=X.dtype)
    return {0: X, 1: X1, 2: X2}


@pytest.mark.parametrize("tag", ["runs", "cens"])
@pytest.mark.parametrize("exhaustive", [True, False])
def test_afni_faithful_grouped_equals_per_group_fits(tag, exhaustive, afni_mode):
    """Grouped designs under the banded R: one multi-design build (the band
    factored once per pair by the pre-pass), the banded criterion per
    256-voxel design tile, the GLS whitened by the pair's band. Each voxel's
    arithmetic is the per-group fit's, so the results are those of fitting
    every group on its own; against the FP64 oracle's grouped fit as the
    other AFNI-mode fits are."""
    from fastfuncstuff_gb300 import fit_glm_arma11_grouped

    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, tag)
    designs = _afni_designs(X)
    gid = np.arange(Y.shape[0]) % 3
    opts = dict(kw, device=DEV, verbose=False, force_exhaustive_search=exhaustive, want_residuals=True)
    got = fit_glm_arma11_grouped(Y, designs, gid, tr=2.0, **opts)
    for h in range(3):
        m = gid == h
        ref = fit_glm_arma11(Y[m], designs[h], tr=2.0, **opts)
        for name in ("arma_params", "reml_likelihood", "betas", "tstats", "sigma2", "r2", "residuals_whitened"):
            np.testing.assert_array_equal(getattr(got, name).numpy()[m], getattr(ref, name).numpy(), err_msg=name)
    ref = o.fit_glm_arma11_grouped(Y, designs, gid, use_double=True, fp64_scaled=True,
                                   force_exhaustive_search=exhaustive, save_profile_likelihoods=True, **kw)
    grid = G.make_grid(d["a_grid"], d["b_grid"])
    idx = _index(got.arma_params.numpy(), grid)
    check_selection(idx, ref.arma_index, ref.reml_lklhd_surface)
    same = idx == ref.arma_index
    assert rel_maxnorm(got.betas.numpy()[same], ref.betas[same]).max() <= BETA_REL


def test_afni_faithful_grouped_learned_fit(afni_mode):
    """The grouped designs' learned fit under the banded R (window and strip
    sums from ffs_reml_band_sums, the grouped banded full grid for the
    fallback): its pairs agree with the grouped exhaustive banded full grid,
    and where they agree the GLS outputs are the full grid's."""
    from fastfuncstuff_gb300 import fit_glm_arma11_grouped
    from fastfuncstuff_gb300.glm import learned

    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, "runs")
    designs = _afni_designs(X)
    gid = np.arange(Y.shape[0]) % 3
    lay = G.run_layout(X.shape[0], kw["run_starts"])
    fam = torch.from_numpy(np.stack([designs[h] for h in range(3)])).to(DEV)
    prop, _ = learned.train_proposal(fam, lay, d["a_grid"], d["b_grid"], n_voxels=200_000, epochs=6)
    opts = dict(kw, device=DEV, verbose=False)
    got = fit_glm_arma11_grouped(Y, designs, gid, tr=2.0, proposal=prop, proposal_recenter=1, **opts)
    full = fit_glm_arma11_grouped(Y, designs, gid, tr=2.0, force_exhaustive_search=True, **opts)
    same = (got.arma_params == full.arma_params).all(1).numpy()
    assert same.mean() >= 0.95, same.mean()
    np.testing.assert_array_equal(got.betas.numpy()[same], full.betas.numpy()[same])
    assert (got.reml_likelihood.numpy() >= full.reml_likelihood.numpy() - 1e-5 *
            np.abs(full.reml_likelihood.numpy())).all()
