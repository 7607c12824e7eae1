"""The CPU oracle against golden vectors produced by the reference itself.

Fixtures come from ``tests/golden/make_golden.py``, which runs the reference's
``fit_glm_arma11`` / ``fit_glm_arma11_grouped`` / ``precompute_reml_grid`` /
``_ljung_box_batched`` on seeded inputs. These tests pin the oracle before it is
trusted to judge the CUDA path.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import reml as o
from tests.conftest import load_golden


def _close(a, b, rtol, atol=0.0):
    np.testing.assert_allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=rtol, atol=atol)


def case_kwargs(d) -> dict:
    """The fit options each golden case was generated with (make_golden.py)."""
    args = dict(a_grid=d["a_grid"], b_grid=d["b_grid"])
    if "run_starts" in d:
        args["run_starts"] = d["run_starts"]
    if "tau" in d:
        args["tau"] = d["tau"]
        args["want_ljung_box"] = True
    if "task_indices" in d:
        args.update(task_indices=list(d["task_indices"]), glt_matrices=[d["glt"][0]],
                    want_ljung_box=True, want_residuals=True)
    if "set_ptr" in d:
        ptr, idx = d["set_ptr"], d["set_idx"]
        args["column_sets"] = [[int(c) for c in idx[ptr[g]:ptr[g + 1]]] for g in range(len(ptr) - 1)]
    return args


def _fit(d, **kw):
    args = case_kwargs(d)
    args.update(kw)
    return o.fit_glm_arma11(d["Y"], d["X"], **args)


# ---------------------------------------------------------------- grid + lambda


def test_valid_grid_counts_match_reference():
    d = load_golden("grid")
    grid = o.valid_grid(d["a_grid"], d["b_grid"], np.float64)
    pairs = np.stack([grid.a, grid.b], 1).astype(np.float64)
    np.testing.assert_array_equal(pairs, d["pairs"])


def test_lambda_known_values():
    # fastfuncstuff tests/test_arma_extended.py:42-57: AR(1) case and white noise
    assert abs(float(o.arma_lambda_f32(0.5, 0.0)) - 0.5) < 1e-6
    assert float(o.arma_lambda_f32(0.0, 0.0)) == 0.0
    a, b = 0.6, 0.2
    assert abs(float(o.arma_lambda_f32(a, b)) - (a + b) * (1 + a * b) / (1 + b * b + 2 * a * b)) < 1e-6


def test_ensure_zero_in_grid():
    a, b = o.ensure_zero_in_grid(np.array([0.1, 0.2, 0.3], np.float32), np.array([2.98e-8, 0.5], np.float32))
    assert a.tolist()[0] == 0.0 and len(a) == 4
    assert b.tolist() == [0.0, 0.5]


def test_censor_run_info_known_answer():
    # fastfuncstuff tests/test_arma_censoring.py:82-91
    starts, tau = o.build_censor_run_info([0, 5], 10, [0, 1, 3, 4, 5, 6, 8, 9])
    assert starts == [0, 4]
    assert tau.tolist() == [0, 1, 3, 4, 0, 1, 3, 4]
    starts, tau = o.build_censor_run_info([0, 100], 200, None)
    assert starts == [0, 100] and tau is None


def test_censored_lag2_gap():
    # fastfuncstuff tests/test_arma_censoring.py:36-49: a censored TR puts its
    # survivors at lag 2 (correlation lam*a)
    a, b = 0.6, 0.2
    lam = float(o.arma_lambda_f32(a, b))
    R = o.corr_block(a, lam, np.array([0, 1, 3, 4]))
    assert abs(R[1, 2] - lam * a) < 1e-6
    assert abs(R[0, 1] - lam) < 1e-6


def test_run_bounds():
    assert o.run_bounds(10, None) == [(0, 10)]
    assert o.run_bounds(10, [4]) == [(0, 4), (4, 10)]


# ---------------------------------------------------------- precompute (grid)


def test_precompute_matches_reference():
    d = load_golden("grid")
    grid = o.valid_grid(d["a_grid"], d["b_grid"], np.float64)
    pre = o.precompute_reml_grid(d["X"].astype(np.float64), grid, run_starts=d["run_starts"])
    _close(pre.logdet_R, d["logdet_R"], rtol=1e-10, atol=1e-9)
    _close(pre.logdet_XtX, d["logdet_XtX"], rtol=1e-10, atol=1e-9)
    _close(pre.X_w, d["X_w"], rtol=1e-9, atol=1e-9)
    _close(pre.Q, d["Q"], rtol=1e-8, atol=1e-9)
    dense = np.stack([w.dense() for w in pre.whiteners[::8]])
    _close(dense, d["Linv"], rtol=1e-9, atol=1e-9)


# ------------------------------------------------------------------------ fits


@pytest.mark.parametrize("case", ["single", "multirun", "censored", "baseline"])
def test_fp64_exhaustive_matches_reference(case):
    d = load_golden(case)
    kw = case_kwargs(d)
    r = _fit(d, use_double=True, force_exhaustive_search=True, save_profile_likelihoods=True)
    ref = "f64_exh__"
    np.testing.assert_array_equal(r.arma_params, d[ref + "arma_params"])
    _close(r.reml_lklhd_surface, d[ref + "reml_lklhd_surface"], rtol=2e-5)
    _close(r.reml_likelihood, d[ref + "reml_likelihood"], rtol=1e-8, atol=1e-5)
    _close(r.betas, d[ref + "betas"], rtol=1e-6, atol=1e-6)
    _close(r.tstats, d[ref + "tstats"], rtol=1e-6, atol=1e-6)
    _close(r.sigma2, d[ref + "sigma2"], rtol=1e-7)
    _close(r.fstats, d[ref + "fstats"], rtol=1e-6, atol=1e-6)
    _close(r.r2, d[ref + "r2"], rtol=0, atol=1e-6)
    _close(r.arma_lambda, d[ref + "arma_lambda"], rtol=1e-12, atol=1e-12)
    if case == "multirun":
        _close(r.contrast_betas, d[ref + "contrast_betas"], rtol=1e-6, atol=1e-6)
        _close(r.contrast_tstats, d[ref + "contrast_tstats"], rtol=1e-6, atol=1e-6)
    if kw.get("want_ljung_box"):
        _close(r.ljung_box, d[ref + "ljung_box"], rtol=1e-5, atol=1e-5)
        assert r.ljung_box_dof == int(d[ref + "ljung_box_dof"])


@pytest.mark.parametrize("case", ["single", "multirun", "censored", "baseline"])
def test_fp64_default_selector_matches_reference(case):
    d = load_golden(case)
    r = _fit(d, use_double=True)
    np.testing.assert_array_equal(r.arma_params, d["f64_def__arma_params"])
    _close(r.reml_likelihood, d["f64_def__reml_likelihood"], rtol=1e-8, atol=1e-5)


@pytest.mark.parametrize("case", ["single", "multirun", "censored", "baseline"])
def test_fp32_mode_matches_reference(case):
    """The oracle in float32 mode mirrors the reference's default run."""
    d = load_golden(case)
    for mode, kw in (("f32_def", {}), ("f32_exh", dict(force_exhaustive_search=True))):
        r = _fit(d, use_double=False, **kw)
        agree = (r.arma_params == d[mode + "__arma_params"]).all(1).mean()
        assert agree >= 0.97, (mode, agree)
        same = (r.arma_params == d[mode + "__arma_params"]).all(1)
        _close(r.betas[same], d[mode + "__betas"][same], rtol=2e-3, atol=2e-3)
        _close(r.reml_likelihood[same], d[mode + "__reml_likelihood"][same], rtol=1e-5, atol=1e-3)


def test_column_sets_match_reference():
    """column_sets (fastfuncstuff/glm/arma.py:3542-3586, unscaled at :5845-5848):
    the Wald F, temporal SD and one-column coefficient of each set, NaN for the
    set that names a column outside the design; FP64 and float32 modes."""
    d = load_golden("sets")
    r = _fit(d, use_double=True)
    np.testing.assert_array_equal(r.arma_params, d["f64_def__arma_params"])
    for name in ("set_fstats", "set_sd", "set_coef"):
        ref = d["f64_def__" + name]
        got = getattr(r, name)
        np.testing.assert_array_equal(np.isnan(got), np.isnan(ref), err_msg=name)
        _close(np.nan_to_num(got), np.nan_to_num(ref), rtol=1e-7, atol=1e-9)
    for mode, kw in (("f32_def", {}), ("f32_exh", dict(force_exhaustive_search=True))):
        r = _fit(d, use_double=False, **kw)
        same = (r.arma_params == d[mode + "__arma_params"]).all(1)
        assert same.mean() >= 0.97, (mode, same.mean())
        for name in ("set_fstats", "set_sd", "set_coef"):
            ref = d[f"{mode}__{name}"][same]
            got = getattr(r, name)[same]
            np.testing.assert_array_equal(np.isnan(got), np.isnan(ref), err_msg=name)
            _close(np.nan_to_num(got), np.nan_to_num(ref), rtol=2e-3, atol=2e-3)


def test_fp64_scaled_oracle_tracks_fp32_reference():
    """The FP64 oracle on float32-mode semantics selects what the float32 reference does
    (fastfuncstuff tests/test_reml_conditioning.py:24-37: float32 selection equals
    float64 selection, sigma2 within rtol 1e-3)."""
    d = load_golden("baseline")
    r = _fit(d, use_double=True, fp64_scaled=True, force_exhaustive_search=True)
    np.testing.assert_array_equal(r.arma_params.astype(np.float32), d["f32_exh__arma_params"])
    _close(r.sigma2, d["f32_exh__sigma2"], rtol=1e-3, atol=1e-5)
    # and the FP64 unscaled selection agrees too
    np.testing.assert_array_equal(d["f64_exh__arma_params"].astype(np.float32), d["f32_exh__arma_params"])


def test_hierarchical_surface_equals_subset_descent():
    """fastfuncstuff tests/test_arma_extended.py:327-397: the descent on the
    surface selects what the subset-GEMM descent selects."""
    d = load_golden("single")
    X, Y = d["X"].astype(np.float64), d["Y"].astype(np.float64)
    grid = o.valid_grid(d["a_grid"], d["b_grid"], np.float64)
    pre = o.precompute_reml_grid(X, grid)
    i_sub, l_sub = o.search_hierarchical_subset(X, Y, pre)
    _, _, surf = o.search_exhaustive(X, Y, pre, return_surface=True)
    i_surf, l_surf = o.select_hierarchical_from_surface(surf, grid)
    np.testing.assert_array_equal(i_sub, i_surf)
    _close(l_sub, l_surf, rtol=1e-12)


def test_afni_default_grid():
    d = load_golden("afni")
    r = o.fit_glm_arma11(d["Y"], d["X"], use_double=True)
    np.testing.assert_array_equal(r.arma_params, d["f64_def__arma_params"])
    _close(r.betas, d["f64_def__betas"], rtol=1e-6, atol=1e-6)


def test_grouped_matches_reference():
    d = load_golden("grouped")
    designs = {h: d[f"X{h}"] for h in range(3)}
    r = o.fit_glm_arma11_grouped(d["Y"], designs, d["gid"], a_grid=d["a_grid"], b_grid=d["b_grid"],
                                 use_double=True, force_exhaustive_search=True)
    np.testing.assert_array_equal(r.arma_params, d["f64_exh__arma_params"])
    _close(r.betas, d["f64_exh__betas"], rtol=1e-6, atol=1e-6)
    _close(r.tstats, d["f64_exh__tstats"], rtol=1e-6, atol=1e-6)
    _close(r.reml_likelihood, d["f64_exh__reml_likelihood"], rtol=1e-8, atol=1e-5)


def test_grouped_errors():
    Y = np.zeros((4, 10), np.float32)
    with pytest.raises(KeyError):
        o.fit_glm_arma11_grouped(Y, {0: np.ones((10, 2))}, [0, 0, 1, 1])
    with pytest.raises(ValueError):
        o.fit_glm_arma11_grouped(Y, {0: np.ones((10, 2)), 1: np.ones((10, 3))}, [0, 0, 1, 1])


def test_fit_errors():
    with pytest.raises(ValueError):
        o.fit_glm_arma11(np.zeros((2, 3, 10)), np.ones((10, 2)))
    with pytest.raises(ValueError):
        o.fit_glm_arma11(np.zeros((2, 10)), np.ones((9, 2)))


# ------------------------------------------------------------------ Ljung-Box


def test_ljung_box_afni_golden():
    """AFNI's ljung_box_uneven outputs recorded by the reference's own tests."""
    d = load_golden("ljung")
    gold = dict(zip(d["golden_keys"].tolist(), d["golden_vals"].tolist()))
    cases = {
        "white_h20": (d["white"], 20, None),
        "white_auto": (d["white"], None, None),
        "ar1_h20": (d["ar1"], 20, None),
        "offset_h20": (d["offset"], 20, None),
        "censored_h18": (d["censored"], 18, d["censored_keep"]),
        "tworun_h20": (d["tworun"], 20, d["tworun_tau"]),
        "tworun_notau_h20": (d["tworun"], 20, None),
    }
    for key, (val, lag, tau) in cases.items():
        got = float(o.ljung_box(val, lag, tau)[0])
        assert got == pytest.approx(gold[key], rel=1e-12), key
        assert got == pytest.approx(float(d[f"ref_{key}"]), rel=1e-12), key
    # out-of-range lag is re-derived; degenerate inputs return 0
    assert float(o.ljung_box(d["white"], 10_000)[0]) == pytest.approx(gold["white_auto"], rel=1e-12)
    assert float(o.ljung_box(np.random.default_rng(0).standard_normal(9), 4)[0]) == 0.0
    assert float(o.ljung_box(np.zeros(100), 10)[0]) == 0.0


def test_ljung_box_max_lag_formula():
    assert o.ljung_box_max_lag(200, n_regressors=10, min_run=200) == 28
    assert o.ljung_box_max_lag(60, n_regressors=40, min_run=60) == 30


@pytest.mark.parametrize("tag", ["two", "runs"])
def test_dsort_matches_reference(tag):
    """-dsort (fastfuncstuff/glm/arma.py:3207-3539): the per-voxel GLS with
    [X | D_v] at the pairs estimated without D, the constant-series guard, the
    per-run expansion of a compact dataset (dsort_run_bounds), dof T - p - q,
    and every statistic of the extended fit, in FP64 and float32 modes."""
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
    r = o.fit_glm_arma11(d["Y"], d["X"], use_double=True, **kw)
    ref = f"{tag}_f64_def__"
    assert r.dof == int(d[ref + "dof"])
    np.testing.assert_array_equal(r.arma_params, d[ref + "arma_params"])
    for name, rtol, atol in (("betas", 1e-6, 1e-6), ("tstats", 1e-6, 1e-6), ("dsort_betas", 1e-6, 1e-6),
                             ("dsort_tstats", 1e-6, 1e-6), ("sigma2", 1e-7, 0), ("fstats", 1e-6, 1e-6),
                             ("r2", 0, 1e-7), ("residuals", 1e-6, 1e-6), ("residuals_whitened", 1e-6, 1e-6),
                             ("ljung_box", 1e-5, 1e-5), ("contrast_betas", 1e-6, 1e-6),
                             ("contrast_tstats", 1e-6, 1e-6)):
        _close(getattr(r, name), d[ref + name], rtol=rtol, atol=atol)
    for name in ("set_fstats", "set_sd", "set_coef"):
        got, want = getattr(r, name), d[ref + name]
        np.testing.assert_array_equal(np.isnan(got), np.isnan(want), err_msg=name)
        _close(np.nan_to_num(got), np.nan_to_num(want), rtol=1e-6, atol=1e-7)
    for mode, extra in (("f32_def", {}), ("f32_exh", dict(force_exhaustive_search=True))):
        r = o.fit_glm_arma11(d["Y"], d["X"], use_double=False, **kw, **extra)
        same = (r.arma_params == d[f"{tag}_{mode}__arma_params"]).all(1)
        assert same.mean() >= 0.97, (mode, same.mean())
        for name in ("betas", "dsort_betas", "sigma2"):
            _close(getattr(r, name)[same], d[f"{tag}_{mode}__{name}"][same], rtol=2e-3, atol=2e-3)


def test_global_arma_matches_reference():
    """estimate_per_voxel=False (fastfuncstuff/glm/arma.py:5603-5778): (a, b)
    from the mean series over the raw grid with the regularised scalar
    criterion (:1106-1294), its criterion for every voxel, then the GLS of
    every voxel at that pair."""
    d = load_golden("global")
    kw = dict(a_grid=d["a_grid"], b_grid=d["b_grid"], run_starts=d["run_starts"], estimate_per_voxel=False)
    r = o.fit_glm_arma11(d["Y"], d["X"], use_double=True, **kw)
    np.testing.assert_array_equal(r.arma_params, d["f64__arma_params"])
    _close(r.reml_likelihood, d["f64__reml_likelihood"], rtol=1e-6)  # the reference forms R in float32
    for name in ("betas", "tstats", "sigma2", "fstats", "r2"):
        _close(getattr(r, name), d["f64__" + name], rtol=2e-5, atol=1e-6)
    r = o.fit_glm_arma11(d["Y"], d["X"], use_double=False, **kw)
    np.testing.assert_array_equal(r.arma_params, d["f32__arma_params"])
    _close(r.betas, d["f32__betas"], rtol=2e-3, atol=2e-3)


@pytest.fixture
def afni_mode():
    o.set_afni_mode(True)
    yield
    o.set_afni_mode(False)


def afni_faithful_case(d, tag):
    """(Y, X, fit options) of the two afni_faithful cases (make_golden.py)."""
    if tag == "runs":
        return d["Y"], d["X"], dict(a_grid=d["a_grid"], b_grid=d["b_grid"], run_starts=d["run_starts"])
    return d["Yc"], d["Xc"], dict(a_grid=d["a_grid"], b_grid=d["b_grid"], run_starts=d["cens_run_starts"],
                                  tau=d["tau"])


def test_afni_bmax_known_values():
    # the band of AFNI's rcmat_arma11: last kept lag where lam * a^(k-1) ~ corcut
    assert o.afni_bmax(0.5, 5e-5, 1e-4) == 0  # below corcut: R = I
    assert o.afni_bmax(0.0, 0.3, 1e-4) == 1  # pure MA(1)
    assert o.afni_bmax(0.5, 0.5, 1e-4) == 1 + int(np.ceil(np.log(2e-4) / np.log(0.5)))
    assert o.afni_bmax(0.95, 0.9, 1e-4) == o.afni_bmax(0.9, 0.9, 1e-4)  # a clamped to 0.9
    assert o.afni_bmax(-0.6, 0.2, 1e-4) == o.afni_bmax(0.6, 0.2, 1e-4)


@pytest.mark.parametrize("tag", ["runs", "cens"])
def test_afni_faithful_matches_reference(tag, afni_mode):
    """set_afni_mode(True): the banded R (fastfuncstuff/glm/arma.py:95-109,
    :918-926, :1075-1089), the grid filter (:1031-1036) and AFNI's ltop."""
    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, tag)
    r = o.fit_glm_arma11(Y, X, use_double=True, force_exhaustive_search=True, save_profile_likelihoods=True,
                         **kw)
    ref = f"{tag}_f64_exh__"
    np.testing.assert_array_equal(r.arma_params, d[ref + "arma_params"])
    _close(r.reml_lklhd_surface, d[ref + "reml_lklhd_surface"], rtol=2e-5)
    _close(r.reml_likelihood, d[ref + "reml_likelihood"], rtol=1e-8, atol=1e-5)
    for name in ("betas", "tstats", "fstats"):
        _close(getattr(r, name), d[ref + name], rtol=1e-6, atol=1e-6)
    _close(r.sigma2, d[ref + "sigma2"], rtol=1e-7)
    r = o.fit_glm_arma11(Y, X, use_double=True, **kw)
    ref = f"{tag}_f64_def__"
    np.testing.assert_array_equal(r.arma_params, d[ref + "arma_params"])
    _close(r.reml_likelihood, d[ref + "reml_likelihood"], rtol=1e-8, atol=1e-5)
    _close(r.betas, d[ref + "betas"], rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("tag", ["runs"])
def test_afni_faithful_band_changes_the_answer(tag, afni_mode):
    """The banded R is not the dense one: the same fit without AFNI mode gives
    other likelihoods (and the golden fixture was made in AFNI mode)."""
    d = load_golden("afni_faithful")
    Y, X, kw = afni_faithful_case(d, tag)
    r = o.fit_glm_arma11(Y, X, use_double=True, force_exhaustive_search=True, **kw)
    o.set_afni_mode(False)
    dense = o.fit_glm_arma11(Y, X, use_double=True, force_exhaustive_search=True, **kw)
    assert np.abs(r.reml_likelihood - dense.reml_likelihood).max() > 1e-7
