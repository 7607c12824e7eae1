"""Generate the golden fixtures by running the reference implementation itself.

Run in a container that has the fastfuncstuff sources (read-only is fine):

    python tests/golden/make_golden.py /path/to/fastfuncstuff-checkout

The reference's hot path never touches nibabel, but its package imports it at
module load, so a throwaway stub package is put on ``sys.path`` first (created in
a temporary directory, never in the checkout). Every case below is a seeded
synthetic input; the fixture stores the inputs and the reference's outputs so the
oracle and the CUDA path can be checked without the reference present.

Cases (all on ``device=cpu``):

* ``single``   one run, N=96, p=6, V=240, grid linspace(-0.8, 0.8, 17)
* ``multirun`` three runs of 48, task_indices, one GLT, Ljung-Box, residuals
* ``censored`` two runs with censored TRs (``tau`` from build_censor_run_info)
* ``grouped``  fit_glm_arma11_grouped with three per-group designs
* ``afni``     the default AFNI grid (9 x 17), default selector only
* ``afni_faithful`` ``set_afni_mode(True)``: the banded covariance, AFNI's
               grid filter and ltop; two runs, and two censored runs
* ``baseline`` a raw 1000-baseline series (the conditioning test's shape)
* ``ljung``    the reference test-suite's Ljung-Box series and AFNI golden values
* ``grid``     logdet(R), logdet(X_w'X_w), X_w and Q of a small precompute
* ``sets``     column_sets (Wald F, temporal SD and coefficient of each set),
               two runs, one set naming a column outside the design
* ``global``   estimate_per_voxel=False: one (a, b) from the mean series, then
               the GLS of every voxel at it
* ``dsort``    voxelwise regressors (-dsort): two datasets per voxel, and one
               dataset expanded per run (dsort_run_bounds), with task columns,
               a GLT, Ljung-Box, residuals and column sets over [X | D]

Each fit is run in four reference modes: FP64 exhaustive, FP64 default
(hierarchical), float32 default and float32 exhaustive, with the likelihood
surface saved where the reference offers it. ``--only NAME`` writes one case.
"""

from __future__ import annotations

import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE


def _stub_nibabel(root: Path) -> None:
    pkg = root / "nibabel"
    pkg.mkdir(parents=True, exist_ok=True)
    (pkg / "__init__.py").write_text(
        "import sys, types\n"
        "class _Any:\n"
        "    def __getattr__(self, k): return _Any()\n"
        "    def __call__(self, *a, **k): return _Any()\n"
        "for _s in ['nifti1','spatialimages','processing','affines','orientations','funcs',"
        "'cifti2','gifti','freesurfer','streamlines']:\n"
        "    _m = types.ModuleType('nibabel.' + _s); _m.__getattr__ = lambda k: _Any()\n"
        "    sys.modules['nibabel.' + _s] = _m\n"
        "def __getattr__(k): return _Any()\n"
    )


def _legendre(n: int, deg: int) -> np.ndarray:
    x = np.linspace(-1.0, 1.0, n)
    cols = [np.polynomial.legendre.Legendre.basis(d)(x) for d in range(deg + 1)]
    return np.stack(cols, 1)


def _arma_noise(rng, n, V, a, b, burn=100):
    e = rng.standard_normal((n + burn, V))
    y = np.zeros_like(e)
    y[0] = e[0]
    for t in range(1, n + burn):
        y[t] = a * y[t - 1] + e[t] + b * e[t - 1]
    y = y[burn:]
    return ((y - y.mean(0)) / y.std(0, ddof=1)).T


def _case(seed, lens, p_task=2, V=240, censor=None, baseline=0.0):
    rng = np.random.default_rng(seed)
    n = sum(lens)
    tasks = (rng.random((n, p_task)) < 0.15).astype(np.float64)
    tasks = np.apply_along_axis(lambda c: np.convolve(c, [0, 0.4, 1.0, 0.7, 0.3, 0.1])[:n], 0, tasks)
    drift = np.zeros((n, 3 * len(lens)))
    s = 0
    for r, m in enumerate(lens):
        drift[s : s + m, 3 * r : 3 * r + 3] = _legendre(m, 2)
        s += m
    X = np.concatenate([tasks, drift], 1)
    a = rng.uniform(0.1, 0.7, V)
    b = rng.uniform(-0.4, 0.3, V)
    noise = np.concatenate([_arma_noise(rng, n, 1, a[v], b[v]) for v in range(V)], 0)
    beta = rng.standard_normal((V, X.shape[1]))
    Y = beta @ X.T + rng.uniform(0.5, 2.0, (V, 1)) * noise + baseline
    keep = None
    if censor is not None:
        keep = np.sort(rng.choice(n, n - censor, replace=False))
        X, Y = X[keep], Y[:, keep]
    return X.astype(np.float32), Y.astype(np.float32), keep


def main(ref_root: str, only: str | None = None) -> None:
    tmp = Path(tempfile.mkdtemp(prefix="ffs_stub_"))
    _stub_nibabel(tmp)
    sys.path[:0] = [str(tmp), ref_root]
    os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
    sys.dont_write_bytecode = True
    import torch

    torch.set_num_threads(4)
    from fastfuncstuff.glm import arma
    from fastfuncstuff.glm.arma import (
        build_censor_run_info,
        fit_glm_arma11,
        fit_glm_arma11_grouped,
        precompute_reml_grid,
    )

    cpu = torch.device("cpu")
    g17 = torch.linspace(-0.8, 0.8, 17)

    def modes(X, Y, **kw):
        out = {}
        for name, extra in {
            "f64_exh": dict(use_double=True, force_exhaustive_search=True),
            "f64_def": dict(use_double=True),
            "f32_def": dict(),
            "f32_exh": dict(force_exhaustive_search=True),
        }.items():
            r = fit_glm_arma11(
                torch.from_numpy(Y), torch.from_numpy(X), tr=2.0, device=cpu, verbose=False,
                save_profile_likelihoods=True, **extra, **kw,
            )
            for attr in ("betas", "tstats", "r2", "arma_params", "arma_lambda", "reml_likelihood",
                         "sigma2", "fstats", "residuals", "residuals_whitened", "ljung_box",
                         "contrast_betas", "contrast_tstats", "reml_lklhd_surface"):
                v = getattr(r, attr, None)
                if attr == "reml_lklhd_surface" and not name.endswith("exh"):
                    continue  # the surface does not depend on the selector
                if attr in ("residuals", "residuals_whitened") and name != "f64_def":
                    continue
                if v is not None:
                    out[f"{name}__{attr}"] = v.numpy()
            out[f"{name}__dof"] = np.array(r.dof)
            if r.ljung_box_dof is not None:
                out[f"{name}__ljung_box_dof"] = np.array(r.ljung_box_dof)
        return out

    # AFNI-faithful mode (banded R, near-white pairs dropped, AFNI's ltop):
    # two runs, then two censored runs (the band counts tau, not rows)
    arma.set_afni_mode(True)
    try:
        out = {}
        X, Y, _ = _case(30, [80, 80], V=150)
        out.update({f"runs_{k}": v for k, v in modes(X, Y, a_grid=g17, b_grid=g17, run_starts=[0, 80]).items()})
        Xc, Yc, keep = _case(31, [70, 74], V=100, censor=10)
        starts, tau = build_censor_run_info([0, 70], 144, keep.tolist())
        out.update({f"cens_{k}": v for k, v in modes(Xc, Yc, a_grid=g17, b_grid=g17, run_starts=starts,
                                                     tau=tau).items()})
    finally:
        arma.set_afni_mode(False)
    np.savez_compressed(OUT / "afni_faithful.npz", X=X, Y=Y, Xc=Xc, Yc=Yc, a_grid=g17.numpy(),
                        b_grid=g17.numpy(), run_starts=np.array([0, 80]), cens_run_starts=np.array(starts),
                        tau=tau.numpy(), keep=keep, corcut=np.array(1e-4), **out)
    if only == "afni_faithful":
        print("wrote", OUT / "afni_faithful.npz")
        return

    # global ARMA: (a, b) estimated once from the mean series
    X, Y, _ = _case(22, [60, 60], p_task=2, V=150)
    out = {}
    for name, extra in {"f64": dict(use_double=True), "f32": dict()}.items():
        r = fit_glm_arma11(torch.from_numpy(Y), torch.from_numpy(X), tr=2.0, device=cpu, verbose=False,
                           a_grid=g17, b_grid=g17, run_starts=[0, 60], estimate_per_voxel=False, **extra)
        for attr in ("betas", "tstats", "arma_params", "reml_likelihood", "sigma2", "fstats", "r2", "arma_lambda"):
            out[f"{name}__{attr}"] = getattr(r, attr).numpy()
    np.savez_compressed(OUT / "global.npz", X=X, Y=Y, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        run_starts=np.array([0, 60]), **out)
    if only == "global":
        print("wrote", OUT / "global.npz")
        return

    # -dsort: per-voxel regressors (one smooth series correlated with the data,
    # one independent; three voxels with a constant series that the guard
    # replaces), then one dataset expanded per run
    X, Y, _ = _case(20, [64, 64], p_task=2, V=120)
    rng = np.random.default_rng(21)
    T = X.shape[0]
    sm = np.apply_along_axis(lambda c: np.convolve(c, np.ones(5) / 5, mode="same"), 1, rng.standard_normal((120, T)))
    D = np.stack([0.3 * Y / Y.std(1, keepdims=True) + sm, rng.standard_normal((120, T))], 1).astype(np.float32)
    D[:3, 1] = 2.5
    glt = np.zeros((1, X.shape[1]), np.float32)
    glt[0, 0], glt[0, 1] = 1.0, -1.0
    K = X.shape[1]
    base = dict(a_grid=g17, b_grid=g17, run_starts=[0, 64], task_indices=[0, 1], glt_labels=["t0-t1"],
                glt_matrices=[glt], want_ljung_box=True, want_residuals=True)
    out = {}
    for tag, dkw, sets in (("two", dict(dsort=torch.from_numpy(D)), [[0], [K], [K, K + 1], [0, 1, K]]),
                           ("runs", dict(dsort=torch.from_numpy(D[:, :1]), dsort_run_bounds=[0, 64, 128]),
                            [[K], [K, K + 1], [2, 3]])):
        for name, extra in {"f64_def": dict(use_double=True), "f32_def": dict(),
                            "f32_exh": dict(force_exhaustive_search=True)}.items():
            r = fit_glm_arma11(torch.from_numpy(Y), torch.from_numpy(X), tr=2.0, device=cpu, verbose=False,
                               column_sets=sets, **base, **dkw, **extra)
            for attr in ("betas", "tstats", "dsort_betas", "dsort_tstats", "sigma2", "fstats", "r2",
                         "arma_params", "residuals", "residuals_whitened", "predicted", "ljung_box",
                         "contrast_betas", "contrast_tstats", "set_fstats", "set_sd", "set_coef", "r2_partial"):
                v = getattr(r, attr, None)
                if attr in ("residuals", "residuals_whitened", "predicted") and name != "f64_def":
                    continue
                if v is not None:
                    out[f"{tag}_{name}__{attr}"] = v.numpy()
            out[f"{tag}_{name}__dof"] = np.array(r.dof)
        out[f"{tag}__sets_ptr"] = np.cumsum([0] + [len(c) for c in sets])
        out[f"{tag}__sets_idx"] = np.concatenate([np.asarray(c) for c in sets])
    np.savez_compressed(OUT / "dsort.npz", X=X, Y=Y, D=D, glt=glt, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        run_starts=np.array([0, 64]), task_indices=np.array([0, 1]), **out)
    if only == "dsort":
        print("wrote", OUT / "dsort.npz")
        return

    # column sets: Wald F, SD and coefficient per set (one set is outside the
    # design, so its statistics are NaN)
    X, Y, _ = _case(19, [64, 64], p_task=3, V=160)
    sets = [[0], [0, 1], [2, 3, 4], [1, 99], [5]]
    kw = dict(a_grid=g17, b_grid=g17, run_starts=[0, 64], column_sets=sets)
    out = {}
    for name, extra in {"f64_def": dict(use_double=True), "f32_def": dict(),
                        "f32_exh": dict(force_exhaustive_search=True)}.items():
        r = fit_glm_arma11(torch.from_numpy(Y), torch.from_numpy(X), tr=2.0, device=cpu, verbose=False,
                           **extra, **kw)
        for attr in ("betas", "sigma2", "arma_params", "set_fstats", "set_sd", "set_coef"):
            out[f"{name}__{attr}"] = getattr(r, attr).numpy()
    np.savez_compressed(OUT / "sets.npz", X=X, Y=Y, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        run_starts=np.array([0, 64]), set_ptr=np.cumsum([0] + [len(c) for c in sets]),
                        set_idx=np.concatenate([np.asarray(c) for c in sets]), **out)
    if only == "sets":
        print("wrote", OUT / "sets.npz")
        return


    # single run
    X, Y, _ = _case(11, [96])
    np.savez_compressed(OUT / "single.npz", X=X, Y=Y, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        **modes(X, Y, a_grid=g17, b_grid=g17))

    # three runs, task columns, one GLT, Ljung-Box and residuals
    X, Y, _ = _case(12, [48, 48, 48], p_task=2, V=160)
    glt = np.zeros((1, X.shape[1]), np.float32)
    glt[0, 0], glt[0, 1] = 1.0, -1.0
    kw = dict(a_grid=g17, b_grid=g17, run_starts=[0, 48, 96], task_indices=[0, 1],
              glt_labels=["t0-t1"], glt_matrices=[glt], want_ljung_box=True, want_residuals=True)
    np.savez_compressed(OUT / "multirun.npz", X=X, Y=Y, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        run_starts=np.array([0, 48, 96]), task_indices=np.array([0, 1]), glt=glt,
                        **modes(X, Y, **kw))

    # censored runs: tau from build_censor_run_info
    lens = [60, 72]
    X, Y, keep = _case(13, lens, V=120, censor=8)
    starts, tau = build_censor_run_info([0, 60], 132, keep.tolist())
    kw = dict(a_grid=g17, b_grid=g17, run_starts=starts, tau=tau, want_ljung_box=True)
    np.savez_compressed(OUT / "censored.npz", X=X, Y=Y, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        run_starts=np.array(starts), tau=tau.numpy(), keep=keep,
                        orig_run_starts=np.array([0, 60]), n_total=np.array(132),
                        **modes(X, Y, **kw))

    # grouped designs: three groups, shared grid
    X0, Y, _ = _case(14, [80], V=150)
    rng = np.random.default_rng(15)
    designs = {}
    for h in range(3):
        Xh = X0.copy()
        Xh[:, :2] = np.roll(X0[:, :2], h, axis=0) * (1.0 + 0.2 * h)
        designs[h] = Xh.astype(np.float32)
    gid = rng.integers(0, 3, Y.shape[0])
    grouped = {}
    for name, extra in {"f64_exh": dict(use_double=True, force_exhaustive_search=True),
                        "f32_def": dict()}.items():
        r = fit_glm_arma11_grouped(
            torch.from_numpy(Y), {h: torch.from_numpy(d) for h, d in designs.items()},
            torch.from_numpy(gid), tr=2.0, a_grid=g17, b_grid=g17, device=cpu, verbose=False,
            **extra,
        )
        for attr in ("betas", "tstats", "arma_params", "reml_likelihood", "sigma2", "fstats", "r2"):
            grouped[f"{name}__{attr}"] = getattr(r, attr).numpy()
    np.savez_compressed(OUT / "grouped.npz", Y=Y, gid=gid, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        **{f"X{h}": d for h, d in designs.items()}, **grouped)

    # AFNI default grid, default selector
    X, Y, _ = _case(16, [100], V=200)
    out = {}
    for name, extra in {"f64_def": dict(use_double=True), "f32_def": dict()}.items():
        r = fit_glm_arma11(torch.from_numpy(Y), torch.from_numpy(X), tr=2.0, device=cpu,
                           verbose=False, **extra)
        out[f"{name}__arma_params"] = r.arma_params.numpy()
        out[f"{name}__reml_likelihood"] = r.reml_likelihood.numpy()
        out[f"{name}__betas"] = r.betas.numpy()
    np.savez_compressed(OUT / "afni.npz", X=X, Y=Y, **out)

    # raw 1000 baseline, three runs of 60 (the conditioning case's shape)
    X, Y, _ = _case(17, [60, 60, 60], V=40, baseline=1000.0)
    np.savez_compressed(OUT / "baseline.npz", X=X, Y=Y, a_grid=g17.numpy(), b_grid=g17.numpy(),
                        run_starts=np.array([0, 60, 120]),
                        **modes(X, Y, a_grid=g17, b_grid=g17, run_starts=[0, 60, 120]))

    # Ljung-Box: the reference test-suite's seeded series and AFNI's golden outputs
    sys.path.insert(0, str(Path(ref_root) / "tests"))
    import test_ljung_box as tlb

    s = tlb._series()
    lj = {
        "white": s["white"], "ar1": s["ar1"], "offset": s["offset"],
        "censored": s["censored"][0], "censored_keep": s["censored"][1],
        "tworun": s["tworun"][0], "tworun_tau": s["tworun"][1],
        "golden_keys": np.array(list(tlb.GOLDEN.keys())),
        "golden_vals": np.array(list(tlb.GOLDEN.values())),
    }
    for key, val, lag, tau in [("white_h20", s["white"], 20, None), ("white_auto", s["white"], None, None),
                               ("ar1_h20", s["ar1"], 20, None), ("offset_h20", s["offset"], 20, None),
                               ("censored_h18", s["censored"][0], 18, s["censored"][1]),
                               ("tworun_h20", s["tworun"][0], 20, s["tworun"][1]),
                               ("tworun_notau_h20", s["tworun"][0], 20, None)]:
        tt = torch.from_numpy(np.asarray(tau, np.int64)) if tau is not None else None
        lj[f"ref_{key}"] = np.array(arma._ljung_box_batched(
            torch.from_numpy(np.asarray(val, np.float64)).reshape(1, -1), lag, tt).item())
    np.savez_compressed(OUT / "ljung.npz", **lj)

    # grid precompute dump (FP64) for K1 checks: two runs, small p
    X, _, _ = _case(18, [40, 56], V=1)
    Xt = torch.from_numpy(X.astype(np.float64))
    g9 = torch.linspace(-0.8, 0.8, 9)
    pre = precompute_reml_grid(Xt, 96, g9, g9, cpu, dtype=torch.float64, run_starts=[0, 40])
    keys = list(pre.keys())
    np.savez_compressed(
        OUT / "grid.npz", X=X, a_grid=g9.numpy(), b_grid=g9.numpy(), run_starts=np.array([0, 40]),
        pairs=np.array(keys, dtype=np.float64),
        logdet_R=np.array([pre[k]["logdet_Rcorr"].item() for k in keys]),
        logdet_XtX=np.array([pre[k]["logdet_XwTXw"].item() for k in keys]),
        X_w=np.stack([pre[k]["X_w"].numpy() for k in keys]),
        Q=np.stack([pre[k]["Q"].numpy() for k in keys]),
        Linv=np.stack([pre[k]["whitener"].dense().numpy() for k in keys[::8]]),
    )
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only")]
    only = next((a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")), None)
    main(args[0] if args else os.environ.get("FFS_REFERENCE", "."), only)
