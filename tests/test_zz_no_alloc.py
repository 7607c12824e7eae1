"""The allocation-free grid build (ffs_grid_build_noalloc), through the C ABI.

Callers that cannot allocate device memory where they build the grid (their
memory is owned by a framework allocator, or they are a foreign-language
embedding handed only input and output buffers) use this entry point; its FP64
scratch is a static device array of 16 MiB instead of a workspace argument.

The test builds the same grids with ffs_grid_build (caller workspace) and with
ffs_grid_build_noalloc, twice in a row with different shapes so the second call
starts from the first call's leftover scratch, and requires the outputs to
agree (the kernel is the same, so they agree exactly; the tolerance is the
factor tolerance of the other GPU tests). It also checks the size limit is
enforced with a clear error. This file is named to be collected last.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")


def _inputs(T, K, run_starts, a_grid, b_grid, seed):
    from fastfuncstuff_gb300.glm import grid as G

    g = G.make_grid(a_grid, b_grid)
    lay = G.run_layout(T, run_starts)
    X = torch.from_numpy(np.random.default_rng(seed).standard_normal((T, K)).astype(np.float32)).to(DEV)
    X[:, 0] = 1.0
    return g, lay, X


def _build(entry, g, lay, X, with_work):
    from fastfuncstuff_gb300 import _lib

    lib = _lib.load()
    T, K = X.shape
    P = g.P
    ld = (T + 63) // 64 * 64
    lt = (T + 3) // 4 * 4  # row stride of U and G
    f32 = dict(device=DEV, dtype=torch.float32)
    keep = dict(
        a=torch.from_numpy(g.a).to(DEV), b=torch.from_numpy(g.b).to(DEV),
        rs=torch.from_numpy(lay.run_start).to(DEV), tau=torch.from_numpy(lay.tau).to(DEV), X=X.contiguous(),
    )
    out = dict(
        coef=torch.full((P, T, 4), np.nan, **f32), logdet_R=torch.full((P,), np.nan, dtype=torch.float64, device=DEV),
        logdet_XtX=torch.full((P,), np.nan, dtype=torch.float64, device=DEV), U=torch.full((P, K, lt), np.nan, **f32),
        U_hi=torch.zeros(P * K, ld, dtype=torch.int16, device=DEV), U_lo=torch.zeros(P * K, ld, dtype=torch.int16, device=DEV),
        uexp=torch.zeros(P, dtype=torch.int32, device=DEV), G=torch.full((P, K, lt), np.nan, **f32),
        Adiag=torch.full((P, K), np.nan, **f32), XtX=torch.full((P, K, K), np.nan, **f32),
        info=torch.full((P,), -1, dtype=torch.int32, device=DEV), Gsum=torch.full((P, K), np.nan, **f32),
    )
    band_w = 0
    if g.band is not None:  # AFNI-faithful mode: R factored as a band
        band_w = int(g.band.max()) + 1
        keep["band"] = torch.from_numpy(g.band).to(DEV)
        out["band_L"] = torch.full((P, T, band_w), np.nan, dtype=torch.float64, device=DEV)
        out["band_coef"] = torch.full((P, T, band_w), np.nan, **f32)
    work = None
    if with_work:
        work = torch.empty(int(lib.ffs_grid_work_bytes(T, K, P)) // 8 + 1, dtype=torch.float64, device=DEV)
    p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    d = _lib.GridDesc(T=T, K=K, P=P, n_runs=lay.n_runs, run_start=p(keep["rs"]), tau=p(keep["tau"]), a=p(keep["a"]),
                      b=p(keep["b"]), X=p(keep["X"]), lambda_fp32=0, ld_u=ld, n_task=0, task_idx=None, n_glt=0,
                      glt=None, band_w=band_w, band=p(keep.get("band")))
    o = _lib.GridOut(coef=p(out["coef"]), logdet_R=p(out["logdet_R"]), logdet_XtX=p(out["logdet_XtX"]), U=p(out["U"]),
                     U_hi=p(out["U_hi"]), U_lo=p(out["U_lo"]), uexp=p(out["uexp"]), G=p(out["G"]),
                     Adiag=p(out["Adiag"]), XtX=p(out["XtX"]), info=p(out["info"]), Ftask=None, glt_var=None,
                     Gsum=p(out["Gsum"]), work=p(work), band_L=p(out.get("band_L")),
                     band_coef=p(out.get("band_coef")))
    status = getattr(lib, entry)(C.byref(d), C.byref(o), torch.cuda.current_stream().cuda_stream)
    _lib.check(status, entry)
    torch.cuda.synchronize()
    return {k: v.cpu() for k, v in out.items()}


def _compare(ref, got):
    for name in ref:
        r, g = ref[name], got[name]
        if r.dtype.is_floating_point:
            assert torch.isfinite(g).all(), name
            np.testing.assert_allclose(g.double().numpy(), r.double().numpy(), rtol=1e-9, atol=1e-9, err_msg=name)
        else:
            assert torch.equal(g, r), name


def test_noalloc_grid_build_matches_workspace_build_twice():
    cases = [
        (200, 8, None, torch.linspace(-0.8, 0.8, 9), torch.linspace(-0.8, 0.8, 9), 1),
        (120, 6, [0, 60], torch.linspace(0.0, 0.8, 9), torch.linspace(-0.8, 0.8, 17), 2),
    ]
    for T, K, rs, ag, bg, seed in cases:  # two calls in a row, different shapes
        g, lay, X = _inputs(T, K, rs, ag, bg, seed)
        ref = _build("ffs_grid_build", g, lay, X, with_work=True)
        got = _build("ffs_grid_build_noalloc", g, lay, X, with_work=False)
        _compare(ref, got)


def test_noalloc_grid_build_matches_workspace_build_with_the_banded_r():
    """AFNI-faithful mode: the banded R's factor (band_L, band_coef) from the
    allocation-free build equals the workspace build's."""
    from fastfuncstuff_gb300.glm import grid as G

    G.set_afni_mode(True)
    try:
        g, lay, X = _inputs(160, 8, [0, 80], torch.linspace(-0.8, 0.8, 17), torch.linspace(-0.8, 0.8, 17), 4)
        assert g.band is not None
        ref = _build("ffs_grid_build", g, lay, X, with_work=True)
        got = _build("ffs_grid_build_noalloc", g, lay, X, with_work=False)
    finally:
        G.set_afni_mode(False)
    assert "band_L" in ref
    _compare(ref, got)


def test_noalloc_grid_build_rejects_oversized_problems():
    from fastfuncstuff_gb300 import _lib

    g, lay, X = _inputs(400, 20, [0, 200], torch.linspace(-0.8, 0.8, 33), torch.linspace(-0.8, 0.8, 33), 3)
    need = _lib.load().ffs_grid_work_bytes(400, 20, g.P)
    assert need > 16 << 20
    with pytest.raises(MemoryError, match="static"):
        _build("ffs_grid_build_noalloc", g, lay, X, with_work=False)
