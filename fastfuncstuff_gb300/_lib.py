"""ctypes binding of libffs_reml.so (declared in include/ffs_reml.h).

The structures below mirror the header field for field. Every wrapper raises on
a non-zero status: ``ValueError`` for an invalid argument, ``MemoryError`` for a
workspace that is too small, ``RuntimeError`` otherwise -- the exception types
the reference raises for the same conditions. There is no fallback: if the
library cannot be loaded, importing the product path fails.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

_c_int_p = C.POINTER(C.c_int)
_c_float_p = C.POINTER(C.c_float)
_c_double_p = C.POINTER(C.c_double)
_c_u16_p = C.POINTER(C.c_uint16)

FFS_OK, FFS_ERR_INVALID, FFS_ERR_CUDA, FFS_ERR_UNSUPPORTED, FFS_ERR_WORKSPACE, FFS_ERR_TIMEOUT = range(6)
FFS_DSORT_QMAX = 16  # most voxelwise columns of ffs_reml_gls_dsort
FFS_BAND_MAX_W = 129  # widest row of the AFNI-faithful banded R (128 off-diagonals)


class GridDesc(C.Structure):
    _fields_ = [
        ("T", C.c_int), ("K", C.c_int), ("P", C.c_int), ("n_runs", C.c_int),
        ("run_start", C.c_void_p), ("tau", C.c_void_p), ("a", C.c_void_p), ("b", C.c_void_p),
        ("X", C.c_void_p), ("lambda_fp32", C.c_int), ("ld_u", C.c_int),
        ("n_task", C.c_int), ("task_idx", C.c_void_p), ("n_glt", C.c_int), ("glt", C.c_void_p),
        ("n_sets", C.c_int), ("set_ptr", C.c_void_p), ("set_idx", C.c_void_p),
        ("band_w", C.c_int), ("band", C.c_void_p),
    ]


class GridOut(C.Structure):
    _fields_ = [
        ("coef", C.c_void_p), ("logdet_R", C.c_void_p), ("logdet_XtX", C.c_void_p),
        ("U", C.c_void_p), ("U_hi", C.c_void_p), ("U_lo", C.c_void_p), ("uexp", C.c_void_p),
        ("G", C.c_void_p),
        ("Adiag", C.c_void_p), ("XtX", C.c_void_p), ("info", C.c_void_p), ("Ftask", C.c_void_p),
        ("glt_var", C.c_void_p), ("Gsum", C.c_void_p), ("work", C.c_void_p), ("Fsets", C.c_void_p),
        ("Afull", C.c_void_p), ("band_L", C.c_void_p), ("band_coef", C.c_void_p),
    ]


class DsortArgs(C.Structure):
    _fields_ = [
        ("V", C.c_int), ("T", C.c_int), ("K", C.c_int), ("q", C.c_int), ("dof", C.c_int),
        ("Y", C.c_void_p), ("scale", C.c_void_p), ("D", C.c_void_p), ("Xt", C.c_void_p), ("xmean", C.c_void_p),
        ("best", C.c_void_p), ("n_pairs", C.c_int),
        ("coef", C.c_void_p), ("G", C.c_void_p), ("U", C.c_void_p), ("Adiag", C.c_void_p), ("XtX", C.c_void_p),
        ("Afull", C.c_void_p),
        ("n_task", C.c_int), ("task_idx", C.c_void_p), ("Ftask", C.c_void_p),
        ("n_glt", C.c_int), ("glt", C.c_void_p), ("glt_var", C.c_void_p),
        ("n_sets", C.c_int), ("set_ptr", C.c_void_p), ("set_idx", C.c_void_p), ("set_col", C.c_void_p),
        ("n_set_out", C.c_int),
        ("lj_h", C.c_int), ("lj_tau", C.c_void_p), ("lj_w", C.c_void_p),
        ("betas", C.c_void_p), ("tstats", C.c_void_p), ("dbetas", C.c_void_p), ("dtstats", C.c_void_p),
        ("sigma2", C.c_void_p), ("fstats", C.c_void_p), ("r2", C.c_void_p),
        ("cbeta", C.c_void_p), ("ct", C.c_void_p),
        ("resid", C.c_void_p), ("resid_w", C.c_void_p), ("pred", C.c_void_p),
        ("ljung_box", C.c_void_p),
        ("set_fstats", C.c_void_p), ("set_sd", C.c_void_p), ("set_coef", C.c_void_p),
        ("status", C.c_void_p),
        ("band_coef", C.c_void_p), ("band_w", C.c_int), ("band", C.c_void_p),
    ]


class SetStatsArgs(C.Structure):
    _fields_ = [
        ("V", C.c_int), ("K", C.c_int), ("n_sets", C.c_int), ("n_out", C.c_int),
        ("set_ptr", C.c_void_p), ("set_idx", C.c_void_p), ("set_col", C.c_void_p), ("msum", C.c_int),
        ("Fsets", C.c_void_p), ("Csets", C.c_void_p), ("best", C.c_void_p), ("design", C.c_void_p),
        ("n_pairs", C.c_int), ("betas", C.c_void_p), ("sigma2", C.c_void_p), ("scale", C.c_void_p),
        ("set_fstats", C.c_void_p), ("set_sd", C.c_void_p), ("set_coef", C.c_void_p),
    ]


class PrepArgs(C.Structure):
    _fields_ = [
        ("V", C.c_int), ("T", C.c_int), ("K", C.c_int), ("Y", C.c_void_p), ("Q0", C.c_void_p),
        ("do_scale", C.c_int), ("center", C.c_int), ("ld_y", C.c_int), ("scale", C.c_void_p),
        ("yr_t", C.c_void_p),
        ("yr_hi", C.c_void_p), ("yr_lo", C.c_void_p), ("yexp", C.c_void_p),
        ("idx", C.c_void_p), ("feats", C.c_void_p), ("n_runs", C.c_int), ("run_start", C.c_void_p),
        ("yr_rows", C.c_void_p), ("center_dev", C.c_void_p), ("tile_design", C.c_void_p),
        ("Y_ref", C.c_void_p), ("Y_copy", C.c_void_p),
    ]


class ProjectArgs(C.Structure):
    _fields_ = [
        ("V", C.c_int), ("T", C.c_int), ("K", C.c_int), ("P", C.c_int), ("ld_y", C.c_int),
        ("ld_u", C.c_int), ("yr_hi", C.c_void_p), ("yr_lo", C.c_void_p), ("u_hi", C.c_void_p),
        ("u_lo", C.c_void_p), ("yexp", C.c_void_p), ("uexp", C.c_void_p),
        ("yr_t", C.c_void_p), ("U", C.c_void_p), ("proj", C.c_void_p),
        ("flag", C.c_void_p), ("V_dev", C.c_void_p),
    ]


class SurfaceArgs(C.Structure):
    _fields_ = [
        ("V", C.c_int), ("T", C.c_int), ("K", C.c_int), ("P", C.c_int), ("p0", C.c_int),
        ("yr_t", C.c_void_p), ("coef", C.c_void_p), ("logdet_R", C.c_void_p),
        ("logdet_XtX", C.c_void_p), ("proj", C.c_void_p), ("chunk_start", C.c_void_p),
        ("n_chunks", C.c_int), ("chunk_pairs", C.c_void_p), ("surf", C.c_void_p),
        ("crit0", C.c_void_p), ("tile_design", C.c_void_p),
        ("band_coef", C.c_void_p), ("band_w", C.c_int), ("band", C.c_void_p),
    ]


class SelectArgs(C.Structure):
    _fields_ = [
        ("V", C.c_int), ("P", C.c_int), ("surf", C.c_void_p), ("crit0", C.c_void_p),
        ("hierarchical", C.c_int), ("n_a", C.c_int), ("n_b", C.c_int), ("ltop", C.c_int),
        ("za", C.c_int), ("zb", C.c_int), ("lattice", C.c_void_p), ("best", C.c_void_p),
        ("best_crit", C.c_void_p),
    ]


class GlsArgs(C.Structure):
    _fields_ = [
        ("V", C.c_int), ("T", C.c_int), ("K", C.c_int), ("dof", C.c_int), ("center", C.c_int),
        ("Gsum", C.c_void_p), ("Y", C.c_void_p), ("scale", C.c_void_p), ("Xt", C.c_void_p),
        ("best", C.c_void_p),
        ("order", C.c_void_p), ("coef", C.c_void_p), ("G", C.c_void_p), ("Adiag", C.c_void_p),
        ("XtX", C.c_void_p), ("a", C.c_void_p), ("b", C.c_void_p), ("lambda_fp32", C.c_int),
        ("n_task", C.c_int), ("task_idx", C.c_void_p), ("Ftask", C.c_void_p),
        ("n_glt", C.c_int), ("glt", C.c_void_p), ("glt_var", C.c_void_p),
        ("betas", C.c_void_p), ("tstats", C.c_void_p), ("sigma2", C.c_void_p),
        ("fstats", C.c_void_p), ("r2", C.c_void_p), ("lam", C.c_void_p),
        ("cbeta", C.c_void_p), ("ct", C.c_void_p), ("resid", C.c_void_p),
        ("resid_w", C.c_void_p), ("pred", C.c_void_p), ("center_dev", C.c_void_p), ("n_pairs", C.c_int),
        ("band_coef", C.c_void_p), ("band_w", C.c_int), ("band", C.c_void_p),
    ]


class MergeField(C.Structure):
    _fields_ = [("dst", C.c_void_p), ("src", C.c_void_p), ("src_sub", C.c_void_p), ("row_bytes", C.c_int)]


# (symbol, argtypes, restype) of every entry point in include/ffs_reml.h
SIGNATURES = {
    "ffs_version": ([], C.c_int),
    "ffs_status_string": ([C.c_int], C.c_char_p),
    "ffs_last_error": ([], C.c_char_p),
    "ffs_grid_work_bytes": ([C.c_int, C.c_int, C.c_int], C.c_size_t),
    "ffs_grid_build": ([C.POINTER(GridDesc), C.POINTER(GridOut), C.c_void_p], C.c_int),
    "ffs_grid_work_bytes_designs": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int], C.c_size_t),
    "ffs_grid_build_designs": ([C.POINTER(GridDesc), C.c_int, C.c_int, C.POINTER(GridOut), C.c_void_p], C.c_int),
    "ffs_grid_build_noalloc": ([C.POINTER(GridDesc), C.POINTER(GridOut), C.c_void_p], C.c_int),
    "ffs_reml_prep": ([C.POINTER(PrepArgs), C.c_void_p], C.c_int),
    "ffs_reml_project_tc": ([C.POINTER(ProjectArgs), C.c_void_p], C.c_int),
    "ffs_reml_project_simt": ([C.POINTER(ProjectArgs), C.c_void_p], C.c_int),
    "ffs_reml_surface": ([C.POINTER(SurfaceArgs), C.c_void_p], C.c_int),
    "ffs_reml_select": ([C.POINTER(SelectArgs), C.c_void_p], C.c_int),
    "ffs_reml_gls": ([C.POINTER(GlsArgs), C.c_void_p], C.c_int),
    "ffs_reml_set_stats": ([C.POINTER(SetStatsArgs), C.c_void_p], C.c_int),
    "ffs_reml_gls_dsort": ([C.POINTER(DsortArgs), C.c_void_p], C.c_int),
    "ffs_reml_tune_tc_pairs": ([C.c_int, C.c_int], C.c_int),
    "ffs_reml_gls_ex": ([C.POINTER(GlsArgs), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p], C.c_int),
    "ffs_reml_gls_grouped": ([C.POINTER(GlsArgs), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                              C.c_void_p, C.c_void_p], C.c_int),
    "ffs_reml_group": ([C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_mlp_param_count": ([], C.c_int),
    "ffs_arma_simulate": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                           C.c_uint64, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_mlp_forward": ([C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_mlp_grad": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                      C.c_void_p], C.c_int),
    "ffs_mlp_adam": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_float,
                      C.c_float, C.c_int, C.c_void_p], C.c_int),
    "ffs_reml_centers": ([C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p],
                         C.c_int),
    "ffs_design_basis_work_bytes": ([C.c_int, C.c_int], C.c_size_t),
    "ffs_design_basis": ([C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                          C.c_void_p], C.c_int),
    "ffs_reml_gather": ([C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_reml_window_items": ([C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                               C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                               C.c_void_p], C.c_int),
    "ffs_reml_window": ([C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_device_view": ([C.c_void_p, C.POINTER(C.c_void_p)], C.c_int),
    "ffs_reml_strip": ([C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                        C.c_void_p, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_reml_band_sums": ([C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                            C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                            C.c_void_p, C.c_int, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_reml_segment_items": ([C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                C.c_void_p, C.c_void_p], C.c_int),
    "ffs_reml_near_line": ([C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                            C.c_void_p], C.c_int),
    "ffs_reml_window_finish": ([C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                C.POINTER(C.c_void_p), C.c_void_p], C.c_int),
    "ffs_reml_compact": ([C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "ffs_merge_rows": ([C.c_int, C.c_void_p, C.c_int, C.POINTER(MergeField), C.c_void_p], C.c_int),
    "ffs_reml_project_tc_list": ([C.POINTER(ProjectArgs), C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                  C.c_void_p], C.c_int),
}

_LIB: C.CDLL | None = None


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libffs_reml.so (building it first when it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build_if_missing and _build._stale():
        _build.build()
    if not path.exists():
        raise RuntimeError(f"{path} is missing: run fastfuncstuff_gb300.build.build()")
    lib = C.CDLL(str(path))
    for name, (argtypes, restype) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = restype
    _LIB = lib
    return lib


def check(status: int, what: str) -> None:
    if status == FFS_OK:
        return
    lib = load()
    msg = lib.ffs_last_error().decode() or lib.ffs_status_string(status).decode()
    if status == FFS_ERR_INVALID:
        raise ValueError(f"{what}: {msg}")
    if status == FFS_ERR_WORKSPACE:
        raise MemoryError(f"{what}: {msg}")
    raise RuntimeError(f"{what}: {msg} (status {status})")


def call(name: str, *args) -> None:
    lib = load()
    check(getattr(lib, name)(*args), name)
