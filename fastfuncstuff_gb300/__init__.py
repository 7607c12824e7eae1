"""fastfuncstuff_gb300: the ARMA(1,1) REML voxelwise GLM of fastfuncstuff on one GB300.

The public API mirrors the reference's (``fit_glm_arma11``,
``fit_glm_arma11_grouped``, ``ARMA11Results``); the work runs in the sm_103a
kernels of ``libffs_reml.so`` through its C ABI (include/ffs_reml.h).
"""

from .glm.arma import (  # noqa: F401
    ARMA11Results,
    build_censor_run_info,
    compute_arma_lambda,
    ensure_zero_in_grid,
    estimate_valid_grid_pairs,
    fit_glm_arma11,
    fit_glm_arma11_grouped,
    fit_glm_arma11_perhrf,
    get_default_arma_grids,
    parse_grid_arg,
    precompute_reml_grid,
    search_voxels_precomputed_grid,
    set_afni_mode,
)
from .glm.rvar import compute_ljung_box_statistic, load_arma_params, save_arma_rvar, save_reml_lklhd  # noqa: F401
from .glm.engine import autotune_projection  # noqa: F401

from . import ops  # noqa: F401,E402  (registers the ffs_gb300:: torch custom operators)

__version__ = "1.0.0"
