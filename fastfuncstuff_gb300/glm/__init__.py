"""GLM engine: the ARMA(1,1) REML path (the reference's fastfuncstuff.glm.arma)."""

from .arma import *  # noqa: F401,F403
from .rvar import compute_ljung_box_statistic, load_arma_params, save_arma_rvar, save_reml_lklhd  # noqa: F401
