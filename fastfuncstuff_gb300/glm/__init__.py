"""GLM engine: the ARMA(1,1) REML path (the reference's fastfuncstuff.glm.arma)."""

from .arma import *  # noqa: F401,F403
