"""The torch custom operators (ffs_gb300::) of fastfuncstuff_gb300.ops."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import fastfuncstuff_gb300  # noqa: F401  (registers the ops)
from tests.conftest import load_golden


def test_ops_are_registered_with_fake_shapes():
    """Registered under torch.ops.ffs_gb300 and traceable with fake tensors (no GPU needed)."""
    from torch._subclasses.fake_tensor import FakeTensorMode

    for name in ("fit_arma11", "reml_search", "reml_gls"):
        assert hasattr(torch.ops.ffs_gb300, name)
    with FakeTensorMode():
        Y = torch.empty(64, 96)
        X = torch.empty(96, 5)
        g = torch.empty(9)
        out = torch.ops.ffs_gb300.fit_arma11(Y, X, g, g, [0], True)
        assert [tuple(t.shape) for t in out] == [(64, 5), (64, 5), (64,), (64,), (64,), (64, 2), (64,), (64,)]
        params, crit, scale = torch.ops.ffs_gb300.reml_search(Y, X, g, g, [0], False)
        assert tuple(params.shape) == (64, 2) and tuple(crit.shape) == (64,)
        gls = torch.ops.ffs_gb300.reml_gls(Y, X, params, g, g, [0])
        assert tuple(gls[0].shape) == (64, 5) and tuple(gls[5].shape) == (64,)


@pytest.mark.gpu
def test_ops_match_the_python_api():
    from fastfuncstuff_gb300 import fit_glm_arma11

    dev = torch.device("cuda:0")
    d = load_golden("single")
    Y = torch.from_numpy(d["Y"]).to(dev)
    X = torch.from_numpy(d["X"]).to(dev)
    ag = torch.as_tensor(d["a_grid"], dtype=torch.float32)
    bg = torch.as_tensor(d["b_grid"], dtype=torch.float32)
    ref = fit_glm_arma11(Y, X, 2.0, a_grid=ag, b_grid=bg, device=dev, verbose=False, force_exhaustive_search=True,
                         return_device=True)
    out = torch.ops.ffs_gb300.fit_arma11(Y, X, ag, bg, [0], False)
    for got, want in zip(out, (ref.betas, ref.tstats, ref.sigma2, ref.fstats, ref.r2, ref.arma_params,
                               ref.arma_lambda, ref.reml_likelihood)):
        assert torch.equal(got, want)
    # the two halves compose to the same fit
    params, crit, scale = torch.ops.ffs_gb300.reml_search(Y, X, ag, bg, [0], False)
    assert torch.equal(params, ref.arma_params)
    betas, tstats, sigma2, fstats, r2, lam = torch.ops.ffs_gb300.reml_gls(Y, X, params, ag, bg, [0])
    np.testing.assert_allclose(betas.cpu().numpy(), ref.betas.cpu().numpy(), rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(tstats.cpu().numpy(), ref.tstats.cpu().numpy(), rtol=1e-6, atol=1e-6)
    torch.testing.assert_close(lam, ref.arma_lambda)
