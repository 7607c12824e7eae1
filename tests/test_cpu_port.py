"""The timed CPU baseline (oracle/cpu_port.py) pinned to the reference's own
float32 outputs on the golden fixtures (tests/golden/make_golden.py), in the
default (hierarchical) and exhaustive selector modes."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import cpu_port
from tests.conftest import load_golden


@pytest.mark.parametrize("case", ["single", "baseline", "multirun"])
@pytest.mark.parametrize("mode", ["def", "exh"])
def test_cpu_port_matches_reference_float32(case, mode):
    d = load_golden(case)
    ti = list(d["task_indices"]) if "task_indices" in d else None
    got = cpu_port.fit(d["Y"], d["X"], d["a_grid"], d["b_grid"], run_starts=d.get("run_starts"),
                       exhaustive=mode == "exh", task_indices=ti)
    ref = {k.split("__")[1]: v for k, v in d.items() if k.startswith(f"f32_{mode}__")}
    # the same float32 arithmetic as the reference, in another operation order:
    # the selected pair agrees on all but near-tie voxels
    same = (got["arma_params"] == ref["arma_params"]).all(1)
    assert same.mean() >= 0.99, same.mean()
    lik = ref["reml_likelihood"]
    gap = np.abs(got["reml_likelihood"] - lik) / np.maximum(np.abs(lik), 1.0)
    assert gap.max() <= 2e-6, gap.max()
    sel = ti if ti is not None else slice(None)
    s = same

    def rel(x, y):
        return np.abs(x - y).max(-1) / np.maximum(np.abs(y).max(-1), 1e-12)

    assert rel(got["betas"][s][:, sel], ref["betas"][s]).max() <= 1e-5
    assert rel(got["tstats"][s][:, sel], ref["tstats"][s]).max() <= 1e-5
    np.testing.assert_allclose(got["sigma2"][s], ref["sigma2"][s], rtol=5e-5)
    np.testing.assert_allclose(got["fstats"][s], ref["fstats"][s], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(got["r2"][s], ref["r2"][s], atol=1e-5)
    np.testing.assert_allclose(got["arma_lambda"][s], ref["arma_lambda"][s], rtol=1e-6, atol=1e-7)
