"""The -Rvar dataset writer/reader (host side; fastfuncstuff/glm/arma.py:6181-6459).

The file is checked field by field against the NIfTI-1 header layout, and the
Ljung-Box fallback against the reference's own values (golden ``ljung``
fixture) and the oracle.
"""

from __future__ import annotations

import gzip
import struct

import numpy as np
import pytest
import torch

from fastfuncstuff_gb300 import ARMA11Results, compute_ljung_box_statistic, load_arma_params, save_arma_rvar
from fastfuncstuff_gb300.glm.grid import build_ljung_box_tau
from oracle import reml as o
from tests.conftest import load_golden


def _results(V, rng, with_lb=True):
    r = ARMA11Results()
    ab = np.stack([rng.uniform(-0.8, 0.8, V), rng.uniform(-0.8, 0.8, V)], 1).astype(np.float32)
    r.arma_params = torch.from_numpy(ab)
    r.arma_lambda = torch.from_numpy(o.arma_lambda_output_f32(ab[:, 0], ab[:, 1]).astype(np.float32))
    r.sigma2 = torch.from_numpy(rng.uniform(0.5, 4.0, V).astype(np.float32))
    r.reml_likelihood = torch.from_numpy(rng.normal(300.0, 20.0, V).astype(np.float32))
    if with_lb:
        r.ljung_box = torch.from_numpy(rng.uniform(0.0, 40.0, V).astype(np.float32))
        r.ljung_box_dof = 17
    return r


def _header(raw):
    return dict(
        sizeof_hdr=struct.unpack_from("<i", raw, 0)[0], dim=struct.unpack_from("<8h", raw, 40),
        datatype=struct.unpack_from("<2h", raw, 70), pixdim=struct.unpack_from("<8f", raw, 76),
        vox_offset=struct.unpack_from("<f", raw, 108)[0], scl=struct.unpack_from("<2f", raw, 112),
        codes=struct.unpack_from("<2h", raw, 252), quat=struct.unpack_from("<6f", raw, 256),
        srow=np.array(struct.unpack_from("<12f", raw, 280)).reshape(3, 4), magic=raw[344:348],
        ext_flag=raw[348], ext=struct.unpack_from("<2i", raw, 352))


@pytest.mark.parametrize("suffix", [".nii", ".nii.gz"])
def test_rvar_layout_and_round_trip(tmp_path, suffix):
    rng = np.random.default_rng(3)
    shape = (5, 4, 3)
    mask = rng.random(shape) < 0.6
    V = int(mask.sum())
    res = _results(V, rng)
    aff = np.array([[-2.0, 0.0, 0.0, 90.0], [0.0, 2.0, 0.0, -126.0], [0.0, 0.0, 2.5, -72.0], [0, 0, 0, 1]])
    path = save_arma_rvar(res, tmp_path / f"rvar{suffix}", volume_shape=shape, voxel_mask=mask, affine=aff)
    raw = path.read_bytes()
    if suffix.endswith(".gz"):
        raw = gzip.decompress(raw)
    h = _header(raw)
    assert h["sizeof_hdr"] == 348 and h["magic"] == b"n+1\x00"
    assert h["dim"][:5] == (4, 5, 4, 3, 6)
    assert h["datatype"] == (16, 32)  # float32, 32 bits
    assert h["codes"] == (1, 1)        # qform, sform: scanner-anatomical
    np.testing.assert_allclose(h["srow"], aff[:3], rtol=1e-6)
    np.testing.assert_allclose(h["pixdim"][:4], [-1.0, 2.0, 2.0, 2.5], rtol=1e-6)  # qfac -1: left-handed
    np.testing.assert_allclose(h["quat"][3:], aff[:3, 3], rtol=1e-6)
    assert h["ext_flag"] == 1 and h["ext"][1] == 4 and h["ext"][0] % 16 == 0
    assert h["vox_offset"] == 352 + h["ext"][0]
    xml = raw[360:352 + h["ext"][0]].decode("utf-8")
    assert '"a~b~lam~StDev~-LogLik~LjungBox"' in xml
    assert 'atr_name="BRICK_STATAUX"' in xml and " 5\n 6\n 1\n 17\n" in xml
    assert '"none;none;none;none;none;Chisq(17)"' in xml
    # the voxels, x fastest, then the six volumes
    vol = np.frombuffer(raw, np.float32, count=5 * 4 * 3 * 6, offset=int(h["vox_offset"])).reshape(
        (5, 4, 3, 6), order="F")
    np.testing.assert_array_equal(vol[..., 0][mask], res.arma_params[:, 0].numpy())
    np.testing.assert_array_equal(vol[..., 2][mask], res.arma_lambda.numpy())
    np.testing.assert_allclose(vol[..., 3][mask], np.sqrt(res.sigma2.numpy()), rtol=1e-7)
    np.testing.assert_array_equal(vol[..., 4][mask], res.reml_likelihood.numpy())
    np.testing.assert_array_equal(vol[..., 5][mask], res.ljung_box.numpy())
    assert not vol[~mask].any()
    # volumes 0 and 1 back as precomputed_arma_params
    np.testing.assert_array_equal(load_arma_params(path, mask), res.arma_params.numpy())
    full = load_arma_params(path)
    assert full.shape == (60, 2)
    np.testing.assert_array_equal(full[mask.reshape(-1, order="C")], res.arma_params.numpy())


def test_rvar_qform_reproduces_the_rotation(tmp_path):
    """The NIfTI-1 quaternion (b, c, d, qfac) rebuilds the affine's rotation."""
    rng = np.random.default_rng(4)
    q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
    aff = np.eye(4)
    aff[:3, :3] = q * np.array([1.5, 2.0, 3.0])
    aff[:3, 3] = [10.0, -20.0, 30.0]
    path = save_arma_rvar(_results(6, rng), tmp_path / "rot.nii", affine=aff)
    h = _header(path.read_bytes())
    b, c, d = h["quat"][:3]
    a = np.sqrt(max(0.0, 1.0 - (b * b + c * c + d * d)))
    R = np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                  [2 * (b * c + a * d), a * a + c * c - b * b - d * d, 2 * (c * d - a * b)],
                  [2 * (b * d - a * c), 2 * (c * d + a * b), a * a + d * d - c * c - b * b]])
    qfac, pix = h["pixdim"][0], np.array(h["pixdim"][1:4])
    M = R * pix
    M[:, 2] *= qfac
    np.testing.assert_allclose(M, aff[:3, :3], atol=1e-5)
    assert h["dim"][:5] == (4, 6, 1, 1, 6)  # no volume shape: (V, 1, 1) columns


def test_rvar_ljung_box_from_whitened_residuals(tmp_path):
    """Without results.ljung_box the writer computes it from the whitened
    residuals (the reference's fallback), else writes zeros with a warning."""
    rng = np.random.default_rng(5)
    res = _results(7, rng, with_lb=False)
    res.residuals_whitened = torch.from_numpy(rng.standard_normal((7, 120)).astype(np.float32))
    path = save_arma_rvar(res, tmp_path / "lb.nii", max_lag=12)
    vol = np.frombuffer(path.read_bytes(), np.float32, offset=int(_header(path.read_bytes())["vox_offset"]))
    lb = vol.reshape((7, 1, 1, 6), order="F")[:, 0, 0, 5]
    np.testing.assert_allclose(lb, o.ljung_box(res.residuals_whitened.numpy(), 12), rtol=1e-5)
    res.residuals_whitened = None
    with pytest.warns(UserWarning, match="LjungBox"):
        save_arma_rvar(res, tmp_path / "zeros.nii")


def test_ljung_box_statistic_matches_reference_values():
    """The host Ljung-Box equals the reference's own values on its test series
    (plain lags, a censored series and two runs with a pseudo-time)."""
    d = load_golden("ljung")
    cases = [("white_h20", d["white"], 20, None), ("white_auto", d["white"], None, None),
             ("ar1_h20", d["ar1"], 20, None), ("offset_h20", d["offset"], 20, None),
             ("censored_h18", d["censored"], 18, d["censored_keep"]),
             ("tworun_h20", d["tworun"], 20, d["tworun_tau"]), ("tworun_notau_h20", d["tworun"], 20, None)]
    for key, series, lag, tau in cases:
        got = compute_ljung_box_statistic(np.asarray(series, np.float64)[None], lag, tau)[0]
        np.testing.assert_allclose(got, float(d[f"ref_{key}"]), rtol=1e-6, err_msg=key)
    # a multi-run pseudo-time from the fit's run layout agrees with the oracle
    r = np.random.default_rng(6).standard_normal((5, 90))
    tau = build_ljung_box_tau(90, [0, 40])
    np.testing.assert_allclose(compute_ljung_box_statistic(r, 10, tau), o.ljung_box(r, 10, tau), rtol=1e-6)


def test_load_arma_params_errors(tmp_path):
    with pytest.raises(FileNotFoundError):
        load_arma_params(tmp_path / "missing.nii")
    bad = tmp_path / "bad.nii"
    bad.write_bytes(b"\x00" * 400)
    with pytest.raises(ValueError):
        load_arma_params(bad)


def test_reml_lklhd_surface_file(tmp_path):
    """-Rlklhd: one float32 volume per valid pair, labelled a=X.XX_b=Y.YY in pair
    order (fastfuncstuff/cli/reml.py:5102-5163); the suffix defaults to .nii.gz."""
    from fastfuncstuff_gb300.glm import grid as G
    from fastfuncstuff_gb300.glm.arma import ARMA11Results
    from fastfuncstuff_gb300.glm.rvar import _read_nifti1, save_reml_lklhd

    rng = np.random.default_rng(8)
    grid = G.make_grid(np.linspace(-0.8, 0.8, 5).astype(np.float32), np.linspace(-0.8, 0.8, 5).astype(np.float32))
    shape = (3, 4, 2)
    mask = rng.random(shape) < 0.7
    V = int(mask.sum())
    res = ARMA11Results()
    res.reml_lklhd_surface = torch.from_numpy(rng.standard_normal((V, grid.P)).astype(np.float32))
    res.reml_surface_params = grid.param_list()
    path = save_reml_lklhd(res, tmp_path / "lk", volume_shape=shape, voxel_mask=mask)
    assert path.name == "lk.nii.gz"
    raw = gzip.decompress(path.read_bytes())
    h = _header(raw)
    assert h["dim"][:5] == (4, 3, 4, 2, grid.P) and h["datatype"] == (16, 32)
    xml = raw[360:352 + h["ext"][0]].decode("utf-8")
    labels = "~".join(f"a={a:.2f}_b={b:.2f}" for a, b in grid.param_list())
    assert f'"{labels}"' in xml and "BRICK_STATAUX" not in xml
    vol = _read_nifti1(path)
    np.testing.assert_array_equal(vol[mask], res.reml_lklhd_surface.numpy())
    assert not vol[~mask].any()
    # without a volume shape: (V, 1, 1, P); a fit without the surface is an error
    flat = _read_nifti1(save_reml_lklhd(res, tmp_path / "flat.nii"))
    np.testing.assert_array_equal(flat.reshape(V, grid.P), res.reml_lklhd_surface.numpy())
    with pytest.raises(ValueError):
        save_reml_lklhd(ARMA11Results(), tmp_path / "none.nii")
