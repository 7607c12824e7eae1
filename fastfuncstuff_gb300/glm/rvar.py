"""The -Rvar and -Rlklhd files of an ARMA(1,1) fit and the -Rvar reuse
(fastfuncstuff/glm/arma.py:6181-6459, fastfuncstuff/cli/reml.py:5102-5163).

``save_arma_rvar`` writes AFNI 3dREMLfit's 6-volume variance-parameter dataset
(a, b, lam, StDev, -LogLik, LjungBox) as a float32 NIfTI-1 file, ``.nii`` or
``.nii.gz``; ``load_arma_params`` reads volumes 0 and 1 back as the
``precomputed_arma_params`` of a later fit. ``save_reml_lklhd`` writes the
REML criterion at every valid (a, b) pair (``save_profile_likelihoods``), one
volume per pair labelled ``a=X.XX_b=Y.YY``. The NIfTI-1 header is packed here
from the format's published field layout (no NIfTI library is needed), with
the sform and qform both set from the affine (code 1, scanner-anatomical, as
the reference writes a map that names no template) and AFNI's header
extension (code 4) carrying the sub-brick labels and the chi-squared tag
(BRICK_STATAUX / BRICK_STATSYM) of the Ljung-Box volume, so AFNI viewers label
and threshold the volumes as they do the reference's file.
"""

from __future__ import annotations

import gzip
import math
import secrets
import struct
import warnings
from pathlib import Path

import numpy as np
import torch

from .grid import resolve_ljung_box_lag

__all__ = ["save_arma_rvar", "save_reml_lklhd", "load_arma_params", "compute_ljung_box_statistic",
           "RVAR_LABELS"]

RVAR_LABELS = ["a", "b", "lam", "StDev", "-LogLik", "LjungBox"]

_HDR_SIZE = 348
_NIFTI_FLOAT32 = 16
_XFORM_SCANNER_ANAT = 1
_ECODE_AFNI = 4
_AFNI_CHISQ = 6  # AFNI's FUNC_CT_TYPE: chi-squared, one parameter (dof)


def _np(x):
    if x is None:
        return None
    if isinstance(x, torch.Tensor):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def compute_ljung_box_statistic(residuals, max_lag: int | None = None, tau=None) -> np.ndarray:
    """Ljung-Box statistic of each row of prewhitened residuals (V, T), float32:
    AFNI's ljung_box_uneven (fastfuncstuff/glm/arma.py:6058-6178). Lag-k
    products are binned by their time lag 0 < dj <= h when ``tau`` (the
    pseudo-time of build_ljung_box_tau) is given, bins need n_k > 1,
    LB = n (n + 2) sum_k c_k^2 / n_k clamped at 1e10; 0 when n < 10 or
    sum r^2 < 1e-10. The GLS computes the same statistic on the GPU
    (want_ljung_box=True); this host form serves the -Rvar writer when a caller
    kept only the whitened residuals."""
    r = torch.as_tensor(_np(residuals), dtype=torch.float64)
    if r.ndim == 1:
        r = r[None]
    V, n = r.shape
    out = torch.zeros(V, dtype=torch.float64)
    if n < 10:
        return out.numpy().astype(np.float32)
    h = resolve_ljung_box_lag(n, max_lag)
    s0 = (r * r).sum(1)
    ok = s0 >= 1e-10
    s0 = torch.where(ok, s0, torch.ones_like(s0))
    sums = torch.zeros(V, h + 1, dtype=torch.float64)
    cnt = np.zeros(h + 1, dtype=np.int64)
    t = None if tau is None else np.asarray(_np(tau), dtype=np.int64).reshape(-1)
    for k in range(1, h + 1):
        prod = r[:, : n - k] * r[:, k:]
        if t is None:
            cnt[k] = n - k
            sums[:, k] = prod.sum(1)
        else:
            dj = t[k:] - t[: n - k]
            keep = np.nonzero((dj > 0) & (dj <= h))[0]
            if keep.size:
                np.add.at(cnt, dj[keep], 1)
                sums.index_add_(1, torch.from_numpy(dj[keep]), prod[:, torch.from_numpy(keep)])
    good = cnt > 1
    good[0] = False
    if good.any():
        gi = torch.from_numpy(np.nonzero(good)[0])
        ck = sums[:, gi] / s0[:, None]
        g = (ck * ck / torch.from_numpy(cnt[good].astype(np.float64))).sum(1) * (n * (n + 2.0))
        out = torch.where(ok, torch.clamp(g, max=1.0e10), torch.zeros_like(g))
    return out.numpy().astype(np.float32)


def _quatern(affine: np.ndarray):
    """qform parameters (b, c, d, qfac, pixdim) of a 4x4 affine: the rotation of
    its normalised 3x3 part as a unit quaternion with a >= 0 (a sign flip of
    the third column, qfac = -1, makes an improper rotation proper), as the
    NIfTI-1 format defines them."""
    M = np.asarray(affine, dtype=np.float64)[:3, :3]
    pix = np.sqrt((M * M).sum(0))
    pix[pix == 0] = 1.0
    R = M / pix
    qfac = 1.0
    if np.linalg.det(R) < 0:
        R[:, 2] = -R[:, 2]
        qfac = -1.0
    # nearest proper rotation (polar factor), then the quaternion of it
    u, _, vt = np.linalg.svd(R)
    R = u @ vt
    tr = R[0, 0] + R[1, 1] + R[2, 2]
    if tr > 0:
        s = math.sqrt(tr + 1.0) * 2
        a, b, c, d = 0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s
    elif R[0, 0] > R[1, 1] and R[0, 0] > R[2, 2]:
        s = math.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2]) * 2
        a, b, c, d = (R[2, 1] - R[1, 2]) / s, 0.25 * s, (R[0, 1] + R[1, 0]) / s, (R[0, 2] + R[2, 0]) / s
    elif R[1, 1] > R[2, 2]:
        s = math.sqrt(1.0 + R[1, 1] - R[0, 0] - R[2, 2]) * 2
        a, b, c, d = (R[0, 2] - R[2, 0]) / s, (R[0, 1] + R[1, 0]) / s, 0.25 * s, (R[1, 2] + R[2, 1]) / s
    else:
        s = math.sqrt(1.0 + R[2, 2] - R[0, 0] - R[1, 1]) * 2
        a, b, c, d = (R[1, 0] - R[0, 1]) / s, (R[0, 2] + R[2, 0]) / s, (R[1, 2] + R[2, 1]) / s, 0.25 * s
    if a < 0:
        b, c, d = -b, -c, -d
    return (b, c, d), qfac, pix


def _afni_extension(labels, stataux, n_sub: int) -> bytes:
    """AFNI's NIfTI header extension: an XML group of attributes (the layout AFNI
    itself writes and reads): a fresh IDCODE, BRICK_LABS ("~"-separated) and,
    for tagged sub-bricks, BRICK_STATAUX (index, code, n params, params...) and
    BRICK_STATSYM ("Chisq(dof)" or "none" per sub-brick)."""
    idc = "FFS_" + secrets.token_hex(11)[:22]
    atr = ("<AFNI_atr\n  ni_type=\"String\"\n  ni_dimen=\"1\"\n  atr_name=\"BRICK_LABS\" >\n"
           f" \"{'~'.join(labels)}\"\n</AFNI_atr>\n")
    if stataux:
        vals: list[float] = []
        syms = []
        for i in range(n_sub):
            if i in stataux:
                code, params = stataux[i]
                vals += [float(i), float(code), float(len(params))] + [float(p) for p in params]
                syms.append(f"Chisq({int(params[0])})" if code == _AFNI_CHISQ and len(params) == 1 else "none")
            else:
                syms.append("none")
        body = " " + "\n ".join(f"{v:g}" for v in vals)
        atr += ("<AFNI_atr\n  ni_type=\"float\"\n"
                f"  ni_dimen=\"{len(vals)}\"\n  atr_name=\"BRICK_STATAUX\" >\n{body}\n</AFNI_atr>\n"
                "<AFNI_atr\n  ni_type=\"String\"\n  ni_dimen=\"1\"\n  atr_name=\"BRICK_STATSYM\" >\n"
                f" \"{';'.join(syms)}\"\n</AFNI_atr>\n")
    xml = ("<?xml version='1.0' ?>\n<AFNI_attributes\n"
           f"  self_idcode=\"{idc}\"\n  ni_form=\"ni_group\" >\n{atr}</AFNI_attributes>\n\x00")
    return xml.encode("utf-8")


def _nifti1_bytes(data: np.ndarray, affine: np.ndarray, extensions: list[tuple[int, bytes]]) -> bytes:
    """A single-file NIfTI-1 image (header, extensions, then the voxels with x
    fastest) of float32 ``data`` (nx, ny, nz, nt)."""
    data = np.asarray(data, dtype=np.float32)
    shape = data.shape
    ext = b""
    for code, content in extensions:
        size = 8 + len(content)
        size += (-size) % 16  # each extension is a multiple of 16 bytes
        ext += struct.pack("<ii", size, code) + content + b"\x00" * (size - 8 - len(content))
    vox_offset = _HDR_SIZE + 4 + len(ext)
    (qb, qc, qd), qfac, pix = _quatern(affine)
    A = np.asarray(affine, dtype=np.float64)
    dim = [len(shape)] + list(shape) + [1] * (7 - len(shape))
    pixdim = [qfac] + list(pix) + [1.0] * (7 - 3)
    h = bytearray(_HDR_SIZE)
    struct.pack_into("<i", h, 0, _HDR_SIZE)
    h[38] = ord("r")                                           # regular
    struct.pack_into("<8h", h, 40, *dim)                       # dim
    struct.pack_into("<2h", h, 70, _NIFTI_FLOAT32, 32)         # datatype, bitpix
    struct.pack_into("<8f", h, 76, *pixdim)                    # pixdim
    struct.pack_into("<f", h, 108, float(vox_offset))          # vox_offset
    struct.pack_into("<2f", h, 112, 1.0, 0.0)                  # scl_slope, scl_inter
    struct.pack_into("<2h", h, 252, _XFORM_SCANNER_ANAT, _XFORM_SCANNER_ANAT)  # qform_code, sform_code
    struct.pack_into("<6f", h, 256, qb, qc, qd, A[0, 3], A[1, 3], A[2, 3])  # quatern_b..d, qoffset_x..z
    struct.pack_into("<12f", h, 280, *A[:3, :].reshape(-1))     # srow_x, srow_y, srow_z
    h[344:348] = b"n+1\x00"                                     # magic
    flag = struct.pack("<4b", 1 if extensions else 0, 0, 0, 0)
    return bytes(h) + flag + ext + np.asfortranarray(data).tobytes(order="F")


def save_arma_rvar(results, output_path, volume_shape=None, voxel_mask=None, affine=None, max_lag=None,
                   tau=None) -> Path:
    """Write the fit's -Rvar dataset (fastfuncstuff/glm/arma.py:6181-6369).

    Volumes: 0 a, 1 b, 2 lam, 3 StDev (sqrt(sigma2)), 4 -LogLik (the REML
    criterion), 5 LjungBox (chi-squared with ljung_box_dof degrees of freedom,
    tagged for AFNI). LjungBox comes from ``results.ljung_box``, else from
    ``results.residuals_whitened`` (``max_lag``, ``tau``), else zeros with a
    warning. With ``volume_shape`` the maps are volumes of that shape
    (``voxel_mask`` placing the fitted voxels, zero elsewhere), otherwise
    (V, 1, 1) columns. ``.gz`` output paths are gzip-compressed.
    """
    output_path = Path(output_path)
    output_path.parent.mkdir(parents=True, exist_ok=True)
    ab = _np(results.arma_params)
    lam = _np(results.arma_lambda)
    sigma = np.sqrt(_np(results.sigma2))
    nll = _np(results.reml_likelihood)
    assert lam is not None, "arma_lambda should not be None"
    assert nll is not None, "reml_likelihood should not be None"
    if results.ljung_box is not None:
        lb = _np(results.ljung_box).astype(np.float32)
    elif results.residuals_whitened is not None:
        lb = compute_ljung_box_statistic(results.residuals_whitened, max_lag=max_lag, tau=tau)
    else:
        warnings.warn("Rvar sub-brick 5 (LjungBox) written as zeros: no whiteness statistic was computed. "
                      "Pass want_ljung_box=True to fit_glm_arma11() to populate it.", stacklevel=2)
        lb = np.zeros(len(ab), dtype=np.float32)
    maps = [ab[:, 0], ab[:, 1], lam, sigma, nll, lb]
    if volume_shape is not None:
        volume_shape = tuple(int(s) for s in volume_shape)
        if voxel_mask is not None:
            mask = _np(voxel_mask).reshape(-1).astype(bool)
            vols = []
            for m in maps:
                full = np.zeros(int(np.prod(volume_shape)), dtype=np.float32)
                full[mask] = m
                vols.append(full.reshape(volume_shape))
        else:
            vols = [np.asarray(m, dtype=np.float32).reshape(volume_shape) for m in maps]
    else:
        vols = [np.asarray(m, dtype=np.float32).reshape(-1, 1, 1) for m in maps]
    rvar = np.stack(vols, axis=-1).astype(np.float32)
    if affine is None and getattr(results, "affine", None) is not None:
        affine = results.affine
    if affine is None:
        affine = np.eye(4)
    stataux = {5: (_AFNI_CHISQ, (float(results.ljung_box_dof),))} if results.ljung_box_dof else None
    blob = _nifti1_bytes(rvar, np.asarray(affine, np.float64),
                         [(_ECODE_AFNI, _afni_extension(RVAR_LABELS, stataux, rvar.shape[-1]))])
    if str(output_path).endswith(".gz"):
        with gzip.open(output_path, "wb", compresslevel=6) as f:
            f.write(blob)
    else:
        output_path.write_bytes(blob)
    return output_path


def save_reml_lklhd(results, output_path, volume_shape=None, voxel_mask=None, affine=None) -> Path:
    """Write the fit's -Rlklhd dataset: the REML criterion of every voxel at
    every valid (a, b) pair, one float32 volume per pair in the fit's pair
    order, labelled ``a=X.XX_b=Y.YY`` (fastfuncstuff/cli/reml.py:5102-5163).

    Needs a fit with ``save_profile_likelihoods=True`` (ValueError
    otherwise). With ``volume_shape`` the volumes have that shape
    (``voxel_mask`` placing the fitted voxels, zero elsewhere), otherwise
    (V, 1, 1). A path without a NIfTI suffix gets ``.nii.gz``, as the
    reference names it; ``.gz`` paths are gzip-compressed."""
    surf = _np(getattr(results, "reml_lklhd_surface", None))
    params = getattr(results, "reml_surface_params", None)
    if surf is None or params is None:
        raise ValueError("save_reml_lklhd needs a fit with save_profile_likelihoods=True "
                         "(no likelihood surface on these results)")
    surf = np.asarray(surf, np.float32)
    V, n_pairs = surf.shape
    name = str(output_path)
    if name.endswith(".nii.zst"):
        raise ValueError(f"{name}: zstd-compressed NIfTI is not written by this build; use .nii or .nii.gz")
    if not name.endswith((".nii", ".nii.gz")):
        name += ".nii.gz"
    output_path = Path(name)
    output_path.parent.mkdir(parents=True, exist_ok=True)
    if volume_shape is not None:
        volume_shape = tuple(int(x) for x in volume_shape)
        if voxel_mask is not None:
            mask = _np(voxel_mask).reshape(-1).astype(bool)
            vol = np.zeros((int(np.prod(volume_shape)), n_pairs), np.float32)
            vol[mask] = surf
            vol = vol.reshape(*volume_shape, n_pairs)
        else:
            vol = surf.reshape(*volume_shape, n_pairs)
    else:
        vol = surf.reshape(V, 1, 1, n_pairs)
    if affine is None and getattr(results, "affine", None) is not None:
        affine = results.affine
    if affine is None:
        affine = np.eye(4)
    labels = [f"a={float(a_k):.2f}_b={float(b_k):.2f}" for (a_k, b_k) in params]
    blob = _nifti1_bytes(vol, np.asarray(affine, np.float64),
                         [(_ECODE_AFNI, _afni_extension(labels, None, n_pairs))])
    if name.endswith(".gz"):
        with gzip.open(output_path, "wb", compresslevel=6) as f:
            f.write(blob)
    else:
        output_path.write_bytes(blob)
    return output_path


_NIFTI_DTYPES = {2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64, 256: np.int8,
                 512: np.uint16, 768: np.uint32}


def _read_nifti1(path: Path):
    raw = path.read_bytes()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    if len(raw) < _HDR_SIZE:
        raise ValueError(f"{path}: not a NIfTI-1 file (short header)")
    endian = "<" if struct.unpack_from("<i", raw, 0)[0] == _HDR_SIZE else ">"
    if struct.unpack_from(endian + "i", raw, 0)[0] != _HDR_SIZE or raw[344:347] != b"n+1":
        raise ValueError(f"{path}: not a single-file NIfTI-1 image")
    dim = struct.unpack_from(endian + "8h", raw, 40)
    dtype_code = struct.unpack_from(endian + "h", raw, 70)[0]
    if dtype_code not in _NIFTI_DTYPES:
        raise ValueError(f"{path}: NIfTI datatype {dtype_code} not supported")
    vox_offset = int(struct.unpack_from(endian + "f", raw, 108)[0])
    slope, inter = struct.unpack_from(endian + "2f", raw, 112)
    shape = tuple(int(d) for d in dim[1:1 + dim[0]])
    dt = np.dtype(_NIFTI_DTYPES[dtype_code]).newbyteorder(endian)
    count = int(np.prod(shape))
    data = np.frombuffer(raw, dtype=dt, count=count, offset=vox_offset).reshape(shape, order="F")
    data = data.astype(np.float32)
    if slope not in (0.0, 1.0) or inter != 0.0:
        data = data * (slope if slope != 0.0 else 1.0) + inter
    return data


def load_arma_params(filepath, voxel_mask=None) -> np.ndarray:
    """(a, b) of every voxel, (V, 2), from an -Rvar file (volumes 0 and 1): the
    masked voxels when ``voxel_mask`` is given, else every voxel flattened
    (fastfuncstuff/glm/arma.py:6372-6459)."""
    filepath = Path(filepath)
    if not filepath.exists():
        raise FileNotFoundError(f"ARMA params file not found: {filepath}")
    vol = _read_nifti1(filepath)
    if vol.ndim != 4 or vol.shape[-1] < 2:
        raise ValueError(f"Expected 4D NIfTI with at least 2 volumes, got shape {vol.shape}")
    a, b = vol[..., 0].reshape(-1), vol[..., 1].reshape(-1)
    if voxel_mask is not None:
        mask = _np(voxel_mask).reshape(-1).astype(bool)
        a, b = a[mask], b[mask]
    return np.stack([a, b], axis=1)
