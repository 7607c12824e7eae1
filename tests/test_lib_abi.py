"""The C ABI library builds, loads and exports what include/ffs_reml.h declares.

No kernel is launched here: these run on the CPU-only container. The ctypes
structures are checked field by field against the header, compiled by gcc.
"""

from __future__ import annotations

import re
import shutil
import subprocess

import pytest

from fastfuncstuff_gb300 import _lib
from fastfuncstuff_gb300 import build as B
from tests.conftest import ROOT

HEADER = ROOT / "include" / "ffs_reml.h"

STRUCTS = {
    "ffs_grid_desc": _lib.GridDesc,
    "ffs_grid_out": _lib.GridOut,
    "ffs_prep_args": _lib.PrepArgs,
    "ffs_project_args": _lib.ProjectArgs,
    "ffs_surface_args": _lib.SurfaceArgs,
    "ffs_select_args": _lib.SelectArgs,
    "ffs_gls_args": _lib.GlsArgs,
    "ffs_merge_field": _lib.MergeField,
    "ffs_dsort_args": _lib.DsortArgs,
}


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ffs_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for n in ("ffs_grid_build", "ffs_reml_prep", "ffs_reml_project_tc", "ffs_reml_surface",
              "ffs_reml_select", "ffs_reml_gls", "ffs_last_error"):
        assert n in names
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def declared_arity() -> dict[str, int]:
    """Number of parameters of every function the header declares."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(ffs_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_take_the_declared_number_of_arguments():
    arity = declared_arity()
    for name, (argtypes, _) in _lib.SIGNATURES.items():
        assert name in arity, name
        assert len(argtypes) == arity[name], (name, len(argtypes), arity[name])


def _kind_of_param(decl: str) -> str:
    """pointer / int / size_t / uint64 / float of one declared parameter."""
    if "*" in decl:
        return "pointer"
    words = decl.replace("const", " ").split()
    ty = " ".join(words[:-1])
    return {"int": "int", "size_t": "size_t", "uint64_t": "uint64", "float": "float"}.get(ty, ty)


def _kind_of_ctype(ct) -> str:
    import ctypes as C

    if ct is C.c_void_p or ct is C.c_char_p or (isinstance(ct, type) and issubclass(ct, C._Pointer)):
        return "pointer"
    return {C.c_int: "int", C.c_size_t: "size_t", C.c_uint64: "uint64", C.c_float: "float"}.get(ct, str(ct))


def test_ctypes_signatures_match_the_declared_parameter_types():
    """Each argument's ctypes type has the kind of the declared parameter
    (ctypes truncates an int passed where a pointer is declared without a
    word, so a pointer typed c_int loses its upper half)."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    decls = {m.group(1): m.group(2) for m in re.finditer(r"\b(ffs_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S)}
    for name, (argtypes, _) in _lib.SIGNATURES.items():
        params = [x.strip() for x in decls[name].split(",") if x.strip() not in ("", "void")]
        for i, (decl, ct) in enumerate(zip(params, argtypes)):
            assert _kind_of_param(decl) == _kind_of_ctype(ct), (name, i, decl, ct)


def test_library_builds_loads_and_exports_every_symbol():
    path = B.build()
    assert path.exists()
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.ffs_version() >> 16 == 1
    assert lib.ffs_status_string(1).decode() == "invalid argument"
    assert lib.ffs_last_error().decode() == ""
    # a host-only entry point: workspace sizing
    assert lib.ffs_grid_work_bytes(400, 20, 561) == 8 * (4 * 400 + 2 * 20 * 400 + 4 * 20 * 20) * 561


def test_argument_validation_needs_no_gpu():
    """Null descriptors are rejected on the host with a message, before any launch."""
    lib = _lib.load()
    st = lib.ffs_grid_build(None, None, None)
    assert st == _lib.FFS_ERR_INVALID
    assert "null" in lib.ffs_last_error().decode()
    with pytest.raises(ValueError, match="ffs_reml_prep"):
        _lib.check(lib.ffs_reml_prep(None, None), "ffs_reml_prep")
    fake = 256  # a non-null address no check reads
    # the banded sums: a band wider than the limit; window mode without ident
    st = lib.ffs_reml_band_sums(8, None, 16, fake, fake, fake, _lib.FFS_BAND_MAX_W + 1, fake, None, None, 0, None,
                                None, 0, 0, None, fake, 1, fake, None)
    assert st == _lib.FFS_ERR_INVALID and "ffs_reml_band_sums" in lib.ffs_last_error().decode()
    st = lib.ffs_reml_band_sums(8, None, 16, fake, fake, fake, 3, fake, fake, fake, 4, fake, fake, 5, 5, None,
                                None, 0, fake, None)
    assert st == _lib.FFS_ERR_INVALID and "window mode" in lib.ffs_last_error().decode()
    # a strip work list whose pair blocks exceed one 256-column MMA tile
    st = lib.ffs_reml_segment_items(2, fake, 16, 20, 13, fake, fake, 64, fake, None)
    assert st == _lib.FFS_ERR_INVALID and "ffs_reml_segment_items" in lib.ffs_last_error().decode()
    # per-row designs need the pairs per design
    st = lib.ffs_reml_strip(8, None, 16, 2, 4, fake, fake, fake, fake, fake, fake, fake, fake, fake, fake, fake, 0,
                            None, None)
    assert st == _lib.FFS_ERR_INVALID and "designs need P" in lib.ffs_last_error().decode()


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_ctypes_structures_match_the_header(tmp_path):
    lines = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            parts = line.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, py in STRUCTS.items():
        assert got[(cname, "size")] == C_sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def C_sizeof(py) -> int:
    import ctypes

    return ctypes.sizeof(py)
