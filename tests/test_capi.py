"""The C-ABI library builds, loads without a GPU and exports exactly what
include/starxpbd.h declares; the ctypes binding matches the declarations."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "starxpbd.h")


def declarations():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    decls = {}
    for m in re.finditer(r"^\s*([A-Za-z_][\w \*]*?)\b(sx_\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.M | re.S):
        args = m.group(3).strip()
        n = 0 if args in ("", "void") else len([a for a in args.split(",") if a.strip()])
        decls[m.group(2)] = n
    return decls


@pytest.fixture(scope="module")
def lib(pkg):
    from starlab_physics_gb300 import _lib

    path = _lib.load().__dict__.get("_name") or _lib.library_path()
    return ctypes.CDLL(_lib.library_path())


def test_header_parses():
    d = declarations()
    assert "sx_predict" in d and "sx_collision_sweep" in d and len(d) >= 20


def test_every_declared_symbol_is_exported(lib):
    for name in declarations():
        assert hasattr(lib, name), f"{name} declared in starxpbd.h but not exported"


def test_binding_matches_header(pkg):
    from starlab_physics_gb300 import _lib

    d = declarations()
    assert set(d) == set(_lib.SIGNATURES), set(d) ^ set(_lib.SIGNATURES)
    for name, n in d.items():
        assert len(_lib.SIGNATURES[name][0]) == n, name


def test_sizing_and_argument_checks_without_gpu(pkg):
    """Workspace sizing and argument validation are host code: they run without a
    device and report errors through return codes and sx_last_error()."""
    from starlab_physics_gb300 import _lib

    L = _lib.load()
    assert L.sx_version() == 1
    assert L.sx_radix_sort_workspace_bytes(1 << 20) >= 8 << 20
    assert L.sx_cell_bvh_workspace_bytes(130050) > 130050 * 4
    assert L.sx_color_workspace_bytes(81, 208) > 0
    rc = L.sx_predict(None, None, None, None, -1, 0.1, 0.0, 0.0, 0.0, None)
    assert rc == _lib.SX_ERR_ARG
    assert b"n_verts" in L.sx_last_error()
    rc = L.sx_jacobi_sweep(None, None, None, None, None, None, 4, 1.0, 1.0, 0, None)
    assert rc == _lib.SX_ERR_ARG and b"null" in L.sx_last_error()
    with pytest.raises(_lib.SxError):
        _lib.sx.sx_karras_build(None, 0, 0, None, None, None, None, None, None)


def test_product_does_not_import_oracle():
    """The package must not reach the CPU oracle (no CPU fallback)."""
    pkg_dir = os.path.join(ROOT, "starlab-physics_gb300")
    pat = re.compile(r"^\s*(from\s+\.*oracle|import\s+oracle|from\s+\S*pyoracle|import\s+\S*pyoracle)|liboracle",
                     re.M)
    for f in os.listdir(pkg_dir):
        if f.endswith(".py"):
            src = open(os.path.join(pkg_dir, f)).read()
            assert not pat.search(src), f
