"""The C-ABI library loads and exports every entry point that
include/getm_gb300.h declares, with the argument lists the ctypes binding
uses; host-only handle calls validate their arguments.  No GPU needed."""

import ctypes
import re
from pathlib import Path

HEADER = Path(__file__).resolve().parent.parent / "include" / "getm_gb300.h"


def header_signatures():
    src = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for name, args in re.findall(r"int\s+(getm_\w+)\s*\(([^)]*)\)\s*;", src, flags=re.S):
        codes = ""
        for a in args.split(","):
            a = a.strip()
            if a.startswith("cudaStream_t"):
                codes += "s"
            elif "*" in a:
                codes += "p"
            elif a.startswith("double"):
                codes += "d"
            elif a.startswith("long long"):
                codes += "l"
            elif a.startswith("int"):
                codes += "i"
            else:
                raise AssertionError(f"unparsed argument {a!r} of {name}")
        out[name] = codes
    return out


def test_every_declared_symbol_is_exported_with_matching_signature():
    from getm_gb300 import _lib

    sigs = header_signatures()
    assert len(sigs) >= 35
    for name, codes in sigs.items():
        assert hasattr(_lib.lib, name), f"{name} not exported"
        bound = _lib._SIGS[name].replace("c", "p")
        assert bound == codes, f"{name}: binding {bound} != header {codes}"
    assert set(_lib._SIGS) == set(sigs)


def test_grid_handle_host_calls():
    from getm_gb300 import _lib

    h = ctypes.c_void_p()
    assert _lib.lib.getm_create_grid(1, 10, 1, 8, 1, 5, 2, 2, ctypes.byref(h)) == 0
    assert h.value
    for name in (b"mask", b"dx", b"dy", b"idx", b"idy", b"iarea", b"area"):
        assert _lib.lib.getm_grid_set_array(h, name, 4096) == 0
    assert _lib.lib.getm_grid_set_array(h, b"not_a_metric", 4096) == 1
    assert _lib.lib.getm_grid_finalize(h) == 0


def test_invalid_extents_are_rejected():
    from getm_gb300 import _lib

    h = ctypes.c_void_p()
    assert _lib.lib.getm_create_grid(5, 1, 1, 8, 1, 5, 2, 2, ctypes.byref(h)) == 1
    assert _lib.lib.getm_create_grid(1, 5, 1, 8, 1, 5, 2, 2, None) == 1
    # argument checks happen before any device work
    assert _lib.lib.getm_elevation2depth(10, None, None, 0.1, None, None, None) == 1
    assert _lib.lib.getm_vertical_diffusion_batch(0, 1, 1, None, None, 1.0, 1.0, None, None, 1, None, None, None, None, None, None) == 1
    assert _lib.lib.getm_surface_pressure_gradient(10, 10, 0, 5, 1, 5, None, None, None, None, None, None, None, None, 0.1, None, None, None) == 1


def test_product_path_has_no_fallback(monkeypatch, tmp_path):
    """With the library missing the binding raises instead of falling back."""
    import importlib
    import sys

    monkeypatch.setenv("GETM_GB300_LIB", str(tmp_path / "missing.so"))
    saved = sys.modules.pop("getm_gb300._lib")
    try:
        try:
            importlib.import_module("getm_gb300._lib")
        except ImportError as e:
            assert "not found" in str(e)
        else:
            raise AssertionError("import succeeded without the library")
    finally:
        sys.modules["getm_gb300._lib"] = saved


def test_split2d_fields_layout_matches_header():
    """getm_split2d_fields: the ctypes mirror has the header's members in the
    header's order (all pointers)."""
    from getm_gb300 import _pygetm

    src = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    body = re.search(r"typedef struct getm_split2d_fields\s*\{(.*?)\}\s*getm_split2d_fields;", src, flags=re.S)
    assert body
    names = []
    for decl in body.group(1).split(";"):
        decl = decl.strip()
        if decl:
            assert "*" in decl, decl
            names.append(decl.split("*")[-1].strip())
    assert tuple(names) == _pygetm.SPLIT2D_FIELDS
    assert ctypes.sizeof(_pygetm.Split2DFields) == 8 * len(names)


def test_split2d_substep_rejects_missing_fields():
    from getm_gb300 import _lib, _pygetm

    f = _pygetm.Split2DFields()
    args = [ctypes.byref(f), 20, 20, 2, 2, 0, 1, 1, 1, 10.0, 0.02, 0.1] + [None] * 4 + [0] + [None] * 4 + [0, None]
    assert _lib.lib.getm_split2d_substep(*args) == 1
    args[0] = None
    assert _lib.lib.getm_split2d_substep(*args) == 1


def test_depth3d_fields_layout_matches_header():
    """getm_depth3d_fields: the ctypes mirror has the header's members in the
    header's order (all pointers)."""
    from getm_gb300 import _pygetm

    src = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    body = re.search(r"typedef struct getm_depth3d_fields\s*\{(.*?)\}\s*getm_depth3d_fields;", src, flags=re.S)
    assert body
    names = [d.strip().split("*")[-1].strip() for d in body.group(1).split(";") if d.strip()]
    assert tuple(names) == _pygetm.DEPTH3D_FIELDS
    assert ctypes.sizeof(_pygetm.Depth3DFields) == 8 * len(names)


def test_package_modules_import():
    """Every module of the package imports without a GPU (syntax, names)."""
    import importlib
    from pathlib import Path

    import getm_gb300

    for f in sorted(Path(getm_gb300.__path__[0]).glob("*.py")):
        importlib.import_module("getm_gb300." + f.stem)
