"""The C-ABI library loads, exports every function include/*.h declares, and the Python struct mirrors
match the C layouts.  No GPU needed: nothing here launches a kernel."""
import ctypes
import os
import re

import pytest

import doonengine_gb300 as dn

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for hdr in ("include/dn_cuda.h", "include/DoonEngine/voxel.h", "include/DoonEngine/dn_math.h",
                "include/DoonEngine/globals.h", "include/DoonEngine/serve.h", "include/DoonEngine/voxelShapes.h"):
        txt = open(os.path.join(ROOT, hdr)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        txt = re.sub(r"#define[^\n]*", "", txt)
        for m in re.finditer(r"\b((?:DN|dn)_[A-Za-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(dnlib):
    missing = [n for n in declared_functions() if not hasattr(dnlib, n)]
    assert not missing, missing
    assert len(declared_functions()) > 80


def test_message_callback_symbol(dnlib):
    ctypes.c_void_p.in_dll(dnlib, "g_DN_message_callback")


def test_struct_layouts_match(dnlib):
    assert dn.check_layout(dnlib) == []


def test_bindings_cover_header(dnlib):
    bound = set(dn.exported_names())
    missing = [n for n in declared_functions() if n not in bound and n not in ("DN_host_malloc", "DN_host_free",
                                                                               "DN_host_realloc")]
    # every declared entry point has a ctypes signature except the raw allocation hooks and pure math helpers
    math_only = {n for n in missing if n.startswith(("DN_vec3_", "DN_mat4_", "DN_mat3_", "DN_deg_"))}
    assert set(missing) - math_only == set(), sorted(set(missing) - math_only)


def test_cuda_path_fails_loudly_without_gpu(dnlib):
    import doonengine_gb300._lib as L
    n = ctypes.c_int(0)
    has_gpu = dnlib.dn_cuda_init(-1) == 0
    if has_gpu:
        pytest.skip("a GPU is present")
    assert not dnlib.DN_init()
    assert not dnlib.DN_create_volume(L.DNuvec3(2, 2, 2), 8)
    assert b"device" in dnlib.dn_cuda_last_error().lower() or dnlib.dn_cuda_last_error()
