"""The C-ABI library loads and exports every entry point include/amcl3d_gpu.h
declares (no compute calls: these run without a GPU)."""

import ctypes
import re

from conftest import ROOT


def declared_functions():
    text = (ROOT / "include" / "amcl3d_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(amcl_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("amcl_grid_build", "amcl_grid_cloud_weights", "amcl_pf_init", "amcl_pf_predict", "amcl_pf_update",
                 "amcl_pf_resample", "amcl_pf_get_mean", "amcl_grid_is_into_map", "amcl_grid_slice",
                 "amcl_grid_save", "amcl_grid_load"):
        assert must in names


def test_library_exports_every_declared_symbol(native_lib):
    lib = ctypes.CDLL(str(native_lib))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(native_lib):
    from amcl3d_gb300 import _native

    bound = set(_native.exported_symbols())
    missing = [n for n in declared_functions() if n not in bound]
    assert not missing, missing


def test_status_strings(native_lib):
    from amcl3d_gb300 import _native

    assert _native.lib.amcl_status_string(0) == b"ok"
    assert _native.lib.amcl_status_string(4) == b"device wait timed out"


def test_build_targets_sm103a_only():
    from amcl3d_gb300 import build

    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "--fmad=false" in build.NVCC_FLAGS
