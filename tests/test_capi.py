"""The C-ABI library loads and exports every entry point the header declares
(no device work: CPU only)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "batoid_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(bt_[A-Za-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert len(names) > 50
    for must in ("bt_optic_trace", "bt_reflect", "bt_refract", "bt_intersect", "bt_huygens_amplitudes",
                 "bt_rv_sum_amplitude", "bt_zernike_normal_equations", "bt_optic_trace_host"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from batoid_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from batoid_gb300 import _lib
    assert set(declared_functions()) == set(_lib.EXPORTED)


def test_host_only_calls():
    """Handle creation and argument checking need no device."""
    from batoid_gb300 import _lib
    L = _lib.load()
    assert L.bt_version() == 1
    h = ctypes.c_void_p()
    assert L.bt_sphere_create(2.0, ctypes.byref(h)) == 0
    child = (ctypes.c_void_p * 2)(h, h)
    s = ctypes.c_void_p()
    assert L.bt_sum_create(child, 2, ctypes.byref(s)) == 0
    nested = (ctypes.c_void_p * 1)(s)
    s2 = ctypes.c_void_p()
    assert L.bt_sum_create(nested, 1, ctypes.byref(s2)) == _lib.BT_ERR_UNSUPPORTED
    assert b"nested" in L.bt_last_error()
    assert L.bt_optic_trace(None, None, 5, None) == _lib.BT_ERR_ARG
    L.bt_surface_destroy(s)
    L.bt_surface_destroy(h)


def test_python_objects_build_without_device():
    import batoid_gb300 as bt
    from batoid_gb300 import workloads as W
    opt = W.tma_optic(bt)
    assert len(opt._interfaces()) == 12
    assert opt["M1"].name == "M1"
    assert opt["L2_exit"].outMedium == bt.ConstMedium(1.0)
    shifted = opt.withGloballyShiftedOptic("M2", [0.0, 1e-3, 0.0])
    assert shifted["M2"].coordSys.origin[1] == pytest.approx(1e-3)
    rotated = opt.withLocallyRotatedOptic("Camera", bt.RotX(1e-5))
    assert rotated["Detector"].coordSys != opt["Detector"].coordSys
