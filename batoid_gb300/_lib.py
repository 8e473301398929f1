"""ctypes binding of ``libbatoid_gb300.so`` (the C-ABI in include/batoid_gb300.h).

This module plays the role of the reference's pybind11 module ``_batoid``
(pysrc/batoid.cpp:31-154).  The library is required: importing any compute
path without it raises ImportError; there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbatoid_gb300.so")

c_double_p = ctypes.POINTER(ctypes.c_double)
c_u8_p = ctypes.POINTER(ctypes.c_uint8)
c_void_p = ctypes.c_void_p
c_int = ctypes.c_int
c_size_t = ctypes.c_size_t
c_double = ctypes.c_double

BT_OK = 0
BT_ERR_ARG = 1
BT_ERR_CUDA = 2
BT_ERR_UNSUPPORTED = 3
BT_ERR_RANK = 4
BT_ERR_TIMEOUT = 5
BT_ERR_ALLOC = 6

STAGE_INTERSECT = 0
STAGE_REFLECT = 1
STAGE_REFRACT = 2
STAGE_SCREEN = 4


class BtRayVector(ctypes.Structure):
    _fields_ = [
        ("x", c_void_p), ("y", c_void_p), ("z", c_void_p),
        ("vx", c_void_p), ("vy", c_void_p), ("vz", c_void_p),
        ("t", c_void_p), ("wavelength", c_void_p), ("flux", c_void_p),
        ("vignetted", c_void_p), ("failed", c_void_p),
        ("size", c_size_t),
    ]


class BatoidError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class BtBatchDesc(ctypes.Structure):
    """bt_batch_desc of include/batoid_gb300.h."""
    _fields_ = [
        ("nstages", c_size_t),
        ("kinds", c_void_p),
        ("surfaces", c_void_p),
        ("dr", c_void_p),
        ("drot", c_void_p),
        ("media", c_void_p),
        ("obscurations", c_void_p),
        ("nvar", c_int),
        ("var_stages", c_void_p),
        ("modal_stage", c_int),
        ("modal_grid", c_double * 4),
        ("modal_nx", c_int),
        ("modal_ny", c_int),
        ("nmodes", c_int),
        ("modes", c_void_p),
        ("modal_use_nan", c_int),
        ("stop_dr", c_double * 3),
        ("stop_drot", c_double * 9),
        ("sphere", c_void_p),
        ("sphere_radius", c_double),
        ("pupil_size", c_double),
        ("r_inner", c_double),
        ("r_outer", c_double),
        ("jmax", c_int),
        ("basis", c_void_p),
        ("side", c_int),
    ]


# (name, restype, argtypes); handles are void*.
_P = c_void_p
_PP = ctypes.POINTER(c_void_p)
_D3 = c_double_p
_SIGS = [
    ("bt_last_error", ctypes.c_char_p, []),
    ("bt_version", c_int, []),
    ("bt_device_sm_count", c_int, [ctypes.POINTER(c_int)]),
    ("bt_plane_create", c_int, [_PP]),
    ("bt_tilted_create", c_int, [c_double, c_double, _PP]),
    ("bt_sphere_create", c_int, [c_double, _PP]),
    ("bt_paraboloid_create", c_int, [c_double, _PP]),
    ("bt_quadric_create", c_int, [c_double, c_double, _PP]),
    ("bt_asphere_create", c_int, [c_double, c_double, c_double_p, c_size_t, _PP]),
    ("bt_polynomial_create", c_int, [c_double_p, c_double_p, c_double_p, c_double, c_double,
                                     c_size_t, c_size_t, _PP]),
    ("bt_table_create", c_int, [c_double, c_double, c_double, c_double, c_double_p, c_double_p,
                                c_double_p, c_double_p, c_size_t, c_size_t, c_int, _PP]),
    ("bt_table_destroy", None, [_P]),
    ("bt_bicubic_create", c_int, [_P, _PP]),
    ("bt_sum_create", c_int, [_PP, c_size_t, _PP]),
    ("bt_surface_destroy", None, [_P]),
    ("bt_surface_sag", c_int, [_P, _P, _P, _P, c_size_t, _P]),
    ("bt_surface_normal", c_int, [_P, _P, _P, _P, c_size_t, _P]),
    ("bt_const_medium_create", c_int, [c_double, _PP]),
    ("bt_table_medium_create", c_int, [c_double_p, c_double_p, c_size_t, _PP]),
    ("bt_sellmeier_medium_create", c_int, [c_double] * 6 + [_PP]),
    ("bt_sumita_medium_create", c_int, [c_double] * 6 + [_PP]),
    ("bt_air_create", c_int, [c_double, c_double, c_double, _PP]),
    ("bt_medium_destroy", None, [_P]),
    ("bt_medium_getN", c_int, [_P, _P, _P, c_size_t, _P]),
    ("bt_obsc_circle_create", c_int, [c_double, c_double, c_double, _PP]),
    ("bt_obsc_annulus_create", c_int, [c_double, c_double, c_double, c_double, _PP]),
    ("bt_obsc_rectangle_create", c_int, [c_double, c_double, c_double, c_double, c_double, _PP]),
    ("bt_obsc_ray_create", c_int, [c_double, c_double, c_double, c_double, _PP]),
    ("bt_obsc_polygon_create", c_int, [c_double_p, c_double_p, c_size_t, _PP]),
    ("bt_obsc_negation_create", c_int, [_P, _PP]),
    ("bt_obsc_union_create", c_int, [_PP, c_size_t, _PP]),
    ("bt_obsc_intersection_create", c_int, [_PP, c_size_t, _PP]),
    ("bt_obsc_destroy", None, [_P]),
    ("bt_obsc_contains", c_int, [_P, _P, _P, _P, c_size_t, _P]),
    ("bt_simple_coating_create", c_int, [c_double, c_double, _PP]),
    ("bt_coating_destroy", None, [_P]),
    ("bt_apply_forward_transform", c_int, [_D3, _D3, ctypes.POINTER(BtRayVector), c_int, _P]),
    ("bt_apply_reverse_transform", c_int, [_D3, _D3, ctypes.POINTER(BtRayVector), c_int, _P]),
    ("bt_apply_forward_transform_arrays", c_int, [_D3, _D3, _P, _P, _P, c_size_t, c_int, _P]),
    ("bt_apply_reverse_transform_arrays", c_int, [_D3, _D3, _P, _P, _P, c_size_t, c_int, _P]),
    ("bt_finish_parallel", c_int, [_D3, _D3, _D3, _P, _P, _P, c_size_t, _P]),
    ("bt_stop_points_grid", c_int, [c_int, c_int, c_double, c_double, _D3, _D3, _P, _P, _P]),
    ("bt_stop_points_rings", c_int, [c_int, _P, _P, _P, ctypes.c_longlong, _P, _P, _P]),
    ("bt_stop_points_spokes", c_int, [_P, c_int, _P, c_int, _P, _P, _P]),
    ("bt_obscure", c_int, [_P, ctypes.POINTER(BtRayVector), c_int, _P]),
    ("bt_refract_screen", c_int, [_P, _D3, _D3, _P, ctypes.POINTER(BtRayVector), c_int, c_int, _P]),
    ("bt_rsplit", c_int, [_P, _D3, _D3, _P, _P, _P, ctypes.POINTER(BtRayVector), ctypes.POINTER(BtRayVector), c_int,
                          c_int, _P]),
    ("bt_intersect", c_int, [_P, _D3, _D3, ctypes.POINTER(BtRayVector), _P, c_int, c_int, _P]),
    ("bt_reflect", c_int, [_P, _D3, _D3, ctypes.POINTER(BtRayVector), _P, c_int, c_int, _P]),
    ("bt_refract", c_int, [_P, _D3, _D3, _P, _P, ctypes.POINTER(BtRayVector), _P, c_int, c_int, _P]),
    ("bt_rv_position_at_time", c_int, [ctypes.POINTER(BtRayVector), c_double, _P, _P, _P, c_int, _P]),
    ("bt_rv_propagate_in_place", c_int, [ctypes.POINTER(BtRayVector), c_double, c_int, _P]),
    ("bt_rv_phase", c_int, [ctypes.POINTER(BtRayVector), c_double, c_double, c_double, c_double, _P, c_int, _P]),
    ("bt_rv_amplitude", c_int, [ctypes.POINTER(BtRayVector), c_double, c_double, c_double, c_double, _P,
                                c_int, _P]),
    ("bt_rv_sum_amplitude", c_int, [ctypes.POINTER(BtRayVector), c_double, c_double, c_double, c_double,
                                    c_int, c_int, c_double_p, _P]),
    ("bt_rv_equal", c_int, [ctypes.POINTER(BtRayVector), ctypes.POINTER(BtRayVector),
                            ctypes.POINTER(c_int), _P]),
    ("bt_optic_create", c_int, [c_size_t, ctypes.POINTER(c_int), _PP, c_double_p, c_double_p, _PP, _PP,
                                _PP, _PP]),
    ("bt_optic_create_ex", c_int, [c_size_t, ctypes.POINTER(c_int), _PP, c_double_p, c_double_p, _PP, _PP,
                                   _PP, _PP, _PP]),
    ("bt_optic_destroy", None, [_P]),
    ("bt_optic_nstages", c_int, [_P, ctypes.POINTER(c_int)]),
    ("bt_optic_trace", c_int, [_P, ctypes.POINTER(BtRayVector), c_int, _P]),
    ("bt_optic_trace_into", c_int, [_P, ctypes.POINTER(BtRayVector), ctypes.POINTER(BtRayVector), c_int, _P]),
    ("bt_optic_trace_full", c_int, [_P, ctypes.POINTER(BtRayVector), ctypes.POINTER(BtRayVector), c_int, _P]),
    ("bt_optic_trace_host", c_int, [_P, ctypes.POINTER(BtRayVector), c_int, c_size_t, _P]),
    ("bt_huygens_amplitudes", c_int, [ctypes.POINTER(BtRayVector), c_double, c_double, c_double, c_double_p,
                                      c_int, c_int, c_double, c_int, _P, _P, _P]),
    ("bt_huygens_amplitudes_fields", c_int, [ctypes.POINTER(BtRayVector), c_int, c_double_p, c_double_p,
                                             c_double_p, c_int, c_int, c_int, _P, _P, _P]),
    ("bt_huygens_amplitudes_noalloc", c_int, [ctypes.POINTER(BtRayVector), c_double, c_double, c_double,
                                              c_double_p, c_int, c_int, c_double, c_int, _P, _P, _P]),
    ("bt_zernike_normal_equations", c_int, [_P, _P, _P, _P, c_int, _P, c_int, c_int, _P, _P, _P]),
    ("bt_batch_create", c_int, [ctypes.POINTER(BtBatchDesc), _PP]),
    ("bt_batch_destroy", None, [_P]),
    ("bt_batch_prepare", c_int, [_P, c_int, _P, _P]),
    ("bt_batch_zernike", c_int, [_P, c_int, _P, _P, _P, _P, _P, c_int, _P, _P, c_int, _P, _P, c_int, c_int, c_int,
                                 _P]),
    ("bt_batch_zernike_graph", c_int, [_P, c_int, _P, _P, _P, _P, _P, c_int, _P, _P, c_int, _P, _P, c_int, c_int,
                                       c_int, _P]),
    ("bt_mlp_gemm", c_int, [_P, _P, c_int, c_int, c_int, c_int, c_int, c_int, _P, _P, _P, _P, _P, _P]),
    ("bt_mlp_pack", c_int, [_P, c_int, c_int, c_int, c_int, _P, _P, _P]),
    ("bt_mlp_loss", c_int, [_P, c_int, _P, _P, c_int, c_int, c_int, c_int, ctypes.c_float, c_int, _P, _P, _P, _P]),
    ("bt_mlp_colsum", c_int, [_P, c_int, c_int, _P, _P]),
    ("bt_mlp_adam", c_int, [_P, c_int, _P, ctypes.c_longlong, _P, _P, _P, ctypes.c_float, ctypes.c_float,
                            ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, c_int, c_int, _P, _P,
                            _P]),
    ("bt_mlp_adam_dev", c_int, [_P, c_int, _P, ctypes.c_longlong, _P, _P, _P, _P, ctypes.c_float, ctypes.c_float,
                                ctypes.c_float, c_int, c_int, _P, _P, _P]),
    ("bt_surrogate_combine", c_int, [_P, c_int, c_int, _P, _P, _P, c_int, _P, c_double, c_int, c_int, _P, _P, c_int,
                                     _P]),
    ("bt_mlp_gather", c_int, [_P, _P, _P, c_int, _P, c_int, c_int, _P, _P, _P]),
    ("bt_mlp_schedule", c_int, [_P, _P, _P, ctypes.c_longlong, _P, _P]),
    ("bt_surrogate_guard", c_int, [_P, c_int, c_int, _P, _P, _P, _P, c_int, c_double, c_double, _P, c_int, _P]),
    ("bt_measure_fp64_peak", c_int, [c_int, c_double_p, _P]),
    ("bt_measure_fp32_peak", c_int, [c_int, c_double_p, _P]),
    ("bt_check_device_status", c_int, [_P]),
]

EXPORTED = [s[0] for s in _SIGS]

_lib = None


def load(path=None):
    """Load the library (once) and attach signatures.  Raises ImportError."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(
            f"{path} not found: build it with `python -m batoid_gb300.build` "
            "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def lib():
    return load()


def check(rc):
    if rc != BT_OK:
        msg = lib().bt_last_error()
        raise BatoidError(rc, msg.decode() if msg else "unknown error")


def new_handle(fn, *args):
    h = c_void_p()
    check(fn(*args, ctypes.byref(h)))
    return h


def dptr(arr):
    """ctypes double* of a contiguous float64 numpy array (host)."""
    a = np.ascontiguousarray(arr, dtype=np.float64)
    return a, a.ctypes.data_as(c_double_p)


def vec(values, n):
    a = np.ascontiguousarray(np.asarray(values, dtype=np.float64).reshape(-1))
    if a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a, a.ctypes.data_as(c_double_p)
