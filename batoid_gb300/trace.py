"""Per-surface trace operations (batoid/trace.py).

Each builds the CoordTransform on the host (3x3 algebra) and launches the
fused trace kernel with a one-stage program through the C-ABI.
"""
from . import _device as D
from . import _lib
from .coordTransform import CoordTransform


def _ct_args(ct):
    dr, pdr = _lib.vec(ct.dr, 3)
    rot, prot = _lib.vec(ct.drot.ravel(), 9)
    return (dr, rot), pdr, prot


def applyForwardTransform(ct, rv):
    keep, pdr, prot = _ct_args(ct)
    r = rv._rv
    _lib.check(_lib.lib().bt_apply_forward_transform(pdr, prot, r, 1, D.stream_ptr()))
    rv.coordSys = ct.toSys
    return rv


def applyReverseTransform(ct, rv):
    keep, pdr, prot = _ct_args(ct)
    r = rv._rv
    _lib.check(_lib.lib().bt_apply_reverse_transform(pdr, prot, r, 1, D.stream_ptr()))
    rv.coordSys = ct.fromSys
    return rv


def applyForwardTransformArrays(ct, x, y, z):
    """In-place on device tensors x, y, z."""
    keep, pdr, prot = _ct_args(ct)
    _lib.check(_lib.lib().bt_apply_forward_transform_arrays(pdr, prot, D.ptr(x), D.ptr(y), D.ptr(z),
                                                           x.numel(), 1, D.stream_ptr()))


def applyReverseTransformArrays(ct, x, y, z):
    keep, pdr, prot = _ct_args(ct)
    _lib.check(_lib.lib().bt_apply_reverse_transform_arrays(pdr, prot, D.ptr(x), D.ptr(y), D.ptr(z),
                                                           x.numel(), 1, D.stream_ptr()))


def obscure(obsc, rv):
    r = rv._rv
    _lib.check(_lib.lib().bt_obscure(obsc._obsc.ptr, r, 1, D.stream_ptr()))
    return rv


def _niter():
    from .global_vars import _batoid_niter
    return _batoid_niter


def intersect(surface, rv, coordSys=None, coating=None):
    """Intersect rays with ``surface`` expressed in ``coordSys`` (in place)."""
    if coordSys is None:
        coordSys = rv.coordSys
    keep, pdr, prot = _ct_args(CoordTransform(rv.coordSys, coordSys))
    r = rv._rv
    _lib.check(_lib.lib().bt_intersect(surface._surface.ptr, pdr, prot, r,
                                       coating._coating.ptr if coating else None, 1, _niter(),
                                       D.stream_ptr()))
    rv.coordSys = coordSys
    return rv


def reflect(surface, rv, coordSys=None, coating=None):
    if coordSys is None:
        coordSys = rv.coordSys
    keep, pdr, prot = _ct_args(CoordTransform(rv.coordSys, coordSys))
    r = rv._rv
    _lib.check(_lib.lib().bt_reflect(surface._surface.ptr, pdr, prot, r,
                                     coating._coating.ptr if coating else None, 1, _niter(),
                                     D.stream_ptr()))
    rv.coordSys = coordSys
    return rv


def refract(surface, rv, m1, m2, coordSys=None, coating=None):
    if coordSys is None:
        coordSys = rv.coordSys
    keep, pdr, prot = _ct_args(CoordTransform(rv.coordSys, coordSys))
    r = rv._rv
    _lib.check(_lib.lib().bt_refract(surface._surface.ptr, pdr, prot, m1._medium.ptr, m2._medium.ptr, r,
                                     coating._coating.ptr if coating else None, 1, _niter(),
                                     D.stream_ptr()))
    rv.coordSys = coordSys
    return rv


def rSplit(surface, rv, inMedium, outMedium, coating, coordSys=None):
    """(refracted, reflected): ``rv`` becomes the refracted rays, a copy the
    reflected ones (batoid/trace.py:119-136; src/batoid.cpp:509-674)."""
    if coordSys is None:
        coordSys = rv.coordSys
    keep, pdr, prot = _ct_args(CoordTransform(rv.coordSys, coordSys))
    rvSplit = rv.copy()
    _lib.check(_lib.lib().bt_rsplit(surface._surface.ptr, pdr, prot, inMedium._medium.ptr, outMedium._medium.ptr,
                                    coating._coating.ptr, rv._rv, rvSplit._rv, 1, _niter(), D.stream_ptr()))
    rv.coordSys = coordSys
    rvSplit.coordSys = coordSys
    return rv, rvSplit


def refractScreen(surface, rv, screen, coordSys=None):
    """Intersect, deflect by the screen's OPD gradient, add its OPD to t
    (batoid/trace.py:139-153; src/batoid.cpp:677-810)."""
    if coordSys is None:
        coordSys = rv.coordSys
    keep, pdr, prot = _ct_args(CoordTransform(rv.coordSys, coordSys))
    _lib.check(_lib.lib().bt_refract_screen(surface._surface.ptr, pdr, prot, screen._surface.ptr, rv._rv, 1,
                                            _niter(), D.stream_ptr()))
    rv.coordSys = coordSys
    return rv
