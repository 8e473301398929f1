"""ORACLE — test infrastructure only.

ctypes driver of oracle/liboracle.so (the C restatement of the reference's
per-ray algorithm).  It walks an optic tree exactly as the reference's Python
layer does (batoid/optic.py:391-424, 1013-1083; batoid/trace.py:47-153):
one CPU pass per surface interaction and one per obscuration, transforms
built from the two CoordSys (batoid/coordTransform.py:16-20).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker or as the timed reference port.  The optic and
surface objects it reads are duck-typed: the same attribute names exist on
batoid_gb300 objects and on the reference's own objects.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

_dp = ctypes.POINTER(ctypes.c_double)


class OraSurface(ctypes.Structure):
    pass


OraSurface._fields_ = [
    ("kind", ctypes.c_int),
    ("a", ctypes.c_double), ("b", ctypes.c_double), ("c", ctypes.c_double), ("d", ctypes.c_double),
    ("e", ctypes.c_double),
    ("n", ctypes.c_int), ("m", ctypes.c_int),
    ("p0", _dp), ("p1", _dp), ("p2", _dp), ("p3", _dp),
    ("children", ctypes.POINTER(ctypes.POINTER(OraSurface))),
    ("nchild", ctypes.c_int),
]


class OraMedium(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("p", ctypes.c_double * 6), ("args", _dp), ("vals", _dp),
                ("n", ctypes.c_int)]


class OraObsc(ctypes.Structure):
    pass


OraObsc._fields_ = [
    ("kind", ctypes.c_int), ("p", ctypes.c_double * 6), ("xs", _dp), ("ys", _dp), ("n", ctypes.c_int),
    ("items", ctypes.POINTER(ctypes.POINTER(OraObsc))),
]


class OraRV(ctypes.Structure):
    _fields_ = [(k, _dp) for k in ("x", "y", "z", "vx", "vy", "vz", "t", "w", "f")] + [
        ("vig", ctypes.POINTER(ctypes.c_uint8)), ("fail", ctypes.POINTER(ctypes.c_uint8)),
        ("n", ctypes.c_size_t)]


_lib = None


def build():
    """Compile liboracle.so with the Makefile beside this file."""
    root = os.path.dirname(HERE)
    subprocess.run(["make", "-s", "-f", os.path.join("oracle", "Makefile")], cwd=root, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        L.ora_intersect.argtypes = [P(OraSurface), _dp, _dp, P(OraRV), _dp, ctypes.c_int, ctypes.c_int]
        L.ora_reflect.argtypes = [P(OraSurface), _dp, _dp, P(OraRV), _dp, ctypes.c_int, ctypes.c_int]
        L.ora_refract.argtypes = [P(OraSurface), _dp, _dp, P(OraMedium), P(OraRV), _dp, ctypes.c_int,
                                  ctypes.c_int]
        L.ora_obscure.argtypes = [P(OraObsc), P(OraRV), ctypes.c_int]
        L.ora_forward_transform.argtypes = [_dp, _dp, P(OraRV), ctypes.c_int]
        L.ora_reverse_transform.argtypes = [_dp, _dp, P(OraRV), ctypes.c_int]
        L.ora_sum_amplitude.argtypes = [P(OraRV), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp]
        L.ora_phase.argtypes = [P(OraRV), ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                _dp, ctypes.c_int]
        L.ora_position_at_time.argtypes = [P(OraRV), ctypes.c_double, _dp, _dp, _dp, ctypes.c_int]
        L.ora_propagate.argtypes = [P(OraRV), ctypes.c_double, ctypes.c_int]
        L.ora_getN.argtypes = [P(OraMedium), ctypes.c_double]
        L.ora_getN.restype = ctypes.c_double
        L.ora_contains.argtypes = [P(OraObsc), ctypes.c_double, ctypes.c_double]
        L.ora_sag_array.argtypes = [P(OraSurface), _dp, _dp, _dp, ctypes.c_size_t]
        L.ora_normal_array.argtypes = [P(OraSurface), _dp, _dp, _dp, ctypes.c_size_t]
        L.ora_finish_parallel.argtypes = [_dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_size_t]
        L.ora_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _arr(a, keep):
    a = np.ascontiguousarray(a, dtype=np.float64)
    keep.append(a)
    return a.ctypes.data_as(_dp)


# ---------------------------------------------------------------------------
# conversions from (duck-typed) optics objects
# ---------------------------------------------------------------------------

def surface(s, keep):
    name = type(s).__name__
    o = OraSurface()
    keep.append(o)
    if name == "Plane":
        o.kind = 0
    elif name == "Tilted":
        o.kind, o.a, o.b = 1, s.tanx, s.tany
    elif name == "Sphere":
        o.kind, o.a = 2, s.R
    elif name == "Paraboloid":
        o.kind, o.a = 3, s.R
    elif name == "Quadric":
        o.kind, o.a, o.b = 4, s.R, s.conic
    elif name == "Asphere":
        o.kind, o.a, o.b = 5, s.R, s.conic
        o.p0 = _arr(s._padded_coefs, keep)
        o.n = len(s._padded_coefs)
    elif name in ("Zernike", "PolynomialSurface"):
        o.kind = 6
        o.a, o.b = s.x_origin, s.y_origin
        o.p0 = _arr(s._xycoef, keep)
        o.p1 = _arr(s._xycoef_gradx, keep)
        o.p2 = _arr(s._xycoef_grady, keep)
        o.n, o.m = s._xycoef.shape[0], s._xycoef.shape[1]
    elif name == "Bicubic":
        o.kind = 7
        o.a, o.b, o.c, o.d = s._x0, s._y0, s._dx, s._dy
        o.e = 1.0 if s.nanpolicy.upper() == "NAN" else 0.0
        o.n, o.m = len(s._xs), len(s._ys)
        o.p0 = _arr(s._zs, keep)
        o.p1 = _arr(s._dzdxs, keep)
        o.p2 = _arr(s._dzdys, keep)
        o.p3 = _arr(s._d2zdxdys, keep)
    elif name == "Sum":
        o.kind = 8
        kids = [surface(c, keep) for c in s.surfaces]
        arr = (ctypes.POINTER(OraSurface) * len(kids))(*[ctypes.pointer(k) for k in kids])
        keep.append(arr)
        o.children = ctypes.cast(arr, ctypes.POINTER(ctypes.POINTER(OraSurface)))
        o.nchild = len(kids)
    else:
        raise NotImplementedError(f"oracle: surface {name}")
    return o


def medium(m, keep):
    name = type(m).__name__
    o = OraMedium()
    keep.append(o)
    if name == "ConstMedium":
        o.kind = 0
        o.p[0] = m.n
    elif name == "TableMedium":
        o.kind = 1
        o.args = _arr(m.wavelengths, keep)
        o.vals = _arr(m.ns, keep)
        o.n = len(m.wavelengths)
    elif name == "SellmeierMedium":
        o.kind = 2
        for i, c in enumerate(m.coefs):
            o.p[i] = c
    elif name == "SumitaMedium":
        o.kind = 3
        for i, c in enumerate(m.coefs):
            o.p[i] = c
    elif name == "Air":
        o.kind = 4
        o.p[0], o.p[1], o.p[2] = m.pressure, m.temperature, m.h2o_pressure
    else:
        raise NotImplementedError(f"oracle: medium {name}")
    return o


def obscuration(ob, keep):
    name = type(ob).__name__
    o = OraObsc()
    keep.append(o)
    if name == "ObscCircle":
        o.kind = 0
        o.p[0], o.p[1], o.p[2] = ob.radius, ob.x, ob.y
    elif name == "ObscAnnulus":
        o.kind = 1
        o.p[0], o.p[1], o.p[2], o.p[3] = ob.inner, ob.outer, ob.x, ob.y
    elif name == "ObscRectangle":
        o.kind = 2
        o.p[0], o.p[1], o.p[2], o.p[3], o.p[4] = ob.width, ob.height, ob.x, ob.y, ob.theta
    elif name == "ObscRay":
        o.kind = 3
        o.p[0], o.p[1], o.p[2], o.p[3] = ob.width, ob.theta, ob.x, ob.y
    elif name == "ObscPolygon":
        o.kind = 4
        o.xs = _arr(ob.xs, keep)
        o.ys = _arr(ob.ys, keep)
        o.n = len(ob.xs)
    elif name in ("ObscNegation", "ObscUnion", "ObscIntersection"):
        items = [ob.original] if name == "ObscNegation" else list(ob.items)
        o.kind = {"ObscNegation": 5, "ObscUnion": 6, "ObscIntersection": 7}[name]
        kids = [obscuration(i, keep) for i in items]
        arr = (ctypes.POINTER(OraObsc) * len(kids))(*[ctypes.pointer(k) for k in kids])
        keep.append(arr)
        o.items = ctypes.cast(arr, ctypes.POINTER(ctypes.POINTER(OraObsc)))
        o.n = len(kids)
    else:
        raise NotImplementedError(f"oracle: obscuration {name}")
    return o


# ---------------------------------------------------------------------------
# host ray bundle
# ---------------------------------------------------------------------------

class Rays:
    """Host SoA rays (numpy) with a coordinate frame (origin, rot)."""

    FIELDS = ("x", "y", "z", "vx", "vy", "vz", "t", "wavelength", "flux")

    def __init__(self, x, y, z, vx, vy, vz, t, wavelength, flux, vignetted, failed, origin=None, rot=None):
        n = len(x)
        self.d = np.empty((9, n))
        for k, a in enumerate((x, y, z, vx, vy, vz, t, wavelength, flux)):
            self.d[k] = np.broadcast_to(np.asarray(a, dtype=float), (n,))
        self.b = np.empty((2, n), dtype=np.uint8)
        self.b[0] = np.broadcast_to(np.asarray(vignetted, dtype=bool), (n,))
        self.b[1] = np.broadcast_to(np.asarray(failed, dtype=bool), (n,))
        self.origin = np.zeros(3) if origin is None else np.asarray(origin, dtype=float)
        self.rot = np.eye(3) if rot is None else np.asarray(rot, dtype=float)

    def copy(self):
        r = Rays.__new__(Rays)
        r.d = self.d.copy()
        r.b = self.b.copy()
        r.origin = self.origin.copy()
        r.rot = self.rot.copy()
        return r

    def __getattr__(self, k):
        if k in Rays.FIELDS:
            return self.d[Rays.FIELDS.index(k)]
        if k == "vignetted":
            return self.b[0].astype(bool)
        if k == "failed":
            return self.b[1].astype(bool)
        raise AttributeError(k)

    def struct(self):
        s = OraRV()
        for k, name in enumerate(("x", "y", "z", "vx", "vy", "vz", "t", "w", "f")):
            setattr(s, name, self.d[k].ctypes.data_as(_dp))
        s.vig = self.b[0].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        s.fail = self.b[1].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        s.n = self.d.shape[1]
        return s


def transform(origin1, rot1, origin2, rot2):
    """(dr, drot column-major) from frame 1 to frame 2 (batoid/coordTransform.py:16-20)."""
    dr = rot1.T @ (np.asarray(origin2) - np.asarray(origin1))
    drot = rot1.T @ rot2
    return np.ascontiguousarray(dr, dtype=float), np.ascontiguousarray(drot.ravel(), dtype=float)


def threads():
    return lib().ora_max_threads()


def interface_trace(iface, rays, reverse=False, niter=5, nthreads=None):
    """Interface.trace of the reference: interact, then obscure (batoid/optic.py:391-424)."""
    L = lib()
    nthreads = nthreads or threads()
    keep = []
    cs = iface.coordSys
    dr, drot = transform(rays.origin, rays.rot, cs.origin, cs.rot)
    keep += [dr, drot]
    st = rays.struct()
    s = surface(iface.surface, keep)
    kind = type(iface).__name__
    if kind == "Mirror" or getattr(iface, "_force_reflect", False):
        L.ora_reflect(s, dr.ctypes.data_as(_dp), drot.ctypes.data_as(_dp), st, None, nthreads, niter)
    elif kind == "RefractiveInterface":
        m2 = iface.inMedium if reverse else iface.outMedium
        L.ora_refract(s, dr.ctypes.data_as(_dp), drot.ctypes.data_as(_dp), medium(m2, keep), st, None, nthreads,
                      niter)
    else:
        L.ora_intersect(s, dr.ctypes.data_as(_dp), drot.ctypes.data_as(_dp), st, None, nthreads, niter)
    rays.origin = np.array(cs.origin, dtype=float)
    rays.rot = np.array(cs.rot, dtype=float)
    if iface.obscuration is not None:
        L.ora_obscure(obscuration(iface.obscuration, keep), st, nthreads)
    return rays


def interfaces(optic, reverse=False):
    """Non-skipped interfaces of an optic tree in trace order."""
    if hasattr(optic, "items"):
        out = []
        for item in (optic.items if not reverse else reversed(optic.items)):
            if item.skip:
                continue
            out.extend(interfaces(item, reverse))
        return out
    return [optic]


def trace(optic, rays, reverse=False, niter=5, nthreads=None, full=False):
    """CompoundOptic.trace / traceFull of the reference on host rays."""
    outs = []
    for it in interfaces(optic, reverse):
        interface_trace(it, rays, reverse, niter, nthreads)
        if full:
            outs.append((it.name, rays.copy()))
    return outs if full else rays


def sum_amplitude(rays, r, t, ignore_vignetted=True, nthreads=None):
    out = np.zeros(2)
    st = rays.struct()
    lib().ora_sum_amplitude(st, float(r[0]), float(r[1]), float(r[2]), float(t), 1 if ignore_vignetted else 0,
                            nthreads or threads(), out.ctypes.data_as(_dp))
    return complex(out[0], out[1])


def sag(surf, x, y):
    keep = []
    s = surface(surf, keep)
    x = np.ascontiguousarray(x, dtype=float)
    y = np.ascontiguousarray(y, dtype=float)
    out = np.empty_like(x)
    lib().ora_sag_array(s, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp), out.ctypes.data_as(_dp), x.size)
    return out


def normal(surf, x, y):
    keep = []
    s = surface(surf, keep)
    x = np.ascontiguousarray(x, dtype=float)
    y = np.ascontiguousarray(y, dtype=float)
    out = np.empty(3 * x.size)
    lib().ora_normal_array(s, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp), out.ctypes.data_as(_dp), x.size)
    return out.reshape(3, x.size).T


def getN(m, w):
    keep = []
    return lib().ora_getN(medium(m, keep), float(w))


def contains(ob, x, y):
    keep = []
    o = obscuration(ob, keep)
    return np.array([bool(lib().ora_contains(o, float(a), float(b))) for a, b in zip(np.ravel(x), np.ravel(y))])
