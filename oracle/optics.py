"""ORACLE — test infrastructure only.

Plain optic description objects for the oracle, independent of the product
package: the same constructor names and attribute names as the reference's
Python classes (batoid/surface.py, batoid/medium.py, batoid/obscuration.py,
batoid/optic.py, batoid/coordSys.py), holding only what oracle.py reads.
The workload builders take a module argument (``build(bt)``), so passing
this module builds an optic the oracle can trace without loading the CUDA
library: ``workloads()`` loads the builders and the Zernike polynomial
module by file path for that reason.

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module.
"""
import importlib.util
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(os.path.dirname(HERE), "batoid_gb300")


def _load(name):
    spec = importlib.util.spec_from_file_location(f"_oracle_{name}", os.path.join(PKG, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


_mods = {}


def _module(name):
    if name not in _mods:
        _mods[name] = _load(name)
    return _mods[name]


def workloads():
    """The benchmark workload builders (pure numpy), without the package."""
    return _module("workloads")


# --- coordinate systems (batoid/coordSys.py) --------------------------------

class CoordSys:
    def __init__(self, origin=None, rot=None):
        self.origin = np.zeros(3) if origin is None else np.array(origin, dtype=float)
        self.rot = np.eye(3) if rot is None else np.array(rot, dtype=float)


# --- surfaces (batoid/surface.py) -------------------------------------------

class Plane:
    pass


class Tilted:
    def __init__(self, tanx, tany):
        self.tanx, self.tany = tanx, tany


class Sphere:
    def __init__(self, R):
        self.R = R


class Paraboloid:
    def __init__(self, R):
        self.R = R


class Quadric:
    def __init__(self, R, conic):
        self.R, self.conic = R, conic


class Asphere:
    """coefs alpha_i of r^(2i) from i = imin (r^4 for the default imin 2)."""

    def __init__(self, R, conic, coefs, imin=2):
        self.R, self.conic = R, conic
        self._padded_coefs = np.concatenate([np.zeros(imin - 1), np.asarray(coefs, dtype=float)])


class PolynomialSurface:
    def __init__(self, coefs, gradx, grady, xorigin=0.0, yorigin=0.0):
        self._xycoef = np.ascontiguousarray(coefs, dtype=float)
        self._xycoef_gradx = np.ascontiguousarray(gradx, dtype=float)
        self._xycoef_grady = np.ascontiguousarray(grady, dtype=float)
        self.x_origin, self.y_origin = xorigin, yorigin


class Zernike(PolynomialSurface):
    """Noll annular Zernike sum as the Cartesian arrays the product builds
    (batoid_gb300/zpoly.py, pinned to Zemax's decomposition by the tests)."""

    def __init__(self, coef, R_outer=1.0, R_inner=0.0, x_origin=0.0, y_origin=0.0):
        zk = _module("zpoly")
        C = zk.zernike_xy(np.asarray(coef, dtype=float), float(R_outer), float(R_inner))
        gx, gy = zk.grad_xy(C)
        PolynomialSurface.__init__(self, C, gx, gy, x_origin, y_origin)


class Sum:
    """Sum(s1, s2, ...) or Sum([s1, s2, ...]), as the reference accepts."""

    def __init__(self, *args):
        if len(args) == 1 and isinstance(args[0], (list, tuple)):
            args = args[0]
        self.surfaces = list(args)


# --- media (batoid/medium.py) -----------------------------------------------

class ConstMedium:
    def __init__(self, n):
        self.n = n


class SellmeierMedium:
    def __init__(self, *coefs):
        self.coefs = coefs[0] if len(coefs) == 1 else coefs


# --- obscurations (batoid/obscuration.py) -----------------------------------

class ObscCircle:
    def __init__(self, radius, x=0.0, y=0.0):
        self.radius, self.x, self.y = radius, x, y


class ObscAnnulus:
    def __init__(self, inner, outer, x=0.0, y=0.0):
        self.inner, self.outer, self.x, self.y = inner, outer, x, y


class ObscNegation:
    def __init__(self, original):
        self.original = original


# --- optics (batoid/optic.py) -----------------------------------------------

class Interface:
    def __init__(self, surface, obscuration=None, name=None, coordSys=None, inMedium=None, outMedium=None,
                 skip=False, **kwargs):
        self.surface = surface
        self.obscuration = obscuration
        self.name = name
        self.coordSys = coordSys or CoordSys()
        self.inMedium = inMedium or ConstMedium(1.0)
        self.outMedium = outMedium or ConstMedium(1.0)
        self.skip = skip


class Mirror(Interface):
    pass


class RefractiveInterface(Interface):
    pass


class Detector(Interface):
    pass


class CompoundOptic:
    def __init__(self, items, name=None, coordSys=None, inMedium=None, outMedium=None, skip=False, **kwargs):
        self.items = list(items)
        self.name = name
        self.coordSys = coordSys or CoordSys()
        self.inMedium = inMedium or ConstMedium(1.0)
        self.outMedium = outMedium or ConstMedium(1.0)
        self.skip = skip
        for k, v in kwargs.items():
            setattr(self, k, v)


class Lens(CompoundOptic):
    def __init__(self, items, medium=None, **kwargs):
        CompoundOptic.__init__(self, items, **kwargs)
        self.medium = medium
