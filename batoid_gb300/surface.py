"""Surfaces (batoid/surface.py; src/{plane,tilted,sphere,paraboloid,quadric,
asphere,polynomialSurface,bicubic,table,sum}.cpp).

Each Python surface owns a C-ABI descriptor.  sag/normal evaluate on the
GPU; intersect/reflect/refract launch the fused kernel with a one-stage
program.
"""
from abc import ABC
from numbers import Integral, Real

import numpy as np

from . import _device as D
from . import _lib
from ._handle import Handle
from .trace import intersect, reflect, refract
from . import zpoly as _zk


class Surface(ABC):
    """Abstract base class of a 2-D surface z(x, y)."""

    def _sag_device(self, x, y, out):
        n = x.numel()
        _lib.check(_lib.lib().bt_surface_sag(self._surface.ptr, D.ptr(x), D.ptr(y), D.ptr(out), n,
                                             D.stream_ptr()))

    def sag(self, x, y):
        """Surface height z(x, y) (GPU evaluation; numpy in, numpy out)."""
        scalar = np.ndim(x) == 0 and np.ndim(y) == 0
        xb, yb = np.broadcast_arrays(np.asarray(x, dtype=float), np.asarray(y, dtype=float))
        dx = D.to_device(xb.ravel())
        dy = D.to_device(yb.ravel())
        out = D.empty(dx.numel())
        self._sag_device(dx, dy, out)
        res = D.to_host(out)
        if scalar:
            return float(res[0])
        return res.reshape(xb.shape)

    def normal(self, x, y):
        """Unit normal vectors, shape (n, 3) (or (3,) for scalars)."""
        scalar = np.ndim(x) == 0
        xb, yb = np.broadcast_arrays(np.asarray(x, dtype=float), np.asarray(y, dtype=float))
        dx = D.to_device(xb.ravel())
        dy = D.to_device(yb.ravel())
        n = dx.numel()
        out = D.empty(3 * n)
        _lib.check(_lib.lib().bt_surface_normal(self._surface.ptr, D.ptr(dx), D.ptr(dy), D.ptr(out), n,
                                                D.stream_ptr()))
        res = D.to_host(out).reshape(3, n).T
        if scalar:
            return res[0].copy()
        return res.reshape(xb.shape + (3,))

    def intersect(self, rv, coordSys=None, coating=None):
        return intersect(self, rv, coordSys, coating)

    def reflect(self, rv, coordSys=None, coating=None):
        return reflect(self, rv, coordSys, coating)

    def refract(self, rv, inMedium, outMedium, coordSys=None, coating=None):
        return refract(self, rv, inMedium, outMedium, coordSys, coating)

    def refractScreen(self, rv, screen, coordSys=None):
        """Rays through a phase screen on this surface (batoid/surface.py:135-150)."""
        from .trace import refractScreen
        return refractScreen(self, rv, screen, coordSys)

    def rSplit(self, rv, inMedium, outMedium, coating, coordSys=None):
        """(refracted, reflected) rays (batoid/surface.py:107-133)."""
        from .trace import rSplit
        return rSplit(self, rv, inMedium, outMedium, coating, coordSys)

    def __ne__(self, rhs):
        return not (self == rhs)

    def __add__(self, rhs):
        return Sum(self, rhs)


def _surf(fn, *args):
    return Handle(_lib.new_handle(getattr(_lib.lib(), fn), *args), "bt_surface_destroy")


class Plane(Surface):
    """z = 0."""

    def __init__(self):
        self._surface = _surf("bt_plane_create")

    def __hash__(self):
        return hash("batoid.Plane")

    def __setstate__(self, tup):
        self.__init__()

    def __getstate__(self):
        return ()

    def __eq__(self, rhs):
        return isinstance(rhs, Plane)

    def __repr__(self):
        return "Plane()"


class Tilted(Surface):
    """z = x tan(theta_x) + y tan(theta_y)."""

    def __init__(self, tanx, tany):
        self.tanx = tanx
        self.tany = tany
        self._surface = _surf("bt_tilted_create", float(tanx), float(tany))

    def __hash__(self):
        return hash(("batoid.Tilted", self.tanx, self.tany))

    def __setstate__(self, tup):
        self.__init__(*tup)

    def __getstate__(self):
        return (self.tanx, self.tany)

    def __eq__(self, rhs):
        return isinstance(rhs, Tilted) and self.tanx == rhs.tanx and self.tany == rhs.tany

    def __repr__(self):
        return f"Tilted({self.tanx}, {self.tany})"


class Paraboloid(Surface):
    """z = r^2 / (2 R)."""

    def __init__(self, R):
        self.R = R
        self._surface = _surf("bt_paraboloid_create", float(R))

    def __hash__(self):
        return hash(("batoid.Paraboloid", self.R))

    def __setstate__(self, R):
        self.__init__(R)

    def __getstate__(self):
        return self.R

    def __eq__(self, rhs):
        return isinstance(rhs, Paraboloid) and self.R == rhs.R

    def __repr__(self):
        return f"Paraboloid({self.R})"


class Sphere(Surface):
    """z = R (1 - sqrt(1 - r^2/R^2))."""

    def __init__(self, R):
        self.R = R
        self._surface = _surf("bt_sphere_create", float(R))

    def __hash__(self):
        return hash(("batoid.Sphere", self.R))

    def __setstate__(self, R):
        self.__init__(R)

    def __getstate__(self):
        return self.R

    def __eq__(self, rhs):
        return isinstance(rhs, Sphere) and self.R == rhs.R

    def __repr__(self):
        return f"Sphere({self.R})"


class Quadric(Surface):
    """Conic of revolution, z = r^2 / (R (1 + sqrt(1 - (1+k) r^2/R^2)))."""

    def __init__(self, R, conic):
        self.R = R
        self.conic = conic
        self._surface = _surf("bt_quadric_create", float(R), float(conic))

    def __hash__(self):
        return hash(("batoid.Quadric", self.R, self.conic))

    def __setstate__(self, args):
        self.__init__(*args)

    def __getstate__(self):
        return (self.R, self.conic)

    def __eq__(self, rhs):
        return isinstance(rhs, Quadric) and self.R == rhs.R and self.conic == rhs.conic

    def __repr__(self):
        return f"Quadric({self.R}, {self.conic})"


class Asphere(Surface):
    """Conic plus even polynomial sum_i alpha_i r^(2i), i from ``imin``
    (batoid/surface.py:343-430)."""

    def __init__(self, R, conic, coefs, imin=2):
        self.R = R
        self.conic = conic
        self.coefs = coefs
        self.imin = imin
        if not isinstance(imin, Integral):
            raise TypeError("imin must be an int")
        if imin <= 0:
            raise ValueError("imin must be >= 1")
        if not all(isinstance(c, Real) for c in coefs):
            raise TypeError("coefs must be a list of floats")
        padded = np.concatenate([np.zeros(imin - 1), coefs]) if imin != 1 else np.asarray(coefs, dtype=float)
        self._padded_coefs = np.ascontiguousarray(padded, dtype=float)
        a, p = _lib.dptr(self._padded_coefs)
        self._surface = _surf("bt_asphere_create", float(R), float(conic), p, len(self._padded_coefs))

    def __hash__(self):
        return hash(("batoid.Asphere", self.R, self.conic, tuple(self.coefs), self.imin))

    def __setstate__(self, args):
        self.__init__(*args)

    def __getstate__(self):
        return self.R, self.conic, self.coefs, self.imin

    def __eq__(self, rhs):
        return (isinstance(rhs, Asphere) and self.R == rhs.R and self.conic == rhs.conic
                and np.array_equal(self.coefs, rhs.coefs) and self.imin == rhs.imin)

    def __repr__(self):
        out = f"Asphere({self.R}, {self.conic}, {self.coefs!r}"
        return out + (")" if self.imin == 2 else f", imin={self.imin})")


class PolynomialSurface(Surface):
    """z = sum C[a][b] (x - x0)^a (y - y0)^b with explicit gradient arrays
    (src/polynomialSurface.cpp)."""

    def __init__(self, coefs, gradx=None, grady=None, x_origin=0.0, y_origin=0.0):
        self._xycoef = np.ascontiguousarray(coefs, dtype=float)
        if gradx is None or grady is None:
            gradx, grady = _zk.grad_xy(self._xycoef)
        self._xycoef_gradx = np.ascontiguousarray(gradx, dtype=float)
        self._xycoef_grady = np.ascontiguousarray(grady, dtype=float)
        self.x_origin = float(x_origin)
        self.y_origin = float(y_origin)
        a, pa = _lib.dptr(self._xycoef)
        b, pb = _lib.dptr(self._xycoef_gradx)
        c, pc = _lib.dptr(self._xycoef_grady)
        self._surface = _surf("bt_polynomial_create", pa, pb, pc, self.x_origin, self.y_origin,
                              self._xycoef.shape[0], self._xycoef.shape[1])

    def __eq__(self, rhs):
        return (isinstance(rhs, PolynomialSurface) and type(rhs) == type(self)
                and np.array_equal(self._xycoef, rhs._xycoef)
                and self.x_origin == rhs.x_origin and self.y_origin == rhs.y_origin)

    def __hash__(self):
        return hash(("PolynomialSurface", tuple(self._xycoef.ravel()), self.x_origin, self.y_origin))


class Zernike(PolynomialSurface):
    """Sum of annular Zernike polynomials (Noll) over (x/R_outer, y/R_outer),
    evaluated as a Cartesian polynomial (batoid/surface.py:433-518)."""

    def __init__(self, coef, R_outer=1.0, R_inner=0.0, x_origin=0.0, y_origin=0.0):
        self.coef = np.array(coef, dtype=float, order="C")
        self.R_outer = float(R_outer)
        self.R_inner = float(R_inner)
        C = _zk.zernike_xy(self.coef, self.R_outer, self.R_inner)
        gx, gy = _zk.grad_xy(C)
        PolynomialSurface.__init__(self, C, gx, gy, x_origin, y_origin)

    def __hash__(self):
        return hash(("batoid.Zernike", tuple(self.coef), self.R_outer, self.R_inner, self.x_origin,
                     self.y_origin))

    def __setstate__(self, args):
        self.__init__(*args)

    def __getstate__(self):
        return self.coef, self.R_outer, self.R_inner, self.x_origin, self.y_origin

    def __eq__(self, rhs):
        return (isinstance(rhs, Zernike) and np.array_equal(self.coef, rhs.coef)
                and self.R_outer == rhs.R_outer and self.R_inner == rhs.R_inner
                and self.x_origin == rhs.x_origin and self.y_origin == rhs.y_origin)

    def __repr__(self):
        out = f"Zernike({self.coef!r}"
        if self.R_outer != 1.0:
            out += f", R_outer={self.R_outer}"
        if self.R_inner != 0.0:
            out += f", R_inner={self.R_inner}"
        if self.x_origin != 0.0:
            out += f", x_origin={self.x_origin}"
        if self.y_origin != 0.0:
            out += f", y_origin={self.y_origin}"
        return out + ")"


class Bicubic(Surface):
    """Hermite bicubic interpolation of a uniform grid (batoid/surface.py:521-663).
    Missing derivative arrays are filled by finite differences as in the
    reference."""

    def __init__(self, xs, ys, zs, dzdxs=None, dzdys=None, d2zdxdys=None, nanpolicy='nan'):
        assert nanpolicy.upper() in ['NAN', 'ZERO']
        self._xs = np.array(xs, dtype=float, order="C")
        self._ys = np.array(ys, dtype=float, order="C")
        self._zs = np.array(zs, dtype=float, order="C")
        self._x0 = self._xs[0]
        self._y0 = self._ys[0]
        dx = self._dx = (self._xs[-1] - self._xs[0]) / (len(self._xs) - 1)
        dy = self._dy = (self._ys[-1] - self._ys[0]) / (len(self._ys) - 1)
        zsa = self._zs
        if dzdxs is None:
            dzdxs = np.empty_like(zsa)
            dzdxs[:, 1:-1] = (zsa[:, 2:] - zsa[:, :-2]) / (2 * dx)
            dzdxs[:, 0] = (zsa[:, 1] - zsa[:, 0]) / dx
            dzdxs[:, -1] = (zsa[:, -1] - zsa[:, -2]) / dx
        if dzdys is None:
            dzdys = np.empty_like(zsa)
            dzdys[1:-1, :] = (zsa[2:, :] - zsa[:-2, :]) / (2 * dy)
            dzdys[0, :] = (zsa[1, :] - zsa[0, :]) / dy
            dzdys[-1, :] = (zsa[-1, :] - zsa[-2, :]) / dy
        if d2zdxdys is None:
            d2zdxdys = np.empty_like(zsa)
            d2zdxdys[:, 1:-1] = (dzdys[:, 2:] - dzdys[:, :-2]) / (2 * dx)
            d2zdxdys[:, 0] = (dzdys[:, 1] - dzdys[:, 0]) / dx
            d2zdxdys[:, -1] = (dzdys[:, -1] - dzdys[:, -2]) / dx
        self._dzdxs = np.array(dzdxs, dtype=float, order="C")
        self._dzdys = np.array(dzdys, dtype=float, order="C")
        self._d2zdxdys = np.array(d2zdxdys, dtype=float, order="C")
        self.nanpolicy = nanpolicy
        self._build()

    def _build(self):
        ptrs = [_lib.dptr(a) for a in (self._zs, self._dzdxs, self._dzdys, self._d2zdxdys)]
        self._table = Handle(_lib.new_handle(
            _lib.lib().bt_table_create, float(self._x0), float(self._y0), float(self._dx), float(self._dy),
            ptrs[0][1], ptrs[1][1], ptrs[2][1], ptrs[3][1], len(self._xs), len(self._ys),
            1 if self.nanpolicy.upper() == 'NAN' else 0), "bt_table_destroy")
        self._surface = _surf("bt_bicubic_create", self._table.ptr)

    xs = property(lambda self: self._xs)
    ys = property(lambda self: self._ys)
    zs = property(lambda self: self._zs)
    dzdxs = property(lambda self: self._dzdxs)
    dzdys = property(lambda self: self._dzdys)
    d2zdxdys = property(lambda self: self._d2zdxdys)

    def __hash__(self):
        return hash(("Bicubic", tuple(self.xs), tuple(self.ys), tuple(self.zs.ravel()),
                     tuple(self.dzdxs.ravel()), tuple(self.dzdys.ravel()),
                     tuple(self.d2zdxdys.ravel()), self.nanpolicy))

    def __setstate__(self, args):
        (self._xs, self._ys, self._zs, self._dzdxs, self._dzdys, self._d2zdxdys, self.nanpolicy) = args
        self._x0 = self._xs[0]
        self._y0 = self._ys[0]
        self._dx = (self._xs[-1] - self._xs[0]) / (len(self._xs) - 1)
        self._dy = (self._ys[-1] - self._ys[0]) / (len(self._ys) - 1)
        self._build()

    def __getstate__(self):
        return (self.xs, self.ys, self.zs, self.dzdxs, self.dzdys, self.d2zdxdys, self.nanpolicy)

    def __eq__(self, rhs):
        return (isinstance(rhs, Bicubic) and np.array_equal(self.xs, rhs.xs)
                and np.array_equal(self.ys, rhs.ys) and np.array_equal(self.zs, rhs.zs)
                and np.array_equal(self.dzdxs, rhs.dzdxs) and np.array_equal(self.dzdys, rhs.dzdys)
                and np.array_equal(self.d2zdxdys, rhs.d2zdxdys)
                and self.nanpolicy.upper() == rhs.nanpolicy.upper())

    def __repr__(self):
        out = f"Bicubic({self.xs!r}, {self.ys!r}, {self.zs!r}, "
        out += f"{self.dzdxs!r}, {self.dzdys!r}, {self.d2zdxdys!r}"
        return out + (")" if self.nanpolicy.upper() == "NAN" else ", nanpolicy='zero')")


class Sum(Surface):
    """Sum of surfaces; intersection starts from the first surface's own
    solution (src/sum.cpp:47-56)."""

    def __init__(self, *args):
        from collections.abc import Sequence
        if len(args) == 1 and isinstance(args[0], Sequence):
            args = args[0]
        assert all(isinstance(arg, Surface) for arg in args)
        self.surfaces = tuple(args)
        arr = (_lib.c_void_p * len(self.surfaces))(*[s._surface.ptr for s in self.surfaces])
        self._surface = _surf("bt_sum_create", arr, len(self.surfaces))

    def __hash__(self):
        return hash(("batoid.Sum", tuple(self.surfaces)))

    def __setstate__(self, surfaces):
        self.__init__(surfaces)

    def __getstate__(self):
        return self.surfaces

    def __eq__(self, rhs):
        return isinstance(rhs, Sum) and self.surfaces == rhs.surfaces

    def __repr__(self):
        return f"Sum({self.surfaces})"
