"""Obscurations (batoid/obscuration.py; src/obscuration.cpp).

Each Python object owns a C-ABI postfix program; compound obscurations copy
their items' programs, so items may be garbage collected independently.
"""
import numpy as np

from . import _device as D
from . import _lib
from ._handle import Handle


class Obscuration:
    def contains(self, x, y):
        """Boolean mask of points inside the obscuration (evaluated on the GPU)."""
        scalar = np.ndim(x) == 0 and np.ndim(y) == 0
        xb, yb = np.broadcast_arrays(np.asarray(x, dtype=float), np.asarray(y, dtype=float))
        dx = D.to_device(xb.ravel())
        dy = D.to_device(yb.ravel())
        out = D.empty(dx.numel(), dtype=D.torch.uint8)
        _lib.check(_lib.lib().bt_obsc_contains(self._obsc.ptr, D.ptr(dx), D.ptr(dy), D.ptr(out),
                                               dx.numel(), D.stream_ptr()))
        res = D.to_host(out).astype(bool)
        if scalar:
            return bool(res[0])
        return res.reshape(xb.shape)

    def obscure(self, rv):
        from .trace import obscure
        obscure(self, rv)

    def __ne__(self, rhs):
        return not (self == rhs)


def _h(fn, *args):
    return Handle(_lib.new_handle(getattr(_lib.lib(), fn), *args), "bt_obsc_destroy")


class ObscCircle(Obscuration):
    def __init__(self, radius, x=0.0, y=0.0):
        self.radius, self.x, self.y = radius, x, y
        self._obsc = _h("bt_obsc_circle_create", float(radius), float(x), float(y))

    def __eq__(self, rhs):
        return type(rhs) == type(self) and (self.radius, self.x, self.y) == (rhs.radius, rhs.x, rhs.y)

    def __getstate__(self):
        return self.radius, self.x, self.y

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("batoid.ObscCircle", self.radius, self.x, self.y))

    def __repr__(self):
        out = f"ObscCircle({self.radius}"
        if self.x != 0 or self.y != 0:
            out += f", {self.x}, {self.y}"
        return out + ")"


class ObscAnnulus(Obscuration):
    def __init__(self, inner, outer, x=0.0, y=0.0):
        self.inner, self.outer, self.x, self.y = inner, outer, x, y
        self._obsc = _h("bt_obsc_annulus_create", float(inner), float(outer), float(x), float(y))

    def __eq__(self, rhs):
        return (type(rhs) == type(self)
                and (self.inner, self.outer, self.x, self.y) == (rhs.inner, rhs.outer, rhs.x, rhs.y))

    def __getstate__(self):
        return self.inner, self.outer, self.x, self.y

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("batoid.ObscAnnulus", self.inner, self.outer, self.x, self.y))

    def __repr__(self):
        out = f"ObscAnnulus({self.inner}, {self.outer}"
        if self.x != 0 or self.y != 0:
            out += f", {self.x}, {self.y}"
        return out + ")"


class ObscRectangle(Obscuration):
    def __init__(self, width, height, x=0.0, y=0.0, theta=0.0):
        self.width, self.height, self.x, self.y, self.theta = width, height, x, y, theta
        self._obsc = _h("bt_obsc_rectangle_create", float(width), float(height), float(x), float(y),
                        float(theta))

    def __eq__(self, rhs):
        return type(rhs) == type(self) and self.__getstate__() == rhs.__getstate__()

    def __getstate__(self):
        return self.width, self.height, self.x, self.y, self.theta

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("batoid.ObscRectangle",) + self.__getstate__())

    def __repr__(self):
        out = f"ObscRectangle({self.width}, {self.height}"
        if self.x != 0.0 or self.y != 0.0:
            out += f", {self.x}, {self.y}"
        if self.theta != 0.0:
            out += f", theta={self.theta}"
        return out + ")"


class ObscRay(Obscuration):
    def __init__(self, width, theta, x=0.0, y=0.0):
        self.width, self.theta, self.x, self.y = width, theta, x, y
        self._obsc = _h("bt_obsc_ray_create", float(width), float(theta), float(x), float(y))

    def __eq__(self, rhs):
        return type(rhs) == type(self) and self.__getstate__() == rhs.__getstate__()

    def __getstate__(self):
        return self.width, self.theta, self.x, self.y

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("batoid.ObscRay",) + self.__getstate__())

    def __repr__(self):
        out = f"ObscRay({self.width}, {self.theta}"
        if self.x != 0.0 or self.y != 0.0:
            out += f", {self.x}, {self.y}"
        return out + ")"


class ObscPolygon(Obscuration):
    def __init__(self, xs, ys):
        self.xs = np.ascontiguousarray(xs, dtype=float)
        self.ys = np.ascontiguousarray(ys, dtype=float)
        a, pa = _lib.dptr(self.xs)
        b, pb = _lib.dptr(self.ys)
        self._obsc = _h("bt_obsc_polygon_create", pa, pb, len(self.xs))

    def __eq__(self, rhs):
        return type(rhs) == type(self) and np.all(self.xs == rhs.xs) and np.all(self.ys == rhs.ys)

    def __getstate__(self):
        return self.xs, self.ys

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("batoid.ObscPolygon", tuple(self.xs), tuple(self.ys)))

    def __repr__(self):
        return f"ObscPolygon({self.xs!r}, {self.ys!r})"

    def containsGrid(self, xgrid, ygrid):
        """contains() on the grid [ny, nx] of xgrid x ygrid."""
        xx, yy = np.meshgrid(np.asarray(xgrid, dtype=float), np.asarray(ygrid, dtype=float))
        return self.contains(xx, yy)


class ObscNegation(Obscuration):
    def __init__(self, original):
        self.original = original
        self._obsc = _h("bt_obsc_negation_create", original._obsc.ptr)

    def __eq__(self, rhs):
        return type(rhs) == type(self) and self.original == rhs.original

    def __getstate__(self):
        return self.original

    def __setstate__(self, original):
        self.__init__(original)

    def __hash__(self):
        return hash(("batoid.ObscNegation", self.original))

    def __repr__(self):
        return f"ObscNegation({self.original!r})"


def _items(items):
    if len(items) == 0:
        raise ValueError("Not enough items")
    if len(items) == 1:
        if isinstance(items[0], Obscuration):
            items = [items[0]]
        elif isinstance(items[0], (list, tuple)):
            items = items[0]
        else:
            raise TypeError("Single input argument must be an Obscuration or a list of them.")
    if not all(isinstance(item, Obscuration) for item in items):
        raise TypeError("All items must be Obscurations")
    return list(items)


class _Compound(Obscuration):
    _ctor = None
    _name = None

    def __init__(self, *items):
        items = _items(items)
        self.items = sorted(items, key=repr)
        arr = (_lib.c_void_p * len(items))(*[it._obsc.ptr for it in items])
        self._obsc = _h(self._ctor, arr, len(items))

    def __eq__(self, rhs):
        return type(rhs) == type(self) and self.items == rhs.items

    def __getstate__(self):
        return self.items

    def __setstate__(self, items):
        self.__init__(items)

    def __hash__(self):
        return hash((self._name, tuple(self.items)))

    def __repr__(self):
        return f"{type(self).__name__}(" + ", ".join(repr(i) for i in self.items) + ")"


class ObscUnion(_Compound):
    _ctor = "bt_obsc_union_create"
    _name = "batoid.ObscUnion"


class ObscIntersection(_Compound):
    _ctor = "bt_obsc_intersection_create"
    _name = "batoid.ObscIntersection"
