"""Transformation between two coordinate systems (batoid/coordTransform.py)."""
import numpy as np

from .coordSys import CoordSys


class CoordTransform:
    """dr = R1^T (o2 - o1), drot = R1^T R2 (batoid/coordTransform.py:16-20)."""

    def __init__(self, fromSys, toSys):
        self.fromSys = fromSys
        self.toSys = toSys
        self.dr = fromSys.rot.T @ (toSys.origin - fromSys.origin)
        self.drot = fromSys.rot.T @ toSys.rot

    @property
    def identity(self):
        return not np.any(self.dr) and np.array_equal(self.drot, np.eye(3))

    def __getstate__(self):
        return self.fromSys, self.toSys

    def __setstate__(self, d):
        self.__init__(*d)

    def __eq__(self, rhs):
        if not isinstance(rhs, CoordTransform):
            return False
        return self.fromSys == rhs.fromSys and self.toSys == rhs.toSys

    def __ne__(self, rhs):
        return not (self == rhs)

    def applyForward(self, rv):
        from .trace import applyForwardTransform
        return applyForwardTransform(self, rv)

    def applyReverse(self, rv):
        from .trace import applyReverseTransform
        return applyReverseTransform(self, rv)

    def applyForwardArray(self, x, y, z):
        r = np.array([x, y, z], dtype=float, copy=True).T
        r -= self.dr
        return self.drot.T @ r.T

    def applyReverseArray(self, x, y, z):
        r = np.array([x, y, z], dtype=float, copy=True)
        r = (self.drot @ r).T
        r += self.dr
        return r.T

    def __repr__(self):
        return f"CoordTransform({self.fromSys!r}, {self.toSys!r})"

    def __hash__(self):
        return hash(("CoordTransform", self.fromSys, self.toSys))
