"""Coordinate systems (host-side 3x3 algebra; batoid/coordSys.py)."""
import numpy as np


def RotX(th):
    """Rotation matrix about the x axis by angle ``th`` (radians)."""
    s, c = np.sin(th), np.cos(th)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def RotY(th):
    """Rotation matrix about the y axis by angle ``th`` (radians)."""
    s, c = np.sin(th), np.cos(th)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def RotZ(th):
    """Rotation matrix about the z axis by angle ``th`` (radians)."""
    s, c = np.sin(th), np.cos(th)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])


class CoordSys:
    """A local frame: ``origin`` in global coordinates and ``rot`` whose
    columns are the local unit vectors expressed globally
    (batoid/coordSys.py:23-208)."""

    def __init__(self, origin=None, rot=None):
        self.origin = np.zeros(3) if origin is None else np.array(origin, dtype=float)
        self.rot = np.eye(3) if rot is None else np.array(rot, dtype=float)

    @property
    def xhat(self):
        return self.rot[:, 0]

    @property
    def yhat(self):
        return self.rot[:, 1]

    @property
    def zhat(self):
        return self.rot[:, 2]

    def shiftGlobal(self, dr):
        return CoordSys(self.origin + dr, self.rot)

    def shiftLocal(self, dr):
        return self.shiftGlobal(self.rot @ dr)

    def toGlobal(self, v):
        v = np.array(v, dtype=float)
        return (self.rot @ v.T).T + self.origin

    def toLocal(self, v):
        v = np.array(v, dtype=float, copy=True)
        v -= self.origin
        return (self.rot.T @ v.T).T

    def rotateGlobal(self, rot, rotCenter=(0, 0, 0), coordSys=None):
        if coordSys is None:
            coordSys = CoordSys()
        center = coordSys.toGlobal(rotCenter)
        return CoordSys(rot @ (self.origin - center) + center, rot @ self.rot)

    def rotateLocal(self, rot, rotCenter=(0, 0, 0), coordSys=None):
        if coordSys is None:
            coordSys = self
        center = coordSys.toGlobal(rotCenter)
        r = self.rot @ rot
        return CoordSys(r @ self.rot.T @ (self.origin - center) + center, r)

    def __getstate__(self):
        return self.origin, self.rot

    def __setstate__(self, d):
        self.origin, self.rot = d

    def __eq__(self, rhs):
        if not isinstance(rhs, CoordSys):
            return False
        return np.array_equal(self.origin, rhs.origin) and np.array_equal(self.rot, rhs.rot)

    def __ne__(self, rhs):
        return not (self == rhs)

    def __hash__(self):
        return hash(("batoid.CoordSys", tuple(self.origin.tolist()), tuple(self.rot.ravel().tolist())))

    def copy(self):
        return CoordSys(self.origin, self.rot)

    def __repr__(self):
        rotstr = np.array2string(self.rot, separator=', ').replace('\n', '')
        return f"CoordSys({self.origin!r}, array({rotstr}))"
