"""Device-resident ray bundle (batoid/rayVector.py, include/rayVector.h).

The reference keeps 11 numpy arrays behind a host/device DualView
(include/dualView.h:15-44).  Here the rays live in HBM: one float64 buffer
of shape (9, N) holding x, y, z, vx, vy, vz, t, wavelength, flux as rows and
one uint8 buffer of shape (2, N) holding vignetted, failed.  Each row is a
contiguous array, so every kernel reads and writes coalesced FP64 streams.
Reading a field (``rv.x``) copies it to the host.
"""
from functools import cached_property
from numbers import Integral, Real

import numpy as np
import torch

from . import _device as D
from . import _lib
from .constants import globalCoordSys, vacuum
from .coordTransform import CoordTransform
from .utils import fieldToDirCos, hexapolar_rings

_FIELDS = ("x", "y", "z", "vx", "vy", "vz", "t", "wavelength", "flux")
_FLAGS = ("vignetted", "failed")


class RayVector:
    """Create a RayVector from 1-d arrays (copied to the device).

    Parameters follow batoid.RayVector (batoid/rayVector.py:23-80): positions
    in meters, velocities in units of the vacuum speed of light, reference
    time t (meters), vacuum wavelength (meters), flux, vignetted and failed
    flags, and the CoordSys the rays are expressed in.
    """

    def __init__(self, x, y, z, vx, vy, vz, t=0.0, wavelength=0.0, flux=1.0,
                 vignetted=False, failed=False, coordSys=globalCoordSys):
        shape = np.broadcast(x, y, z, vx, vy, vz, t, wavelength, flux, vignetted, failed).shape
        if shape == ():
            shape = (1,)
        n = int(np.prod(shape))
        dbl = np.empty((9, n), dtype=np.float64)
        for k, a in enumerate((x, y, z, vx, vy, vz, t, wavelength, flux)):
            dbl[k] = np.broadcast_to(np.asarray(a, dtype=np.float64), shape).ravel()
        flg = np.empty((2, n), dtype=np.uint8)
        for k, a in enumerate((vignetted, failed)):
            flg[k] = np.broadcast_to(np.asarray(a, dtype=bool), shape).ravel()
        self._d = D.to_device(dbl)
        self._b = D.to_device(flg, dtype=torch.uint8)
        self.coordSys = coordSys

    # -- construction from device buffers ---------------------------------
    @staticmethod
    def _fromBuffers(dbuf, bbuf, coordSys):
        ret = RayVector.__new__(RayVector)
        ret._d = dbuf
        ret._b = bbuf
        ret.coordSys = coordSys
        return ret

    @staticmethod
    def _empty(n, coordSys=globalCoordSys):
        return RayVector._fromBuffers(D.empty((9, n)), D.empty((2, n), torch.uint8), coordSys)

    @staticmethod
    def _directInit(x, y, z, vx, vy, vz, t, wavelength, flux, vignetted, failed, coordSys):
        """From device tensors or host arrays of equal length (no broadcasting)."""
        n = len(x)
        ret = RayVector._empty(n, coordSys)
        for k, a in enumerate((x, y, z, vx, vy, vz, t, wavelength, flux)):
            ret._d[k].copy_(D.to_device(a))
        for k, a in enumerate((vignetted, failed)):
            ret._b[k].copy_(D.to_device(np.asarray(a, dtype=np.uint8) if not isinstance(a, torch.Tensor)
                                        else a.to(torch.uint8), dtype=torch.uint8))
        return ret

    # -- C-ABI view ------------------------------------------------------------
    @property
    def _rv(self):
        n = self._d.shape[1]
        base = self._d.data_ptr()
        fb = self._b.data_ptr()
        s = self._d.stride(0) * 8
        bs = self._b.stride(0)
        if n == 0:
            return _lib.BtRayVector(*([None] * 11), 0)
        return _lib.BtRayVector(
            base, base + s, base + 2 * s, base + 3 * s, base + 4 * s, base + 5 * s,
            base + 6 * s, base + 7 * s, base + 8 * s, fb, fb + bs, n)

    # -- device field access -----------------------------------------------------
    def field(self, name):
        """Device tensor (view) of one field; no copy."""
        if name in _FIELDS:
            return self._d[_FIELDS.index(name)]
        return self._b[_FLAGS.index(name)]

    def _host(self, name):
        if name in _FIELDS:
            return D.to_host(self._d[_FIELDS.index(name)])
        return D.to_host(self._b[_FLAGS.index(name)]).astype(bool)

    @property
    def x(self):
        return self._host("x")

    @property
    def y(self):
        return self._host("y")

    @property
    def z(self):
        return self._host("z")

    @property
    def vx(self):
        return self._host("vx")

    @property
    def vy(self):
        return self._host("vy")

    @property
    def vz(self):
        return self._host("vz")

    @property
    def t(self):
        return self._host("t")

    @property
    def wavelength(self):
        return self._host("wavelength")

    @property
    def flux(self):
        return self._host("flux")

    @property
    def vignetted(self):
        return self._host("vignetted")

    @property
    def failed(self):
        return self._host("failed")

    @property
    def r(self):
        return D.to_host(self._d[0:3]).T.copy()

    @property
    def v(self):
        return D.to_host(self._d[3:6]).T.copy()

    @property
    def k(self):
        v = self.v
        out = 2 * np.pi * v
        out /= self.wavelength[:, None]
        out /= np.sum(v * v, axis=-1)[:, None]
        return out

    @property
    def kx(self):
        return self.k[:, 0]

    @property
    def ky(self):
        return self.k[:, 1]

    @property
    def kz(self):
        return self.k[:, 2]

    @property
    def omega(self):
        return 2 * np.pi / self.wavelength

    # -- RayVector methods (src/rayVector.cpp) ---------------------------------
    def positionAtTime(self, t):
        n = len(self)
        out = D.empty((3, n))
        rv = self._rv
        _lib.check(_lib.lib().bt_rv_position_at_time(
            rv, float(t), D.ptr(out[0]), D.ptr(out[1]), D.ptr(out[2]), 1, D.stream_ptr()))
        return D.to_host(out).T.copy()

    def propagate(self, t):
        rv = self._rv
        _lib.check(_lib.lib().bt_rv_propagate_in_place(rv, float(t), 1, D.stream_ptr()))
        return self

    def phase(self, r, t):
        out = D.empty(len(self))
        rv = self._rv
        _lib.check(_lib.lib().bt_rv_phase(rv, float(r[0]), float(r[1]), float(r[2]), float(t),
                                          D.ptr(out), 1, D.stream_ptr()))
        return D.to_host(out)

    def amplitude(self, r, t):
        out = D.empty(2 * len(self))
        rv = self._rv
        _lib.check(_lib.lib().bt_rv_amplitude(rv, float(r[0]), float(r[1]), float(r[2]), float(t),
                                              D.ptr(out), 1, D.stream_ptr()))
        return D.to_host(out).view(np.complex128)

    def sumAmplitude(self, r, t, ignoreVignetted=True):
        out = (_lib.c_double * 2)()
        rv = self._rv
        _lib.check(_lib.lib().bt_rv_sum_amplitude(
            rv, float(r[0]), float(r[1]), float(r[2]), float(t), 1 if ignoreVignetted else 0, 1,
            out, D.stream_ptr()))
        return complex(out[0], out[1])

    # -- factories (batoid/rayVector.py:220-1081) ----------------------------------
    @classmethod
    def asGrid(cls, optic=None, backDist=None, medium=None, stopSurface=None, coordSys=None,
               wavelength=None, source=None, dirCos=None, theta_x=None, theta_y=None,
               projection='postel', nx=None, ny=None, dx=None, dy=None, lx=None, ly=None,
               flux=1, nrandom=None, rng=None):
        """Rays on a parallelogram grid of the stop surface, backed up by
        ``backDist`` (batoid/rayVector.py:220-444)."""
        backDist, medium, stopSurface, coordSys, dirCos, lx = _defaults(
            optic, backDist, medium, stopSurface, coordSys, dirCos, source, theta_x, theta_y,
            projection, wavelength, lx=lx, want_lx=(nx is None or dx is None))
        if sum(a is not None for a in [nx, dx, lx]) != 2:
            raise ValueError("Exactly 2 of nx, dx, lx must be specified")
        if nx is not None and ny is None:
            ny = nx
        if dx is not None and dy is None:
            dy = dx
        if lx is not None and ly is None:
            ly = lx if isinstance(lx, Real) else np.dot(np.array([[0, -1], [1, 0]]), lx)
        if nx is not None and dx is not None:
            lx = dx * (nx - 2) if nx % 2 == 0 else dx * (nx - 1)
            ly = dy * (ny - 2) if ny % 2 == 0 else dy * (ny - 1)
        elif lx is not None and dx is not None:
            slop = 0.1
            nx = int((lx / dx + slop) // 2) * 2 + 2
            ny = int((ly / dy + slop) // 2) * 2 + 2
        if isinstance(lx, Real):
            lx = (lx, 0.0)
        if isinstance(ly, Real):
            ly = (0.0, ly)
        if nrandom is not None:
            rng = _rng(rng)
            xx = rng.uniform(-0.5, 0.5, size=nrandom)
            yy = rng.uniform(-0.5, 0.5, size=nrandom)
            stack = np.stack([xx, yy])
            x = np.dot(lx, stack)
            y = np.dot(ly, stack)
            return cls._fromStopPoints(x, y, stopSurface, coordSys, wavelength, medium, backDist,
                                       source, dirCos, flux)
        # fftshift(fftfreq(n, d)) lattice, generated on the device
        nx, ny = int(nx), int(ny)
        x_d = 1. if nx <= 2 else (nx - (2 if nx % 2 == 0 else 1)) / nx
        y_d = 1. if ny <= 2 else (ny - (2 if ny % 2 == 0 else 1)) / ny
        valx, valy = 1.0 / (nx * x_d), 1.0 / (ny * y_d)
        a_lx, p_lx = _lib.vec(lx, 2)
        a_ly, p_ly = _lib.vec(ly, 2)

        def gen(dx, dy):
            _lib.check(_lib.lib().bt_stop_points_grid(nx, ny, valx, valy, p_lx, p_ly, D.ptr(dx), D.ptr(dy),
                                                      D.stream_ptr()))
        return cls._fromStopPoints(None, None, stopSurface, coordSys, wavelength, medium, backDist,
                                   source, dirCos, flux, gen=(nx * ny, gen))

    @classmethod
    def asFan(cls, nx=None, ny=None, **kwargs):
        rvs = []
        if nx > 1:
            rvs.append(RayVector.asGrid(nx=nx, ny=1, **kwargs))
        if ny > 1:
            rvs.append(RayVector.asGrid(nx=1, ny=ny, **kwargs))
        return concatenateRayVectors(rvs)

    @classmethod
    def asPolar(cls, optic=None, backDist=None, medium=None, stopSurface=None, coordSys=None,
                wavelength=None, outer=None, inner=None, source=None, dirCos=None, theta_x=None,
                theta_y=None, projection='postel', nrad=None, naz=None, kfold=6, flux=1,
                nrandom=None, rng=None):
        """Rays on hexapolar rings (or uniform random) in an annulus of the
        stop surface (batoid/rayVector.py:460-643)."""
        if optic is not None:
            if outer is None:
                outer = optic.pupilSize / 2
            if inner is None:
                inner = (optic.pupilSize * optic.pupilObscuration / 2
                         if hasattr(optic, 'pupilObscuration') else 0.0)
        elif inner is None:
            inner = 0.0
        backDist, medium, stopSurface, coordSys, dirCos, _ = _defaults(
            optic, backDist, medium, stopSurface, coordSys, dirCos, source, theta_x, theta_y,
            projection, wavelength, strict_stop=True)
        if nrandom is not None:
            rng = _rng(rng)
            rr = np.sqrt(rng.uniform(inner ** 2, outer ** 2, size=nrandom))
            th = rng.uniform(0, 2 * np.pi, size=nrandom)
            return cls._fromStopPoints(rr * np.cos(th), rr * np.sin(th), stopSurface, coordSys, wavelength,
                                       medium, backDist, source, dirCos, flux)
        # hexapolar rings (batoid/utils.py:512-535), points generated on the device
        r_tab, step, off = hexapolar_rings(outer=outer, inner=inner, nrad=nrad, naz=naz, kfold=kfold)
        d_r, d_step, d_off = D.to_device(r_tab), D.to_device(step), torch.from_numpy(off).to(D.device())

        def gen(dx, dy):
            _lib.check(_lib.lib().bt_stop_points_rings(len(r_tab), D.ptr(d_r), D.ptr(d_step), D.ptr(d_off),
                                                       int(off[-1]), D.ptr(dx), D.ptr(dy), D.stream_ptr()))
        return cls._fromStopPoints(None, None, stopSurface, coordSys, wavelength, medium, backDist,
                                   source, dirCos, flux, gen=(int(off[-1]), gen))

    @classmethod
    def asSpokes(cls, optic=None, backDist=None, medium=None, stopSurface=None, coordSys=None,
                 wavelength=None, outer=None, inner=0.0, source=None, dirCos=None, theta_x=None,
                 theta_y=None, projection='postel', spokes=None, rings=None, spacing='uniform',
                 flux=1):
        """Rays on spokes x rings of the stop surface (batoid/rayVector.py:646-814)."""
        if optic is not None and outer is None:
            outer = optic.pupilSize / 2
        backDist, medium, stopSurface, coordSys, dirCos, _ = _defaults(
            optic, backDist, medium, stopSurface, coordSys, dirCos, source, theta_x, theta_y,
            projection, wavelength, strict_stop=True)
        if isinstance(rings, Integral):
            if spacing == 'uniform':
                rings = np.linspace(inner, outer, rings)
            elif spacing == 'GQ':
                if spokes is None:
                    spokes = 2 * rings + 1
                Li, w = np.polynomial.legendre.leggauss(rings)
                eps = inner / outer
                area = np.pi * (1 - eps ** 2)
                rings = np.sqrt(eps ** 2 + (1 + Li) * (1 - eps ** 2) / 2) * outer
                flux = w * area / (2 * spokes)
            if isinstance(spokes, Integral):
                spokes = np.linspace(0, 2 * np.pi, spokes, endpoint=False)
        # meshgrid(rings, spokes) raveled: point i on ring i % nr of spoke i / nr
        rings = np.ascontiguousarray(np.atleast_1d(rings), dtype=float).ravel()
        spokes = np.ascontiguousarray(np.atleast_1d(spokes), dtype=float).ravel()
        nr, ns = len(rings), len(spokes)
        flux = np.broadcast_to(flux, (ns, nr)).ravel()
        d_rings, d_spokes = D.to_device(rings), D.to_device(spokes)

        def gen(dx, dy):
            _lib.check(_lib.lib().bt_stop_points_spokes(D.ptr(d_rings), nr, D.ptr(d_spokes), ns, D.ptr(dx),
                                                        D.ptr(dy), D.stream_ptr()))
        return cls._fromStopPoints(None, None, stopSurface, coordSys, wavelength, medium, backDist,
                                   source, dirCos, flux, gen=(nr * ns, gen))

    @classmethod
    def fromStop(cls, x, y, optic=None, backDist=None, medium=None, stopSurface=None,
                 coordSys=None, wavelength=None, source=None, dirCos=None, theta_x=None,
                 theta_y=None, projection='postel', flux=1):
        """Rays through given stop-surface points (batoid/rayVector.py:861-982)."""
        backDist, medium, stopSurface, coordSys, dirCos, _ = _defaults(
            optic, backDist, medium, stopSurface, coordSys, dirCos, source, theta_x, theta_y,
            projection, wavelength, strict_stop=True)
        x = np.atleast_1d(x).astype(float)
        y = np.atleast_1d(y).astype(float)
        return cls._fromStopPoints(x, y, stopSurface, coordSys, wavelength, medium, backDist,
                                   source, dirCos, flux)

    @classmethod
    def fromFieldAngles(cls, theta_x, theta_y, projection='postel', optic=None, backDist=None,
                        medium=None, stopSurface=None, wavelength=None, x=0, y=0, flux=1):
        """One ray per field angle through a stop point (batoid/rayVector.py:985-1081)."""
        from .optic import Interface
        from .surface import Plane
        if optic is not None:
            backDist = optic.backDist if backDist is None else backDist
            medium = optic.inMedium if medium is None else medium
            stopSurface = optic.stopSurface if stopSurface is None else stopSurface
        backDist = 40.0 if backDist is None else backDist
        stopSurface = Interface(Plane()) if stopSurface is None else stopSurface
        medium = vacuum if medium is None else medium
        if wavelength is None:
            raise ValueError("Missing wavelength keyword")
        vx, vy, vz = fieldToDirCos(theta_x, theta_y, projection=projection)
        n = medium.getN(wavelength)
        vx = np.asarray(vx, dtype=float) / n
        vy = np.asarray(vy, dtype=float) / n
        vz = np.asarray(vz, dtype=float) / n
        z = stopSurface.surface.sag(x, y)
        rv = RayVector(np.full_like(vx, x), np.full_like(vx, y), np.full_like(vx, z), vx, vy, vz,
                       np.zeros_like(vx), wavelength, flux, coordSys=stopSurface.coordSys)
        rv.propagate(-backDist * n)
        return rv

    @classmethod
    def _fromStopPoints(cls, x, y, stopSurface, coordSys, wavelength, medium, backDist, source,
                        dirCos, flux, gen=None):
        """Common tail of the factories: stop sag, transform into ``coordSys``,
        back-propagation (batoid/rayVector.py:817-858).  The stop points are
        host arrays ``x, y`` or, with ``gen = (n, fill)``, written on the
        device by ``fill(dx, dy)``."""
        if source is not None:
            raise NotImplementedError("point sources are not implemented (the reference's "
                                      "source branch is also a no-op, batoid/rayVector.py:847-858)")
        n_rays = len(x) if gen is None else gen[0]
        ret = RayVector._empty(n_rays, coordSys)
        dx = ret._d[0]
        dy = ret._d[1]
        dz = ret._d[2]
        if gen is None:
            dx.copy_(D.to_device(x))
            dy.copy_(D.to_device(y))
        elif n_rays > 0:
            gen[1](dx, dy)
        stopSurface.surface._sag_device(dx, dy, dz)
        ct = CoordTransform(stopSurface.coordSys, coordSys)
        L = _lib.lib()
        a_dr, p_dr = _lib.vec(ct.dr, 3)
        a_rot, p_rot = _lib.vec(ct.drot, 9)
        s = D.stream_ptr()
        _lib.check(L.bt_apply_forward_transform_arrays(p_dr, p_rot, D.ptr(dx), D.ptr(dy), D.ptr(dz),
                                                        n_rays, 1, s))
        n = medium.getN(wavelength)
        vv = np.array(dirCos, dtype=float, copy=True)
        vv /= n * np.sqrt(np.dot(vv, vv))
        zhat = -n * vv
        xhat = np.cross(np.array([1.0, 0.0, 0.0]), zhat)
        xhat /= np.sqrt(np.dot(xhat, xhat))
        yhat = np.cross(xhat, zhat)
        origin = zhat * backDist
        rot = np.stack([xhat, yhat, zhat]).T
        a_o, p_o = _lib.vec(origin, 3)
        a_r, p_r = _lib.vec(rot.ravel(), 9)
        a_v, p_v = _lib.vec(vv, 3)
        _lib.check(L.bt_finish_parallel(p_o, p_r, p_v, D.ptr(dx), D.ptr(dy), D.ptr(dz), n_rays, s))
        ret._d[3].fill_(float(vv[0]))
        ret._d[4].fill_(float(vv[1]))
        ret._d[5].fill_(float(vv[2]))
        ret._d[6].zero_()
        ret._d[7].fill_(float(wavelength))
        if isinstance(flux, Real):
            ret._d[8].fill_(float(flux))
        else:
            ret._d[8].copy_(D.to_device(np.asarray(flux, dtype=float)))
        ret._b.zero_()
        return ret

    # -- misc -----------------------------------------------------------------
    def copy(self):
        return RayVector._fromBuffers(self._d.clone(), self._b.clone(), self.coordSys.copy())

    def toCoordSys(self, coordSys):
        from .trace import applyForwardTransform
        applyForwardTransform(CoordTransform(self.coordSys, coordSys), self)
        return self

    def __len__(self):
        return self._d.shape[1]

    def __eq__(self, rhs):
        if not isinstance(rhs, RayVector):
            return False
        if len(self) != len(rhs):
            return False
        out = _lib.c_int(0)
        a, b = self._rv, rhs._rv
        _lib.check(_lib.lib().bt_rv_equal(a, b, _lib.ctypes.byref(out), D.stream_ptr()))
        return bool(out.value)

    def __ne__(self, rhs):
        return not (self == rhs)

    def __repr__(self):
        out = f"RayVector({self.x!r}, {self.y!r}, {self.z!r}"
        out += f", {self.vx!r}, {self.vy!r}, {self.vz!r}"
        out += f", {self.t!r}, {self.wavelength!r}, {self.flux!r}"
        out += f", {self.vignetted!r}, {self.failed!r}, {self.coordSys!r})"
        return out

    def __getstate__(self):
        return (self.x, self.y, self.z, self.vx, self.vy, self.vz, self.t, self.wavelength,
                self.flux, self.vignetted, self.failed, self.coordSys)

    def __setstate__(self, args):
        rv = RayVector._directInit(*args)
        self._d, self._b, self.coordSys = rv._d, rv._b, rv.coordSys

    def __getitem__(self, idx):
        n = len(self)
        if isinstance(idx, Integral):
            if idx >= n or idx < -n:
                raise IndexError(f"index {idx} is out of bounds for axis 0 with size {n}")
            idx = idx % n
            idx = slice(idx, idx + 1)
        if isinstance(idx, np.ndarray) or isinstance(idx, list):
            idx = torch.as_tensor(np.asarray(idx), device=D.device())
            if idx.dtype == torch.bool:
                idx = torch.nonzero(idx).ravel()
        return RayVector._fromBuffers(self._d[:, idx].contiguous(), self._b[:, idx].contiguous(),
                                      self.coordSys)


def _rng(rng):
    if rng is None:
        return np.random.default_rng()
    if isinstance(rng, int):
        return np.random.default_rng(rng)
    return rng


def _defaults(optic, backDist, medium, stopSurface, coordSys, dirCos, source, theta_x, theta_y,
              projection, wavelength, lx=None, want_lx=False, strict_stop=False):
    from .optic import Interface
    from .surface import Plane
    if optic is not None:
        if backDist is None:
            backDist = optic.backDist
        if medium is None:
            medium = optic.inMedium
        if stopSurface is None:
            if strict_stop:
                stopSurface = optic.stopSurface
            else:
                stopSurface = getattr(optic, 'stopSurface', None)
        if lx is None and want_lx:
            lx = getattr(optic, 'pupilSize', None)
        if coordSys is None:
            coordSys = optic.coordSys
    if backDist is None:
        backDist = 40.0
    if stopSurface is None:
        stopSurface = Interface(Plane())
    if medium is None:
        medium = vacuum
    if coordSys is None:
        coordSys = globalCoordSys
    if dirCos is None and source is None:
        dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    if wavelength is None:
        raise ValueError("Missing wavelength keyword")
    return backDist, medium, stopSurface, coordSys, dirCos, lx


def concatenateRayVectors(rvs):
    d = torch.cat([rv._d for rv in rvs], dim=1)
    b = torch.cat([rv._b for rv in rvs], dim=1)
    return RayVector._fromBuffers(d, b, rvs[0].coordSys)
