"""ORACLE — test infrastructure only.

CPU restatement of the reference's wavefront analysis on the C oracle trace:
RayVector.asGrid + _finish (batoid/rayVector.py:220-444, 817-858;
finishParallel src/batoid.cpp:40-69), batoid.wavefront
(batoid/analysis.py:308-388) and batoid.zernike (batoid/analysis.py:479-573),
with numpy's lstsq as the reference uses it.  The annular Zernike basis is
this project's (GalSim, which the reference calls, is not available), so the
fit's parity with GalSim is unpinned; the trace underneath is pinned.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module.
"""
import ctypes

import numpy as np

import oracle as ora


def _forward(dr, drot, x, y, z):
    """Forward transform of point arrays (src/batoid.cpp:8-38)."""
    m = np.asarray(drot, dtype=float).ravel()
    dx, dy, dz = x - dr[0], y - dr[1], z - dr[2]
    return (dx * m[0] + dy * m[3] + dz * m[6], dx * m[1] + dy * m[4] + dz * m[7],
            dx * m[2] + dy * m[5] + dz * m[8])


def as_grid(optic, wavelength, nx, dirCos):
    """RayVector.asGrid(optic=optic, wavelength, nx, dirCos) on the host."""
    stop = optic.stopSurface
    lx = optic.pupilSize
    x_d = 1. if nx <= 2 else (nx - (2 if nx % 2 == 0 else 1)) / nx
    xx = np.fft.fftshift(np.fft.fftfreq(nx, x_d))
    xx, yy = np.meshgrid(xx, xx)
    stack = np.stack([xx.ravel(), yy.ravel()])
    x = np.dot((lx, 0.0), stack)
    y = np.dot((0.0, lx), stack)
    z = ora.sag(stop.surface, x, y)
    cs = optic.coordSys
    dr, drot = ora.transform(stop.coordSys.origin, stop.coordSys.rot, cs.origin, cs.rot)
    x, y, z = _forward(dr, drot, x, y, z)
    n = optic.inMedium.getN(wavelength)
    vv = np.array(dirCos, dtype=float, copy=True)
    vv /= n * np.sqrt(np.dot(vv, vv))
    zhat = -n * vv
    xhat = np.cross(np.array([1.0, 0.0, 0.0]), zhat)
    xhat /= np.sqrt(np.dot(xhat, xhat))
    yhat = np.cross(xhat, zhat)
    origin = zhat * optic.backDist
    r = np.stack([xhat, yhat, zhat]).T.ravel()
    vxl = -vv[0] * r[0] - vv[1] * r[3] - vv[2] * r[6]
    vyl = -vv[0] * r[1] - vv[1] * r[4] - vv[2] * r[7]
    vzl = -vv[0] * r[2] - vv[1] * r[5] - vv[2] * r[8]
    lx_, ly_, lz_ = _forward(origin, r, x, y, z)
    dt = -lz_ / vzl
    lx_ = lx_ + dt * vxl
    ly_ = ly_ + dt * vyl
    lz_ = lz_ + dt * vzl
    X = lx_ * r[0] + ly_ * r[1] + lz_ * r[2] + origin[0]
    Y = lx_ * r[3] + ly_ * r[4] + lz_ * r[5] + origin[1]
    Z = lx_ * r[6] + ly_ * r[7] + lz_ * r[8] + origin[2]
    N = nx * nx
    return ora.Rays(X, Y, Z, vv[0], vv[1], vv[2], 0.0, wavelength, 1.0, np.zeros(N, bool), np.zeros(N, bool),
                    origin=cs.origin, rot=cs.rot)


def _intersect_in(rays, surface, origin, rot, niter=5):
    """Surface.intersect(rays, coordSys) with rays ending in that frame."""
    L = ora.lib()
    keep = []
    dr, drot = ora.transform(rays.origin, rays.rot, origin, rot)
    st = rays.struct()
    s = ora.surface(surface, keep)
    dp = ctypes.POINTER(ctypes.c_double)
    L.ora_intersect(s, dr.ctypes.data_as(dp), drot.ctypes.data_as(dp), st, None, ora.threads(), niter)
    rays.origin = np.array(origin, dtype=float)
    rays.rot = np.array(rot, dtype=float)
    return rays


def wavefront(optic, dirCos, wavelength, nx, sphereRadius=None):
    """batoid.wavefront(..., reference='chief'): (opd waves (nx*nx), mask)."""
    from batoid_gb300.surface import Sphere
    rays = as_grid(optic, wavelength, nx, dirCos)
    if sphereRadius is None:
        sphereRadius = optic.sphereRadius
    ora.trace(optic, rays)
    cridx = (nx // 2) * nx + nx // 2 if (nx % 2) == 0 else (nx * nx - 1) // 2
    point = np.array([rays.x[cridx], rays.y[cridx], rays.z[cridx]])
    # targetCoordSys = rays.coordSys.shiftLocal(point + (0, 0, R))
    origin = rays.origin + rays.rot @ (point + np.array([0, 0, sphereRadius]))
    rays = _intersect_in(rays, Sphere(-sphereRadius), origin, rays.rot)
    t0 = rays.t[cridx]
    return (t0 - rays.t) / wavelength, rays.vignetted


def zernike(optic, dirCos, wavelength, nx, jmax, eps, sphereRadius=None):
    """batoid.zernike(..., reference='chief', include_vignetted=False):
    coefficients 0..jmax in waves, entry 0 = 0."""
    from batoid_gb300 import zpoly
    from batoid_gb300.surface import Plane
    rays = as_grid(optic, wavelength, nx, dirCos)
    stop = optic.stopSurface
    ep = _intersect_in(rays.copy(), stop.surface if stop.surface is not None else Plane(), stop.coordSys.origin,
                       stop.coordSys.rot)
    orig_x, orig_y = ep.x.copy(), ep.y.copy()
    opd, vig = wavefront(optic, dirCos, wavelength, nx, sphereRadius)
    w = ~vig
    R_outer = optic.pupilSize / 2
    cart = zpoly.basis_xy(jmax, R_outer, R_outer * eps)
    basis = np.zeros((jmax + 1, int(w.sum())))
    for j in range(jmax):
        basis[j + 1] = zpoly.horner2d_host(orig_x[w], orig_y[w], cart[j])
    coefs, _, rank, _ = np.linalg.lstsq(basis.T, opd[w], rcond=None)
    if rank < jmax:
        raise RuntimeError(f"Rank {rank} matrix found when fitting {jmax} Zernike coefficients.  ")
    coefs[0] = 0.0
    return np.array(coefs)
