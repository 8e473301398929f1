"""Wavefront, Huygens PSF and Zernike fit (batoid/analysis.py).

huygensPSF evaluates every lattice pixel in one device call (the reference
loops over pixels in Python, batoid/analysis.py:302-303).  The Zernike fit
accumulates its normal equations on the device; only the jmax x jmax solve
runs on the host.
"""
from numbers import Real

import numpy as np

from . import _device as D
from . import _lib
from .lattice import Lattice
from .rayVector import RayVector
from .utils import bilinear_fit, fieldToDirCos
from . import zpoly as _zk


def _reciprocalLatticeVectors(a1, a2, N):
    norm = 2 * np.pi / (a1[0] * a2[1] - a1[1] * a2[0]) / N
    b1 = norm * np.array([a2[1], a2[0]])
    b2 = norm * np.array([a1[1], a1[0]])
    return b1, b2


def dkdu(optic, theta_x, theta_y, wavelength, nrad=6, naz=36, projection='postel'):
    """Jacobian d(kx, ky)/d(pupil u) from a bilinear fit (batoid/analysis.py:17-56)."""
    rays = RayVector.asPolar(optic=optic, theta_x=theta_x, theta_y=theta_y, wavelength=wavelength,
                             projection=projection, nrad=nrad, naz=naz)
    ux = rays.x.copy()
    uy = rays.y.copy()
    optic.trace(rays)
    w = ~rays.vignetted
    k = rays.k
    soln = bilinear_fit(ux[w], uy[w], k[w, 0], k[w, 1])
    return soln[1:]


def _chief_index(nx):
    return (nx // 2) * nx + nx // 2 if (nx % 2) == 0 else (nx * nx - 1) // 2


def huygensPSF(optic, theta_x, theta_y, wavelength, projection='postel', nx=None, dx=None, dy=None,
               nxOut=None, reference='chief'):
    """PSF by the Huygens construction |sum_u exp(i phi_u)|^2 on a lattice
    (batoid/analysis.py:181-305)."""
    if dx is None:
        d = optic.pupilSize / (nx - 2) if (nx % 2) == 0 else optic.pupilSize / (nx - 1)
        primitiveU = np.array([[d, 0], [0, d]])
        primitiveK = dkdu(optic, theta_x, theta_y, wavelength, projection=projection).dot(primitiveU)
        pad_factor = 2
        primitiveX = np.vstack(_reciprocalLatticeVectors(primitiveK[0], primitiveK[1], pad_factor * nx))
    elif isinstance(dx, Real):
        if dy is None:
            dy = dx
        primitiveX = np.vstack([[dx, 0], [0, dy]])
        pad_factor = 1
    else:
        primitiveX = np.vstack([dx, dy])
        pad_factor = 1
    if nxOut is None:
        nxOut = nx
    dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    rays = RayVector.asGrid(optic=optic, wavelength=wavelength, dirCos=dirCos, nx=nx)
    optic.trace(rays)
    N = nxOut * pad_factor
    if reference == 'mean':
        w = np.where(1 - rays.vignetted)[0]
        point = np.mean(rays.r[w], axis=0)
    else:
        point = rays.r[_chief_index(nx)]
    time = float(rays.t[0])
    re, im = huygens_amplitudes(rays, (point[0], point[1], 0.0), primitiveX, N, N, time)
    out = Lattice(np.zeros((N, N)), primitiveX)
    out.array = re * re + im * im
    return out


def huygens_amplitudes(rays, point, primitiveX, na, nb, t0, ignoreVignetted=True):
    """Complex amplitudes at P(a, b) = point + (b - nb//2) p0 + (a - na//2) p1,
    arrays of shape (na, nb) -- the reference's per-pixel sumAmplitude."""
    lat = np.ascontiguousarray([primitiveX[0][0], primitiveX[0][1], primitiveX[1][0], primitiveX[1][1]],
                               dtype=float)
    re = D.empty(na * nb)
    im = D.empty(na * nb)
    r = rays._rv
    _lib.check(_lib.lib().bt_huygens_amplitudes(
        r, float(point[0]), float(point[1]), float(point[2]), lat.ctypes.data_as(_lib.c_double_p),
        int(na), int(nb), float(t0), 1 if ignoreVignetted else 0, D.ptr(re), D.ptr(im), D.stream_ptr()))
    return D.to_host(re).reshape(na, nb), D.to_host(im).reshape(na, nb)


def wavefront(optic, theta_x, theta_y, wavelength, projection='postel', nx=32, sphereRadius=None,
              reference='chief'):
    """OPD in waves on the exit-pupil reference sphere (batoid/analysis.py:308-388)."""
    from .surface import Sphere
    dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    rays = RayVector.asGrid(optic=optic, wavelength=wavelength, nx=nx, dirCos=dirCos)
    if sphereRadius is None:
        sphereRadius = optic.sphereRadius
    optic.trace(rays)
    cridx = _chief_index(nx)
    if reference == 'mean':
        w = np.where(1 - rays.vignetted)[0]
        point = np.mean(rays.r[w], axis=0)
    else:
        point = rays.r[cridx]
    target = rays.coordSys.shiftLocal(point + np.array([0, 0, sphereRadius]))
    rays.toCoordSys(target)
    Sphere(-sphereRadius).intersect(rays)
    t = rays.t
    vig = rays.vignetted
    if reference == 'mean':
        t0 = np.mean(t[~vig])
    else:
        t0 = t[cridx]
    arr = np.ma.masked_array((t0 - t) / wavelength, mask=vig).reshape(nx, nx)
    d = optic.pupilSize / (nx - 2) if (nx % 2) == 0 else optic.pupilSize / (nx - 1)
    return Lattice(arr, np.vstack([[d, 0], [0, d]]))


def zernike(optic, theta_x, theta_y, wavelength, projection='postel', nx=32, sphereRadius=None,
            reference='chief', jmax=22, eps=0.0, include_vignetted=False):
    """Zernike coefficients (waves, Noll, index 0 unused) of the wavefront
    (batoid/analysis.py:479-573)."""
    dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    rays = RayVector.asGrid(optic=optic, wavelength=wavelength, nx=nx, dirCos=dirCos)
    epRays = rays.toCoordSys(optic.stopSurface.coordSys)
    optic.stopSurface.surface.intersect(epRays)
    orig_x = epRays.x.reshape(nx, nx)
    orig_y = epRays.y.reshape(nx, nx)
    wf = wavefront(optic, theta_x, theta_y, wavelength, nx=nx, projection=projection,
                   sphereRadius=sphereRadius, reference=reference)
    wfarr = wf.array
    if include_vignetted:
        w = np.hypot(wf.coords[..., 0], wf.coords[..., 1]) <= optic.pupilSize / 2
    else:
        w = ~wfarr.mask
    return fit_zernike(orig_x[w], orig_y[w], np.asarray(wfarr[w]), jmax, optic.pupilSize / 2,
                       optic.pupilSize / 2 * eps)


def fit_zernike(x, y, values, jmax, R_outer, R_inner):
    """Least-squares annular Zernike fit; returns jmax+1 coefficients with
    entry 0 = 0.  The normal equations B^T B and B^T v are accumulated on the
    device in FP64; RuntimeError when the system has rank < jmax
    (batoid/analysis.py:563-573)."""
    basis = _zk.basis_xy(jmax, R_outer, R_inner)
    G, b = normal_equations(x, y, values, basis)
    coefs = np.zeros(jmax + 1)
    # rank test as numpy.linalg.lstsq would see the basis: singular values of
    # B from the eigenvalues of B^T B
    ev, V = np.linalg.eigh(G)
    smax = np.sqrt(max(ev.max(), 0.0))
    tol = smax * max(len(x), jmax) * np.finfo(float).eps
    rank = int(np.sum(np.sqrt(np.clip(ev, 0.0, None)) > tol))
    if rank < jmax:
        raise RuntimeError(f"Rank {rank} matrix found when fitting {jmax} Zernike coefficients.  ")
    coefs[1:] = np.linalg.solve(G, b)
    return coefs


def normal_equations(x, y, values, basis):
    """(B^T B, B^T v) for the Cartesian-polynomial basis over the points."""
    from . import _fit
    return _fit.normal_equations(x, y, values, basis)
