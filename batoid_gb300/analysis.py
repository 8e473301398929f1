"""Wavefront, Huygens PSF and Zernike fit (batoid/analysis.py).

huygensPSF evaluates every lattice pixel in one device call (the reference
loops over pixels in Python, batoid/analysis.py:302-303).  The Zernike fit
accumulates its normal equations on the device; only the jmax x jmax solve
runs on the host.
"""
from numbers import Real

import numpy as np
import torch

from . import _device as D
from . import _lib
from .lattice import Lattice
from .rayVector import RayVector, concatenateRayVectors
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


def _check_reference(reference):
    """The reference point is 'chief' or 'mean'; the reference fails on any
    other value (its point is never set), so an unknown one is an error."""
    if reference not in ('chief', 'mean'):
        raise ValueError(f"reference must be 'chief' or 'mean', not {reference!r}")


def _chief_index(nx):
    return (nx // 2) * nx + nx // 2 if (nx % 2) == 0 else (nx * nx - 1) // 2


def _huygens_lattice(optic, theta_x, theta_y, wavelength, projection, nx, dx, dy):
    """(primitiveX, pad_factor) of huygensPSF (batoid/analysis.py:181-305)."""
    if dx is None:
        d = optic.pupilSize / (nx - 2) if (nx % 2) == 0 else optic.pupilSize / (nx - 1)
        primitiveU = np.array([[d, 0], [0, d]])
        primitiveK = dkdu(optic, theta_x, theta_y, wavelength, projection=projection).dot(primitiveU)
        pad_factor = 2
        return np.vstack(_reciprocalLatticeVectors(primitiveK[0], primitiveK[1], pad_factor * nx)), pad_factor
    if isinstance(dx, Real):
        if dy is None:
            dy = dx
        return np.vstack([[dx, 0], [0, dy]]), 1
    return np.vstack([dx, dy]), 1


def huygensPSF(optic, theta_x, theta_y, wavelength, projection='postel', nx=None, dx=None, dy=None,
               nxOut=None, reference='chief'):
    """PSF by the Huygens construction |sum_u exp(i phi_u)|^2 on a lattice
    (batoid/analysis.py:181-305)."""
    _check_reference(reference)
    primitiveX, pad_factor = _huygens_lattice(optic, theta_x, theta_y, wavelength, projection, nx, dx, dy)
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


def huygensPSFs(optic, theta_x, theta_y, wavelength, projection='postel', nx=None, dx=None, dy=None,
                nxOut=None, reference='chief'):
    """huygensPSF for many field angles (arrays theta_x, theta_y): every
    field's pupil grid is traced in one launch, the phasor sums of all
    fields run back to back into one device buffer, and the amplitudes come
    to the host in one copy.  Element f equals huygensPSF(optic,
    theta_x[f], theta_y[f], wavelength, ...)."""
    _check_reference(reference)
    thx = np.atleast_1d(np.asarray(theta_x, dtype=float))
    thy = np.atleast_1d(np.asarray(theta_y, dtype=float))
    if thx.shape != thy.shape:
        raise ValueError("theta_x and theta_y must have the same shape")
    F = len(thx)
    if F == 0:
        return []
    if nxOut is None:
        nxOut = nx
    lattices, grids = [], []
    for f in range(F):
        lattices.append(_huygens_lattice(optic, thx[f], thy[f], wavelength, projection, nx, dx, dy))
        dirCos = fieldToDirCos(thx[f], thy[f], projection=projection)
        grids.append(RayVector.asGrid(optic=optic, wavelength=wavelength, dirCos=dirCos, nx=nx))
    rays = concatenateRayVectors(grids)
    optic.trace(rays)
    n = nx * nx
    if reference == 'mean':
        r = rays.r
        vig = rays.vignetted
        points = [np.mean(r[f * n:(f + 1) * n][~vig[f * n:(f + 1) * n]], axis=0) for f in range(F)]
    else:
        idx = torch.as_tensor([f * n + _chief_index(nx) for f in range(F)], device=D.device())
        points = list(D.to_host(rays._d[0:3, idx]).T)
    t0 = D.to_host(rays._d[6, torch.as_tensor([f * n for f in range(F)], device=D.device())])
    N = nxOut * lattices[0][1]
    pts = np.ascontiguousarray([[p[0], p[1], 0.0] for p in points], dtype=float)
    lat = np.ascontiguousarray([[pX[0][0], pX[0][1], pX[1][0], pX[1][1]] for pX, _ in lattices], dtype=float)
    t0 = np.ascontiguousarray(t0, dtype=float)
    re = D.empty(F * N * N)
    im = D.empty(F * N * N)
    _lib.check(_lib.lib().bt_huygens_amplitudes_fields(
        rays._rv, F, pts.ctypes.data_as(_lib.c_double_p), lat.ctypes.data_as(_lib.c_double_p),
        t0.ctypes.data_as(_lib.c_double_p), N, N, 1, D.ptr(re), D.ptr(im), D.stream_ptr()))
    re_h, im_h = D.to_host(re).reshape(F, N, N), D.to_host(im).reshape(F, N, N)
    out = [Lattice(re_h[f] * re_h[f] + im_h[f] * im_h[f], lattices[f][0]) for f in range(F)]
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
    _check_reference(reference)
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


# ---------------------------------------------------------------------------
# Further analyses (batoid/analysis.py:59-180, 391-476, 576-1090): the rays
# are traced on the device; the small reductions that follow run on the host
# as in the reference.
# ---------------------------------------------------------------------------

def zernikeBasis(jmax, x, y, R_outer=1.0, R_inner=0.0):
    """Annular Zernike basis values, shape (jmax+1, npoints), row 0 zero
    (the layout of galsim.zernike.zernikeBasis the reference calls)."""
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    cart = _zk.basis_xy(jmax, R_outer, R_inner)
    out = np.zeros((jmax + 1,) + x.shape)
    for j in range(jmax):
        out[j + 1] = _zk.horner2d_host(x, y, cart[j])
    return out


def _dZernikeBasis(jmax, x, y, R_outer=1.0, R_inner=0.0):
    """Gradients of the basis: array (2, jmax+1, npoints) (batoid/analysis.py:715-730)."""
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    cart = _zk.basis_xy(jmax, R_outer, R_inner)
    xout = np.zeros((jmax + 1,) + x.shape)
    yout = np.zeros_like(xout)
    for j in range(jmax):
        gx, gy = _zk.grad_xy(cart[j])
        xout[j + 1] = _zk.horner2d_host(x, y, gx)
        yout[j + 1] = _zk.horner2d_host(x, y, gy)
    return np.array([xout, yout])


def drdth(optic, theta_x, theta_y, wavelength, nrad=6, naz=36, projection='postel'):
    """Focal-plane Jacobian d(x, y)/d(theta_x, theta_y) by finite differences
    (batoid/analysis.py:59-136)."""
    from .rayVector import concatenateRayVectors
    dth = 1e-5
    nominalCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    dthxCos = fieldToDirCos(theta_x + dth, theta_y, projection=projection)
    dthyCos = fieldToDirCos(theta_x, theta_y + dth, projection=projection)
    rays = RayVector.asPolar(optic=optic, wavelength=wavelength, dirCos=nominalCos, nrad=nrad, naz=naz)
    rays_x = RayVector.asPolar(optic=optic, wavelength=wavelength, dirCos=dthxCos, nrad=nrad, naz=naz)
    rays_y = RayVector.asPolar(optic=optic, wavelength=wavelength, dirCos=dthyCos, nrad=nrad, naz=naz)
    rays_c = concatenateRayVectors([rays, rays_x, rays_y])
    optic.trace(rays_c)
    n = len(rays)
    rays, rays_x, rays_y = rays_c[:n], rays_c[n:2 * n], rays_c[2 * n:3 * n]
    w = ~rays.vignetted
    mx = np.mean(rays.x[w])
    my = np.mean(rays.y[w])
    drx_dthx = (np.mean(rays_x.x[w]) - mx) / dth
    drx_dthy = (np.mean(rays_y.x[w]) - mx) / dth
    dry_dthx = (np.mean(rays_x.y[w]) - my) / dth
    dry_dthy = (np.mean(rays_y.y[w]) - my) / dth
    return np.array([[drx_dthx, drx_dthy], [dry_dthx, dry_dthy]])


def dthdr(optic, theta_x, theta_y, wavelength, nrad=6, naz=36, projection='postel'):
    """Inverse of drdth (batoid/analysis.py:139-178)."""
    return np.linalg.inv(drdth(optic, theta_x, theta_y, wavelength, nrad=nrad, naz=naz, projection=projection))


def spot(optic, theta_x, theta_y, wavelength, projection='postel', nx=32, reference='chief'):
    """Spot diagram: focal-plane x, y of non-vignetted grid rays relative to
    the reference point (batoid/analysis.py:391-413)."""
    dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    rays = RayVector.asGrid(optic=optic, wavelength=wavelength, nx=nx, dirCos=dirCos)
    optic.trace(rays)
    if reference == 'mean':
        w = np.where(1 - rays.vignetted)[0]
        point = np.mean(rays.r[w], axis=0)
    elif reference == 'chief':
        point = rays[_chief_index(nx)].r[0]
    else:
        point = [0, 0, 0]
    targetCoordSys = rays.coordSys.shiftLocal(point)
    rays.toCoordSys(targetCoordSys)
    w = ~rays.vignetted
    return rays.x[w], rays.y[w]


def fftPSF(optic, theta_x, theta_y, wavelength, projection='postel', nx=32, pad_factor=2, sphereRadius=None,
           reference='chief'):
    """PSF as |FFT(pupil function)|^2 of the wavefront (batoid/analysis.py:416-476)."""
    wf = wavefront(optic, theta_x, theta_y, wavelength, nx=nx, projection=projection, sphereRadius=sphereRadius,
                   reference=reference)
    wfarr = wf.array
    pad_size = nx * pad_factor
    expwf = np.zeros((pad_size, pad_size), dtype=np.complex128)
    start = pad_size // 2 - nx // 2
    stop = pad_size // 2 + nx // 2
    expwf[start:stop, start:stop][~wfarr.mask] = np.exp(2j * np.pi * wfarr[~wfarr.mask])
    psf = np.abs(np.fft.fftshift(np.fft.fft2(expwf))) ** 2
    primitiveU = wf.primitiveVectors
    primitiveK = dkdu(optic, theta_x, theta_y, wavelength, projection=projection).dot(primitiveU)
    primitiveX = np.vstack(_reciprocalLatticeVectors(primitiveK[0], primitiveK[1], pad_size))
    return Lattice(psf, primitiveX)


def _chief_ray(optic, wavelength, dirCos):
    return RayVector.fromStop(0.0, 0.0, backDist=optic.backDist, wavelength=wavelength, dirCos=dirCos,
                              medium=optic.inMedium, stopSurface=optic.stopSurface)


def zernikeGQ(optic, theta_x, theta_y, wavelength, projection='postel', rings=6, spokes=None, sphereRadius=None,
              reference='chief', jmax=22, eps=0.0):
    """Zernike coefficients (waves) by Gaussian quadrature over the annulus
    (batoid/analysis.py:576-712)."""
    from .surface import Sphere
    dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    inner = eps * optic.pupilSize / 2
    rays = RayVector.asSpokes(optic=optic, wavelength=wavelength, inner=inner, dirCos=dirCos, rings=rings,
                              spokes=spokes, spacing='GQ')
    epRays = rays.copy().toCoordSys(optic.stopSurface.coordSys)
    optic.stopSurface.surface.intersect(epRays)
    basis = zernikeBasis(jmax, epRays.x, epRays.y, R_outer=optic.pupilSize / 2, R_inner=inner)
    if sphereRadius is None:
        sphereRadius = optic.sphereRadius
    optic.trace(rays)
    if np.any(rays.failed):
        raise ValueError("Cannot compute zernike with Gaussian Quadrature with failed rays.")
    if reference == 'mean':
        w = np.where(1 - rays.vignetted)[0]
        point = np.mean(rays.r[w], axis=0)
    elif reference == 'chief':
        chiefRay = _chief_ray(optic, wavelength, dirCos)
        optic.trace(chiefRay)
        point = chiefRay.r[0]
    targetCoordSys = rays.coordSys.shiftLocal(point + np.array([0, 0, sphereRadius]))
    rays.toCoordSys(targetCoordSys)
    sphere = Sphere(-sphereRadius)
    sphere.intersect(rays)
    if reference == 'mean':
        w = np.where(1 - rays.vignetted)[0]
        t0 = np.mean(rays.t[w])
    elif reference == 'chief':
        chiefRay.toCoordSys(targetCoordSys)
        sphere.intersect(chiefRay)
        t0 = chiefRay.t
    area = np.pi * (1. - eps ** 2)
    return np.dot(basis, (t0 - rays.t) / wavelength * rays.flux) / area


def zernikeTA(optic, theta_x, theta_y, wavelength, projection='postel', nrad=6, naz=36, reference='chief', jmax=22,
              eps=0.0, focal_length=None, include_vignetted=False):
    """Zernike coefficients (waves) whose wavefront gradient matches the
    transverse ray aberrations (batoid/analysis.py:732-833)."""
    dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    rays = RayVector.asPolar(optic=optic, wavelength=wavelength, dirCos=dirCos, nrad=nrad, naz=naz)
    epRays = rays.copy().toCoordSys(optic.stopSurface.coordSys)
    optic.stopSurface.surface.intersect(epRays)
    u = np.array(epRays.x)
    v = np.array(epRays.y)
    rays = optic.trace(rays)
    w = slice(None) if include_vignetted else ~rays.vignetted
    if reference == 'mean':
        point = np.mean(rays.r[w], axis=0)
    elif reference == 'chief':
        chief = RayVector.fromStop(0, 0, optic, wavelength=wavelength, dirCos=dirCos)
        optic.trace(chief)
        point = chief.r[0]
    x = rays.x - point[0]
    y = rays.y - point[1]
    if focal_length is None:
        focal_length = np.sqrt(np.linalg.det(drdth(optic, theta_x, theta_y, wavelength, projection=projection)))
    dzb = _dZernikeBasis(jmax, u[w], v[w], optic.pupilSize / 2, eps * optic.pupilSize / 2)
    a = np.hstack(dzb).T
    b = np.hstack([x[w], y[w]])
    r, _, rank, _ = np.linalg.lstsq(a, b, rcond=None)
    if rank < jmax - 1:
        raise RuntimeError(f"Rank {rank} matrix found when fitting {jmax} Zernike coefficients.  ")
    r[0] = 0.0
    return -r / focal_length / wavelength


def zernikeXYAberrations(optic, theta_x, theta_y, wavelength, projection='postel', nrad=6, naz=36,
                         reference='chief', jmax=22, eps=0.0, include_vignetted=False):
    """Zernike fits (meters) of the x and y transverse aberrations
    (batoid/analysis.py:836-925)."""
    dirCos = fieldToDirCos(theta_x, theta_y, projection=projection)
    rays = RayVector.asPolar(optic=optic, wavelength=wavelength, dirCos=dirCos, nrad=nrad, naz=naz)
    epRays = rays.copy().toCoordSys(optic.stopSurface.coordSys)
    optic.stopSurface.surface.intersect(epRays)
    u = np.array(epRays.x)
    v = np.array(epRays.y)
    rays = optic.trace(rays)
    if reference == 'mean':
        w = ~rays.vignetted
        point = np.mean(rays.r[w], axis=0)
    elif reference == 'chief':
        chief = RayVector.fromStop(0, 0, optic, wavelength=wavelength, dirCos=dirCos)
        optic.trace(chief)
        point = chief.r[0]
    x = rays.x - point[0]
    y = rays.y - point[1]
    if not include_vignetted:
        w = ~rays.vignetted
        u, v, x, y = u[w], v[w], x[w], y[w]
    basis = zernikeBasis(jmax, u, v, R_outer=optic.pupilSize / 2, R_inner=optic.pupilSize / 2 * eps)
    x_coefs, _, x_rank, _ = np.linalg.lstsq(basis.T, x, rcond=None)
    y_coefs, _, y_rank, _ = np.linalg.lstsq(basis.T, y, rcond=None)
    rank = min(x_rank, y_rank)
    if rank < jmax:
        raise RuntimeError(f"Rank {rank} matrix found when fitting {jmax} Zernike coefficients.  ")
    x_coefs[0] = 0.0
    y_coefs[0] = 0.0
    return x_coefs, y_coefs


def doubleZernike(optic, field, wavelength, rings=6, spokes=None, kmax=22, **kwargs):
    """Double Zernike coefficients (waves) over pupil and field by Gaussian
    quadrature in both (batoid/analysis.py:928-993)."""
    if spokes is None:
        spokes = 2 * rings + 1
    Li, w = np.polynomial.legendre.leggauss(rings)
    radii = np.sqrt((1 + Li) / 2) * field
    w *= np.pi / (2 * spokes)
    azs = np.linspace(0, 2 * np.pi, spokes, endpoint=False)
    radii, azs = np.meshgrid(radii, azs)
    w = np.broadcast_to(w, radii.shape)
    radii = radii.ravel()
    azs = azs.ravel()
    w = w.ravel()
    thx = radii * np.cos(azs)
    thy = radii * np.sin(azs)
    coefs = np.array([zernikeGQ(optic, thx_, thy_, wavelength, rings=rings, spokes=spokes, **kwargs)
                      for thx_, thy_ in zip(thx, thy)])
    basis = zernikeBasis(kmax, thx, thy, R_outer=field)
    return np.dot(basis, coefs * w[:, None]) / np.pi


def _closestApproach(P, u, Q, v):
    """Point on P + u t closest to the line Q + v t."""
    a = np.dot(u, u)
    b = np.dot(u, v)
    c = np.dot(v, v)
    w0 = P - Q
    d = np.dot(u, w0)
    e = np.dot(v, w0)
    den = a * c - b * b
    if den == 0:
        raise ValueError("Lines are parallel")
    sc = (b * e - c * d) / den
    return P + sc * u


def exitPupilPos(optic, wavelength, smallAngle=np.deg2rad(1. / 3600), **kwargs):
    """Exit-pupil position from small-angle chief rays' closest approach to
    the optic axis (batoid/analysis.py:1025-1065)."""
    from .constants import globalCoordSys
    thx = np.array([0, 0, smallAngle, -smallAngle])
    thy = np.array([smallAngle, -smallAngle, 0, 0])
    rays = RayVector.fromFieldAngles(thx, thy, optic=optic, wavelength=wavelength, **kwargs)
    optic.trace(rays)
    rays.toCoordSys(globalCoordSys)
    ps = [_closestApproach(ray.r[0], ray.v[0], np.array([0., 0., 0.]), np.array([0., 0., 1.0])) for ray in rays]
    return np.mean(ps, axis=0)


def focalLength(*args, **kwargs):
    """sqrt(det(drdth)) (batoid/analysis.py:1068-1090)."""
    return np.sqrt(np.linalg.det(drdth(*args, **kwargs)))
