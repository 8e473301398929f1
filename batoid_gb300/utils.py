"""Field-angle projections and small host utilities (batoid/utils.py).

These convert field angles to direction cosines for ray generation; they
run once per ray bundle on the host, not per ray-surface.
"""
import numpy as np


def normalized(args):
    args = np.atleast_1d(args)
    return args / np.linalg.norm(args)


def bilinear_fit(ux, uy, kx, ky):
    """Least-squares fit of (kx, ky) = c0 + c1 ux + c2 uy (batoid/utils.py:9-18)."""
    a = np.stack([np.ones_like(ux), ux, uy], axis=1)
    b = np.stack([kx, ky], axis=1)
    return np.linalg.lstsq(a, b, rcond=-1)[0]


def _radial(u, v, angle_of_rho):
    """Direction cosines for a radial projection where the polar angle from
    the -z axis is ``angle_of_rho(rho)``; rho = |(u, v)|."""
    u = np.asarray(u, dtype=float)
    v = np.asarray(v, dtype=float)
    rho = np.sqrt(u * u + v * v)
    th = angle_of_rho(rho)
    st = np.sin(th)
    with np.errstate(invalid='ignore', divide='ignore'):
        alpha = np.where(rho == 0, 0.0, u / np.where(rho == 0, 1.0, rho) * st)
        beta = np.where(rho == 0, 0.0, v / np.where(rho == 0, 1.0, rho) * st)
    gamma = np.where(rho == 0, -1.0, -np.cos(th))
    if alpha.ndim == 0:
        return float(alpha), float(beta), float(gamma)
    return alpha, beta, gamma


def gnomonicToDirCos(u, v):
    gamma = 1 / np.sqrt(1.0 + u * u + v * v)
    return u * gamma, v * gamma, -gamma


def dirCosToGnomonic(alpha, beta, gamma):
    return -alpha / gamma, -beta / gamma


def postelToDirCos(u, v):
    """Azimuthal equidistant: polar angle = rho."""
    return _radial(u, v, lambda rho: rho)


def dirCosToPostel(alpha, beta, gamma):
    alpha, beta, gamma = (np.asarray(a, dtype=float) for a in (alpha, beta, gamma))
    rho = np.arccos(-gamma)
    s = np.sin(rho)
    with np.errstate(invalid='ignore', divide='ignore'):
        k = np.where(gamma == -1, 0.0, rho / np.where(gamma == -1, 1.0, s))
    u, v = alpha * k, beta * k
    return (float(u), float(v)) if u.ndim == 0 else (u, v)


def zemaxToDirCos(u, v):
    tu, tv = np.tan(u), np.tan(v)
    norm = np.sqrt(1 + tu * tu + tv * tv)
    return tu / norm, tv / norm, -1 / norm


def dirCosToZemax(alpha, beta, gamma):
    return np.arctan(-alpha / gamma), np.arctan(-beta / gamma)


def stereographicToDirCos(u, v):
    """Polar angle = 2 atan(rho/2)."""
    return _radial(u, v, lambda rho: 2 * np.arctan(rho / 2))


def dirCosToStereographic(alpha, beta, gamma):
    alpha, beta, gamma = (np.asarray(a, dtype=float) for a in (alpha, beta, gamma))
    th = np.arccos(-gamma)
    rho = 2 * np.tan(th / 2)
    s = np.sin(th)
    with np.errstate(invalid='ignore', divide='ignore'):
        k = np.where(gamma == -1, 0.0, rho / np.where(gamma == -1, 1.0, s))
    u, v = alpha * k, beta * k
    return (float(u), float(v)) if u.ndim == 0 else (u, v)


def orthographicToDirCos(u, v):
    rho = np.sqrt(u * u + v * v)
    return u, v, -np.cos(np.arcsin(rho))


def dirCosToOrthographic(alpha, beta, gamma):
    return alpha, beta


def lambertToDirCos(u, v):
    """Lambert azimuthal equal-area: gamma = 1 - rho^2/2."""
    u = np.asarray(u, dtype=float)
    v = np.asarray(v, dtype=float)
    rho2 = u * u + v * v
    rho = np.sqrt(rho2)
    g = (2 - rho2) / 2
    r = np.sqrt(1 - g * g)
    with np.errstate(invalid='ignore', divide='ignore'):
        k = np.where(rho2 == 0, 0.0, r / np.where(rho2 == 0, 1.0, rho))
    alpha, beta = u * k, v * k
    gamma = np.where(rho2 == 0, -1.0, -g)
    if alpha.ndim == 0:
        return float(alpha), float(beta), float(gamma)
    return alpha, beta, gamma


def dirCosToLambert(alpha, beta, gamma):
    alpha, beta, gamma = (np.asarray(a, dtype=float) for a in (alpha, beta, gamma))
    rho = np.sqrt(2 + 2 * gamma)
    norm = np.sqrt(1 - gamma * gamma)
    with np.errstate(invalid='ignore', divide='ignore'):
        k = np.where(gamma == -1, 0.0, rho / np.where(gamma == -1, 1.0, norm))
    u, v = alpha * k, beta * k
    return (float(u), float(v)) if u.ndim == 0 else (u, v)


_TO = {
    'postel': postelToDirCos, 'zemax': zemaxToDirCos, 'gnomonic': gnomonicToDirCos,
    'stereographic': stereographicToDirCos, 'lambert': lambertToDirCos,
    'orthographic': orthographicToDirCos,
}
_FROM = {
    'postel': dirCosToPostel, 'zemax': dirCosToZemax, 'gnomonic': dirCosToGnomonic,
    'stereographic': dirCosToStereographic, 'lambert': dirCosToLambert,
    'orthographic': dirCosToOrthographic,
}


def fieldToDirCos(u, v, projection='postel'):
    """Field angle (radians) to direction cosines (batoid/utils.py:409-444)."""
    try:
        return _TO[projection](u, v)
    except KeyError:
        raise ValueError("Bad projection: {}".format(projection)) from None


def dirCosToField(alpha, beta, gamma, projection='postel'):
    try:
        return _FROM[projection](alpha, beta, gamma)
    except KeyError:
        raise ValueError("Bad projection: {}".format(projection)) from None


def _hexapolar_layout(outer, inner, nrad, naz, kfold):
    rhos = np.linspace(outer, inner, nrad)
    nphis = []
    for rho in rhos:
        nphi = int((naz * rho / outer) // kfold) * kfold
        nphis.append(nphi if nphi else kfold)
    if inner == 0.0:
        nphis[-1] = 1
    return rhos, nphis


def hexapolar_rings(outer=1.0, inner=0.0, nrad=5, naz=30, kfold=6):
    """Ring table of ``hexapolar``: radius, azimuth step and first point of
    each ring (offsets has nrad + 1 entries).  Point j of ring k sits at
    azimuth j * step[k] (numpy's linspace(0, 2 pi, n, endpoint=False))."""
    rhos, nphis = _hexapolar_layout(outer, inner, nrad, naz, kfold)
    r = np.array(rhos, dtype=float)
    if inner == 0.0:
        r[-1] = 0.0
    step = np.array([(2 * np.pi - 0.0) / k for k in nphis], dtype=float)
    off = np.concatenate([[0], np.cumsum(nphis)]).astype(np.int64)
    return r, step, off


def hexapolar(outer=1.0, inner=0.0, nrad=5, naz=30, kfold=6, rth=False):
    """Rings of points with a multiple of ``kfold`` points per ring
    (batoid/utils.py:483-535)."""
    rhos, nphis = _hexapolar_layout(outer, inner, nrad, naz, kfold)
    rr = np.concatenate([np.full(k, rho) for rho, k in zip(rhos, nphis)])
    th = np.concatenate([np.linspace(0, 2 * np.pi, k, endpoint=False) for k in nphis])
    if inner == 0.0:
        rr[-1] = 0.0
        th[-1] = 0.0
    if rth:
        return rr, th
    return rr * np.cos(th), rr * np.sin(th)
