"""Algorithmic work of the reference trace, for roofline accounting.

Counting convention (fixed; never tuned to the kernel): every FP64 add, sub,
mul, div and sqrt of the REFERENCE's expressions counts 1 flop (the
reference has no fused multiply-add, so a*b+c is 2), comparisons and sign
flips count 0, and Newton solves run the full ``niter`` iterations the
reference always executes (src/surface.cpp:37-47).  The kernel does less
arithmetic than this (it stops Newton at an exact fixed point, shares
square roots between sag and slope, evaluates each medium's index once per
ray), so "algorithmic flop/s" measures useful reference work per second.

Per-ray bytes of one fused trace: every ray is read once (9 doubles + 2
flags = 74 B) and written once (74 B), whatever the number of surfaces.
"""

READ_BYTES_PER_RAY = 9 * 8 + 2
WRITE_BYTES_PER_RAY = 9 * 8 + 2

TRANSFORM = 33      # src/batoid.cpp:225-233 (3 sub, 2x(9 mul + 6 add))
PROPAGATE = 7       # src/batoid.cpp:240-243
REFLECT_TAIL = 14   # src/batoid.cpp:346-353
REFRACT_TAIL = 36   # src/batoid.cpp:455-496 without getN
NEWTON_STEP = 20    # src/surface.cpp:41-45: dt (8 + 5 + 1 div) + new point (6)
NEWTON_SETUP = 8    # initial point (6) + final |sz - z| test (2)
OBSC = {"ObscCircle": 6, "ObscAnnulus": 6, "ObscRectangle": 14, "ObscRay": 14}


def _poly2d(nx, ny):
    # horner2d: per row nx (mul+add) + per row (mul+add)
    return 2 * nx * ny + 2 * ny


def sag_flops(s):
    k = type(s).__name__
    if k == "Plane":
        return 0
    if k == "Tilted":
        return 3
    if k == "Sphere":
        return 6 + 3      # r2, *Rinvsq, 1-, sqrt, 1-, *R
    if k == "Paraboloid":
        return 4
    if k == "Quadric":
        return 9
    if k == "Asphere":
        return 12 + 3 * len(s._padded_coefs)
    if k in ("Zernike", "PolynomialSurface"):
        return 2 + _poly2d(*s._xycoef.shape)
    if k == "Bicubic":
        return 8 + 4 * 20 + 20   # cell index + 4 Hermite splines of the 16 corners + 1
    if k == "Sum":
        return sum(sag_flops(c) for c in s.surfaces) + len(s.surfaces) - 1
    raise ValueError(k)


def normal_flops(s):
    k = type(s).__name__
    if k == "Plane":
        return 0
    if k == "Tilted":
        return 6
    if k == "Sphere":
        return 19
    if k == "Paraboloid":
        return 12
    if k == "Quadric":
        return 20
    if k == "Asphere":
        return 21 + 3 * len(s._padded_coefs)
    if k in ("Zernike", "PolynomialSurface"):
        nx, ny = s._xycoef.shape
        return 2 + 2 * _poly2d(max(nx - 1, 0), max(ny - 1, 0)) + 9
    if k == "Bicubic":
        return 8 + 8 * 20 + 2 * 24 + 9
    if k == "Sum":
        return sum(normal_flops(c) + 2 + 2 for c in s.surfaces) + 9
    raise ValueError(k)


def newton_flops(s, niter):
    return NEWTON_SETUP + sag_flops(s) + niter * (normal_flops(s) + NEWTON_STEP + sag_flops(s))


def intersect_flops(s, niter):
    k = type(s).__name__
    if k == "Plane":
        return 1
    if k == "Tilted":
        return 7
    if k == "Sphere":
        return 29
    if k == "Paraboloid":
        return 24
    if k == "Quadric":
        return 35
    if k == "Asphere":
        return 35 + newton_flops(s, niter)
    if k == "Sum":
        return intersect_flops(s.surfaces[0], niter) + newton_flops(s, niter)
    return newton_flops(s, niter)


def getN_flops(m):
    k = type(m).__name__
    return {"ConstMedium": 0, "SellmeierMedium": 15, "SumitaMedium": 14, "Air": 30, "TableMedium": 6}.get(k, 0)


def obsc_flops(o):
    if o is None:
        return 0
    k = type(o).__name__
    if k == "ObscNegation":
        return obsc_flops(o.original)
    if k in ("ObscUnion", "ObscIntersection"):
        return sum(obsc_flops(i) for i in o.items)
    if k == "ObscPolygon":
        return 6 * len(o.xs)
    return OBSC.get(k, 6)


def stage_flops(iface, kind, medium, niter=5):
    """FP64 flops of one interface for one ray: interaction + obscuration."""
    f = TRANSFORM + intersect_flops(iface.surface, niter) + PROPAGATE
    if kind == 1:     # reflect
        f += normal_flops(iface.surface) + REFLECT_TAIL
    elif kind == 2:   # refract
        f += normal_flops(iface.surface) + REFRACT_TAIL + getN_flops(medium)
    return f + obsc_flops(iface.obscuration)


def optic_flops_per_ray(optic, niter=5):
    """Algorithmic FP64 flops per ray of optic.trace (reference convention)."""
    return sum(stage_flops(it, kind, med, niter) for it, kind, med, _ in optic._stages())


def optic_stages(optic):
    return len(optic._stages())


def wavefront_flops_per_ray(optic, jmax, niter=5):
    """Algorithmic FP64 flops per pupil ray of one wavefront + Zernike fit
    (reference batoid/analysis.py wavefront and zernike): the optic's trace,
    the reference sphere (transform, Sphere intersection, propagation; OPD
    as a time difference, 2 flops) and the fit's projection onto the basis
    (jmax multiply-adds).  The reference solves the fit with numpy lstsq;
    only the normal-equation projection is counted, so this undercounts the
    reference's fit arithmetic."""
    return optic_flops_per_ray(optic, niter) + TRANSFORM + 29 + PROPAGATE + 2 + 2 * jmax
