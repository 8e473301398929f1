"""Synthetic benchmark workloads (seeded, reproducible).

Two optics and their ray bundles:

* ``paraboloid``: f/4 paraboloid mirror, R = 8 m, 1 m diameter with a
  0.2 m radius central obscuration (clear annulus 0.2-0.5 m), reflecting onto
  a flat detector at the paraxial focus z = R/2 = 4 m, in vacuum.  Rays are
  uniform in area over the annulus on the z = 0 plane, each with its own
  field angle uniform in +-0.5 deg on both axes (postel projection), backed up
  10 m along their direction; wavelength 500 nm.  2 ray-surface operations
  per ray.
* ``tma_corrector``: 12 surfaces -- three aspheric mirrors (Sum(Asphere,
  Zernike) primary), three fused-silica lenses and a filter (8 faces:
  Sphere / Plane / Asphere / Quadric) and a flat detector.  Spacings, radii
  and clear apertures follow the LSST design (batoid/data/LSST/LSST_r.yaml),
  with the mirror conics kept in [-1.3, 0.1]: M3 has conic 0.1 instead of
  LSST's 0.155, and its r^4..r^20 terms absorb the difference (the Taylor
  series of the two conics' sags), so the mirror's shape is LSST's to
  ~1e-13 m.  Every mirror carries seeded even asphere terms r^6..r^20 with
  |a| < 1e-18 added to those design terms, and the primary a seeded Zernike
  perturbation (Noll j = 4..28, N(0, 50 nm)).  Glass is 3-term Sellmeier
  fused silica.  Rays: pupil annulus 2.558-4.18 m uniform in area, field
  uniform in a 1.75 deg radius disk, 6 wavelengths equally spaced
  350-1000 nm assigned per ray at random, backed up 15 m.  12 ray-surface
  operations per ray.

The builders take the batoid-like module to build with (``bt``) so the same
geometry can be instantiated by this package and by the reference.
"""
import numpy as np

SILICA = (0.696183020, 0.407925877, 0.897464057, 0.00467926519, 0.0135122244, 97.9323636)


def paraboloid_optic(bt):
    m1 = bt.Mirror(bt.Paraboloid(8.0), obscuration=bt.ObscNegation(bt.ObscAnnulus(0.2, 0.5)), name="M1",
                   coordSys=bt.CoordSys())
    det = bt.Detector(bt.Plane(), name="D", coordSys=bt.CoordSys(origin=[0.0, 0.0, 4.0]))
    return bt.CompoundOptic([m1, det], name="paraboloid", coordSys=bt.CoordSys())


def _postel(u, v):
    rho = np.sqrt(u * u + v * v)
    s = np.where(rho > 0, np.sin(rho) / np.where(rho > 0, rho, 1.0), 1.0)
    return u * s, v * s, -np.cos(rho)


def paraboloid_rays(n, seed=57721):
    """Host arrays (x, y, z, vx, vy, vz, t, wavelength, flux, vignetted, failed)."""
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.uniform(0.2 ** 2, 0.5 ** 2, n))
    th = rng.uniform(0.0, 2 * np.pi, n)
    fx = np.deg2rad(rng.uniform(-0.5, 0.5, n))
    fy = np.deg2rad(rng.uniform(-0.5, 0.5, n))
    vx, vy, vz = _postel(fx, fy)
    x0, y0 = r * np.cos(th), r * np.sin(th)
    back = 10.0
    x = x0 - back * vx
    y = y0 - back * vy
    z = -back * vz
    return (x, y, z, vx, vy, vz, np.zeros(n), np.full(n, 500e-9), np.ones(n), np.zeros(n, bool),
            np.zeros(n, bool))


def _conic_series(R, k, nmax=10):
    """Taylor coefficients of the conic sag r^2 / (R (1 + sqrt(1 - (1+k) r^2/R^2)))
    in r^2, r^4, ..., r^(2 nmax): sag = sum_n b_n (1+k)^(n-1) r^(2n) / R^(2n-1)
    with b_n the series coefficients of (1 - sqrt(1 - u)) / u * u."""
    b = np.zeros(nmax + 1)
    # 1 - sqrt(1-u) = sum_{n>=1} C(2n-2, n-1) / (n 2^(2n-1)) u^n
    from math import comb
    for n in range(1, nmax + 1):
        b[n] = comb(2 * n - 2, n - 1) / (n * 2 ** (2 * n - 1))
    return np.array([b[n] * (1 + k) ** (n - 1) / R ** (2 * n - 1) for n in range(1, nmax + 1)])


def _reconic(R, k_design, k_used):
    """Asphere terms r^4..r^20 that make conic k_used carry the sag of conic
    k_design (the difference of the two series; the r^2 terms agree)."""
    return list((_conic_series(R, k_design) - _conic_series(R, k_used))[1:])


def _mirror_terms(rng, design, first_seeded):
    """Asphere coefficients r^4..r^20: the design's leading terms plus seeded
    terms |a| < 1e-18 on r^6..r^20.  The terms from r^(2 first_seeded + 2) up
    are drawn first (in the order the earlier versions of this workload drew
    them, so those coefficients are unchanged), then the ones below."""
    c = np.zeros(9)
    c[:len(design)] = design
    c[first_seeded:] += rng.uniform(-1e-18, 1e-18, 9 - first_seeded)
    return c


def _low_terms(rng, c, first_seeded):
    """The seeded terms on r^6 .. r^(2 first_seeded) (index 1 .. first_seeded-1)."""
    c = np.array(c)
    c[1:first_seeded] += rng.uniform(-1e-18, 1e-18, first_seeded - 1)
    return list(c)


def tma_zernike_coefs(seed=20231):
    rng = np.random.default_rng(seed)
    coef = np.zeros(29)
    coef[4:] = rng.normal(0.0, 50e-9, 25)
    return coef


def tma_optic(bt, zernike_factory=None, seed=20231):
    """LSST-like 12-surface system.  ``zernike_factory(coef, R_outer, R_inner)``
    builds the primary's Zernike perturbation (default: bt.Zernike)."""
    rng = np.random.default_rng(seed + 1)
    CS = bt.CoordSys
    silica = bt.SellmeierMedium(*SILICA)
    vac = bt.ConstMedium(1.0)
    zfac = zernike_factory or (lambda c, ro, ri: bt.Zernike(c, R_outer=ro, R_inner=ri))
    c1 = _mirror_terms(rng, [0.0, -1.381e-9], 2)
    c2 = _mirror_terms(rng, [0.0, 1.274e-5, 9.68e-7], 3)
    c3 = _mirror_terms(rng, np.add(_reconic(8.3445, 0.155, 0.1), [0.0, 4.5e-7, 8.15e-9, 0, 0, 0, 0, 0, 0]), 3)
    c1, c2, c3 = _low_terms(rng, c1, 2), _low_terms(rng, c2, 3), _low_terms(rng, c3, 3)
    m1_surf = bt.Sum(bt.Asphere(19.835, -1.215, c1), zfac(tma_zernike_coefs(seed), 4.18, 2.558))
    z0 = np.zeros(3)

    def cs(z):
        return CS(origin=[0.0, 0.0, z])

    items = [
        bt.Mirror(m1_surf, obscuration=bt.ObscNegation(bt.ObscAnnulus(2.558, 4.18)), name="M1", coordSys=cs(0.0),
                  inMedium=vac, outMedium=vac),
        bt.Mirror(bt.Asphere(6.788, -0.222, c2),
                  obscuration=bt.ObscNegation(bt.ObscAnnulus(0.9, 1.71)), name="M2", coordSys=cs(6.1562006),
                  inMedium=vac, outMedium=vac),
        bt.Mirror(bt.Asphere(8.3445, 0.1, c3),
                  obscuration=bt.ObscNegation(bt.ObscAnnulus(0.55, 2.508)), name="M3", coordSys=cs(-0.2338),
                  inMedium=vac, outMedium=vac),
    ]
    cam = 3.3974725882045593

    def lens(name, zl, s1, s2, dz2, r):
        e = bt.RefractiveInterface(s1, obscuration=bt.ObscNegation(bt.ObscCircle(r)), name=name + "_entrance",
                                   coordSys=cs(cam + zl), inMedium=vac, outMedium=silica)
        x = bt.RefractiveInterface(s2, obscuration=bt.ObscNegation(bt.ObscCircle(r)), name=name + "_exit",
                                   coordSys=cs(cam + zl + dz2), inMedium=silica, outMedium=vac)
        return bt.Lens([e, x], name=name, coordSys=cs(cam + zl), inMedium=vac, outMedium=vac, medium=silica)

    camera = bt.CompoundOptic([
        lens("L1", 0.0, bt.Sphere(2.824), bt.Sphere(5.021), 0.08223, 0.775),
        lens("L2", 0.49487202, bt.Plane(), bt.Asphere(2.529, -1.57, [0.0, -0.001656]), 0.03, 0.551),
        lens("Filter", 0.87445202, bt.Sphere(5.632), bt.Sphere(5.606), 0.0179, 0.375),
        lens("L3", 0.94345202, bt.Quadric(3.169, -0.962), bt.Sphere(-13.36), 0.06, 0.361),
        bt.Detector(bt.Plane(), obscuration=bt.ObscNegation(bt.ObscCircle(0.4)), name="Detector",
                    coordSys=cs(cam + 1.03195202), inMedium=vac, outMedium=vac),
    ], name="Camera", coordSys=cs(cam), inMedium=vac, outMedium=vac)
    items.append(camera)
    stop = bt.Interface(bt.Plane(), name="entrancePupil", coordSys=cs(0.4393899))
    return bt.CompoundOptic(items, name="tma_corrector", coordSys=CS(), inMedium=vac, outMedium=vac,
                            backDist=15.0, sphereRadius=5.0, pupilSize=8.36, pupilObscuration=0.612,
                            stopSurface=stop)


WAVELENGTHS = np.linspace(350e-9, 1000e-9, 6)


def tma_rays(n, seed=8675309, field_radius_deg=1.75):
    """Host arrays for the 12-surface system: stop-plane annulus, field disk,
    6 wavelengths, backed up 15 m from the stop plane z = 0.4393899."""
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.uniform(2.558 ** 2, 4.18 ** 2, n))
    th = rng.uniform(0.0, 2 * np.pi, n)
    fr = np.deg2rad(field_radius_deg) * np.sqrt(rng.uniform(0.0, 1.0, n))
    fth = rng.uniform(0.0, 2 * np.pi, n)
    vx, vy, vz = _postel(fr * np.cos(fth), fr * np.sin(fth))
    w = WAVELENGTHS[rng.integers(0, 6, n)]
    back = 15.0
    zstop = 0.4393899
    x = r * np.cos(th) - back * vx
    y = r * np.sin(th) - back * vy
    z = zstop - back * vz
    return (x, y, z, vx, vy, vz, np.zeros(n), w, np.ones(n), np.zeros(n, bool), np.zeros(n, bool))


WORKLOADS = {
    "paraboloid": (paraboloid_optic, paraboloid_rays, 2),
    "tma_corrector": (tma_optic, tma_rays, 12),
}
