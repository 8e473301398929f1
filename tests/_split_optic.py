"""Shared inputs of the split-trace (ghost) tests: built with either the
reference's API or this package's (same names), so the golden generator and
the tests use identical optics and rays."""
import numpy as np

SILICA = (0.6961663, 0.4079426, 0.8974794, 0.0684043 ** 2, 0.1162414 ** 2, 9.896161 ** 2)


def split_optic(bt):
    """Two singlets and a detector; every glass surface reflects 2 %."""
    air = bt.ConstMedium(1.0)
    glass = bt.SellmeierMedium(*SILICA)
    CS = bt.CoordSys

    def lens(name, z, R1, R2, th, r):
        e = bt.RefractiveInterface(bt.Sphere(R1), obscuration=bt.ObscNegation(bt.ObscCircle(r)),
                                   name=name + "_entrance", coordSys=CS(origin=[0, 0, z]), inMedium=air,
                                   outMedium=glass)
        x = bt.RefractiveInterface(bt.Sphere(R2), obscuration=bt.ObscNegation(bt.ObscCircle(r)),
                                   name=name + "_exit", coordSys=CS(origin=[0, 0, z + th]), inMedium=glass,
                                   outMedium=air)
        for s in (e, x):
            s.forwardCoating = bt.SimpleCoating(0.02, 0.98)
            s.reverseCoating = bt.SimpleCoating(0.02, 0.98)
        return bt.Lens([e, x], name=name, coordSys=CS(origin=[0, 0, z]), inMedium=air, outMedium=air)

    det = bt.Detector(bt.Plane(), name="D", coordSys=CS(origin=[0, 0, 0.3]), inMedium=air, outMedium=air)
    return bt.CompoundOptic([lens("L1", 0.0, 0.3, -0.5, 0.01, 0.03), lens("L2", 0.1, 0.8, 0.25, 0.008, 0.03), det],
                            name="ghosts", inMedium=air, outMedium=air)


def split_rays(n=800, seed=11):
    """Host arrays: a near-collimated bundle 0.1 m before the first lens."""
    rng = np.random.default_rng(seed)
    r = 0.025 * np.sqrt(rng.uniform(0, 1, n))
    th = rng.uniform(0, 2 * np.pi, n)
    vx = np.full(n, 0.01)
    vy = np.full(n, -0.005)
    vz = np.sqrt(1 - vx ** 2 - vy ** 2)
    return (r * np.cos(th), r * np.sin(th), np.full(n, -0.1), vx, vy, vz, np.zeros(n), np.full(n, 600e-9),
            np.ones(n), np.zeros(n, bool), np.zeros(n, bool))


def rsplit_rays(n=600, seed=12, speed=1.0):
    """Host arrays for one-surface rSplit, some missing the surface; `speed`
    = 1/n of the medium the rays start in."""
    rng = np.random.default_rng(seed)
    x = rng.uniform(-0.3, 0.3, n)
    y = rng.uniform(-0.3, 0.3, n)
    vx = rng.uniform(-0.2, 0.2, n)
    vy = rng.uniform(-0.2, 0.2, n)
    vz = np.sqrt(1 - vx ** 2 - vy ** 2)
    fail = np.zeros(n, bool)
    fail[::61] = True
    return (x, y, np.full(n, -0.2), speed * vx, speed * vy, speed * vz, np.zeros(n), rng.choice([450e-9, 800e-9], n),
            rng.uniform(0.5, 1, n), np.zeros(n, bool), fail)


def rsplit_cases(bt):
    """(surface, m1, m2, coating, coordSys, ray speed) cases; the last one
    leaves glass at ~46 degrees incidence (total internal reflection)."""
    air = bt.ConstMedium(1.0)
    glass = bt.SellmeierMedium(*SILICA)
    cs = bt.CoordSys(origin=[0.01, -0.02, 0.05], rot=bt.RotX(0.03) @ bt.RotY(-0.02))
    return [
        (bt.Sphere(0.4), air, glass, bt.SimpleCoating(0.05, 0.9), cs, 1.0),
        (bt.Asphere(-0.6, -0.5, [1e-3, -2e-4]), glass, air, bt.SimpleCoating(0.1, 0.85), cs, 1 / 1.46),
        (bt.Plane(), glass, air, bt.SimpleCoating(0.04, 0.96), bt.CoordSys(rot=bt.RotX(0.8)), 1 / 1.46),
    ]


def screen_cases(bt):
    """(surface, screen, coordSys) cases for refractScreen."""
    return [
        (bt.Plane(), bt.Sphere(5000.0), bt.CoordSys(origin=[0.0, 0.0, 0.05])),
        (bt.Sphere(2.0), bt.Paraboloid(300.0), bt.CoordSys(origin=[0.01, 0.0, 0.02], rot=bt.RotY(0.05))),
    ]


def screen_optic(bt):
    """A phase screen between two planes of a two-element system."""
    CS = bt.CoordSys
    air = bt.ConstMedium(1.0)
    return bt.CompoundOptic([
        bt.OPDScreen(bt.Plane(), bt.Sphere(4000.0), name="S", coordSys=CS(origin=[0, 0, 0.1]), inMedium=air,
                     outMedium=air),
        bt.Detector(bt.Plane(), name="D", coordSys=CS(origin=[0, 0, 1.0]), inMedium=air, outMedium=air),
    ], name="screened", inMedium=air, outMedium=air)
