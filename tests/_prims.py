"""Surface / obscuration / medium sets matching tests/golden/make_golden.py."""
import numpy as np

SURFACES = ["plane", "tilted", "sphere", "sphere_neg", "paraboloid", "quadric", "quadric_obl", "asphere",
            "zernike", "bicubic", "bicubic_zero", "sum_asphere_zernike", "sum_quadric_bicubic",
            "sum_tilted_sphere"]


def make_surfaces(bt):
    rng = np.random.default_rng(31415)
    xs = np.linspace(-1.1, 1.1, 40)
    ys = np.linspace(-1.2, 1.2, 44)
    X, Y = np.meshgrid(xs, ys)
    Zt = 0.01 * np.cos(1.3 * X) * np.sin(0.9 * Y) + 0.003 * X * X
    bic = bt.Bicubic(xs, ys, Zt)
    bic0 = bt.Bicubic(xs, ys, Zt, nanpolicy='zero')
    zc = np.zeros(23)
    zc[4:] = rng.normal(0, 1e-4, 19)
    return {
        "plane": bt.Plane(),
        "tilted": bt.Tilted(0.01, -0.02),
        "sphere": bt.Sphere(5.3),
        "sphere_neg": bt.Sphere(-4.1),
        "paraboloid": bt.Paraboloid(3.7),
        "quadric": bt.Quadric(6.1, -0.7),
        "quadric_obl": bt.Quadric(-8.2, 0.4),
        "asphere": bt.Asphere(7.5, -1.1, [1e-4, -2e-5, 3e-7, -1e-8]),
        "zernike": bt.Zernike(zc, R_outer=1.3, R_inner=0.4),
        "bicubic": bic,
        "bicubic_zero": bic0,
        "sum_asphere_zernike": bt.Sum([bt.Asphere(9.0, -0.9, [2e-5, -1e-7]), bt.Zernike(zc, R_outer=1.5)]),
        "sum_quadric_bicubic": bt.Sum([bt.Quadric(8.0, -0.5), bic]),
        "sum_tilted_sphere": bt.Sum([bt.Tilted(0.005, 0.003), bt.Sphere(20.0)]),
    }


def make_obscurations(bt):
    return {
        "circle": bt.ObscCircle(0.7, 0.1, -0.2),
        "annulus": bt.ObscAnnulus(0.3, 0.9, -0.05, 0.02),
        "rectangle": bt.ObscRectangle(1.1, 0.4, 0.1, 0.2, 0.3),
        "ray": bt.ObscRay(0.2, 0.7, -0.1, 0.05),
        "polygon": bt.ObscPolygon([0.0, 1.0, 0.3, -0.8, -0.4], [-1.0, 0.2, 1.1, 0.6, -0.5]),
        "negation": bt.ObscNegation(bt.ObscCircle(0.5)),
        "union": bt.ObscUnion([bt.ObscCircle(0.3, 0.5, 0.5), bt.ObscRectangle(0.5, 2.0), bt.ObscRay(0.1, 2.0)]),
        "intersection": bt.ObscIntersection([bt.ObscCircle(1.0), bt.ObscNegation(bt.ObscCircle(0.4)),
                                             bt.ObscRectangle(1.6, 1.2, 0.0, 0.0, -0.2)]),
    }


def make_media(bt, g):
    from batoid_gb300 import workloads as W
    tw, tn = g["media_table_args"]
    return {
        "sellmeier": bt.SellmeierMedium(*W.SILICA),
        "sumita": bt.SumitaMedium(2.2705778, -0.010059376, 0.010414999, 0.00028872517, -2.2214495e-05,
                                  1.4258559e-06),
        "air": bt.Air(),
        "air2": bt.Air(pressure=60.0, temperature=280.0, h2o_pressure=0.5),
        "table": bt.TableMedium(tw, tn),
    }


def cs_from(v):
    return np.asarray(v[:3]), np.asarray(v[3:]).reshape(3, 3)
