"""The oracle (C restatement) reproduces the reference's golden vectors.

CPU only: pins oracle/oracle.c against outputs of the reference itself
(tests/golden/make_golden.py) and against the reference's own Sellmeier
known-answer table (tests/test_Medium.py:66-102 of the reference).
"""
import numpy as np
import pytest

import oracle as ora
import batoid_gb300 as bt
from batoid_gb300 import workloads as W
from _helpers import golden, assert_rays_match, ray_inputs, FIELDS

from _prims import SURFACES, make_surfaces, cs_from


def oracle_rays(arrs):
    return ora.Rays(*arrs)


def test_oracle_paraboloid_workload():
    g = golden("workloads")
    opt = W.paraboloid_optic(bt)
    rays = oracle_rays(W.paraboloid_rays(4096, seed=57721))
    np.testing.assert_array_equal(rays.x, W.paraboloid_rays(4096, seed=57721)[0])
    outs = ora.trace(opt, rays, full=True)
    for name, r in outs:
        assert_rays_match(r, g, f"paraboloid_{name}", label=name)
    assert_rays_match(rays, g, "paraboloid_final", label="final")


def test_oracle_tma_workload():
    g = golden("workloads")
    opt = W.tma_optic(bt)
    rays = oracle_rays(W.tma_rays(2048, seed=8675309))
    outs = ora.trace(opt, rays, full=True)
    assert [n for n, _ in outs] == list(g["tma_names"])
    for name, r in outs:
        assert_rays_match(r, g, f"tma_{name}", label=name)


def test_oracle_sum_amplitude():
    g = golden("workloads")
    rays = ora.Rays(*ray_inputs(g, "paraboloid_final"))
    t0 = float(g["paraboloid_amp_t0"])
    for p, want, want_all in zip(g["paraboloid_amp_points"], g["paraboloid_sumamp"],
                                 g["paraboloid_sumamp_all"]):
        got = ora.sum_amplitude(rays, p, t0)
        assert abs(got - want) <= 1e-9 * max(1.0, abs(want))
        got = ora.sum_amplitude(rays, p, t0, ignore_vignetted=False)
        assert abs(got - want_all) <= 1e-9 * max(1.0, abs(want_all))


@pytest.mark.parametrize("name", SURFACES)
def test_oracle_surface_primitives(name):
    g = golden("primitives")
    surf = make_surfaces(bt)[name]
    x, y = g[f"surf_{name}_xy"]
    np.testing.assert_allclose(ora.sag(surf, x, y), g[f"surf_{name}_sag"], rtol=0, atol=1e-14, equal_nan=True)
    np.testing.assert_allclose(ora.normal(surf, x, y), g[f"surf_{name}_normal"], rtol=0, atol=1e-14,
                               equal_nan=True)
    origin, rot = cs_from(g[f"surf_{name}_cs"])
    silica = bt.SellmeierMedium(*W.SILICA)
    vac = bt.ConstMedium(1.0)
    for op in ("intersect", "reflect", "refract", "refract_rev"):
        arrs = list(ray_inputs(g, f"surf_{name}_in"))
        if op == "refract_rev":
            for k in (3, 4, 5):
                arrs[k] = arrs[k] / 1.45
        rays = ora.Rays(*arrs)
        iface = _iface(op, surf, origin, rot, vac, silica)
        ora.interface_trace(iface, rays, reverse=(op == "refract_rev"))
        assert_rays_match(rays, g, f"surf_{name}_{op}", label=f"{name} {op}")


class _Iface:
    def __init__(self, kind, surf, cs, inM, outM):
        self.surface = surf
        self.coordSys = cs
        self.inMedium = inM
        self.outMedium = outM
        self.obscuration = None
        self.name = kind
        self._kind = kind


def _iface(op, surf, origin, rot, vac, silica):
    cs = bt.CoordSys(origin, rot)
    if op == "intersect":
        return bt.Detector(surf, coordSys=cs)
    if op == "reflect":
        return bt.Mirror(surf, coordSys=cs)
    if op == "refract":
        return bt.RefractiveInterface(surf, coordSys=cs, inMedium=vac, outMedium=silica)
    # reverse through the same interface: silica -> vacuum
    return bt.RefractiveInterface(surf, coordSys=cs, inMedium=vac, outMedium=silica)


def test_oracle_obscurations():
    g = golden("primitives")
    from _prims import make_obscurations
    pts = g["obsc_pts"]
    for k, o in make_obscurations(bt).items():
        np.testing.assert_array_equal(ora.contains(o, pts[0], pts[1]), g[f"obsc_{k}"], err_msg=k)


def test_oracle_media():
    g = golden("primitives")
    from _prims import make_media
    wl = g["media_wavelengths"]
    for k, m in make_media(bt, g).items():
        got = np.array([ora.getN(m, w) for w in wl])
        np.testing.assert_allclose(got, g[f"media_{k}"], rtol=1e-15, atol=0, equal_nan=True, err_msg=k)


def test_oracle_sellmeier_known_answers():
    """refractiveindex.info silica table at rtol 1e-13 (reference tests/test_Medium.py:94-101)."""
    g = golden("sellmeier_csv")
    silica = bt.SellmeierMedium(0.6961663, 0.4079426, 0.8974794, 0.00467914825849, 0.013512063073959999,
                                97.93400253792099)
    got = np.array([ora.getN(silica, w * 1e-6) for w in g["csv_wmicron"]])
    np.testing.assert_allclose(got, g["csv_n"], atol=0, rtol=1e-13)


@pytest.mark.parametrize("workload", ["paraboloid", "tma_corrector"])
def test_oracle_optics_builder_matches_package(workload):
    """oracle/optics.py builds the workloads without the product package (the
    reference arm of bench.py uses it); its trace equals the trace of the
    package-built optic bit for bit."""
    import optics as OO
    Wo = OO.workloads()
    build, make_rays, _ = Wo.WORKLOADS[workload]
    arrs = make_rays(3000, seed=11)
    a = ora.trace(build(OO), ora.Rays(*arrs))
    b = ora.trace(W.WORKLOADS[workload][0](bt), ora.Rays(*arrs))
    np.testing.assert_array_equal(a.d, b.d)
    np.testing.assert_array_equal(a.b, b.b)
