"""CUDA path vs the Zemax golden traces of the reference's tests and vs the
reference's own traces of the same rays (LSST and HSC, from their YAML
prescriptions)."""
import numpy as np
import pytest

import batoid_gb300 as bt
from _helpers import golden, assert_rays_match, FIELDS
from _zemax import optic, check_lsst, check_hsc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [0, 1, 2])
def test_lsst_zemax(k):
    g = golden("zemax")
    tel = optic("lsst")
    Hx, Hy, Px, Py = g[f"lsst{k}_hp"]
    ray = bt.RayVector.fromStop(Px * 4.18, Py * 4.18, optic=tel, wavelength=500e-9,
                                theta_x=np.deg2rad(Hx * 1.75), theta_y=np.deg2rad(Hy * 1.75), projection='zemax')
    assert_rays_match(ray, g, f"lsst{k}_in", label="fromStop")
    tf = tel.traceFull(ray)
    assert list(tf.keys()) == list(g[f"lsst{k}_names"])
    glob_rays = []
    for name, v in tf.items():
        r = v["out"].toCoordSys(bt.CoordSys())
        assert_rays_match(r, g, f"lsst{k}_{name}", label=name)
        glob_rays.append(tuple(getattr(r, c)[0] for c in ("x", "y", "z", "vx", "vy", "vz")))
    check_lsst(glob_rays, g[f"lsst{k}_zemax"])


@pytest.mark.parametrize("k", [1, 2, 3])
def test_hsc_zemax(k):
    g = golden("zemax")
    tel = optic("hsc")
    a0 = g[f"hsc{k}_zemax"][0]
    rv = bt.RayVector(a0[1] / 1000, a0[2] / 1000, 16.0, a0[4], a0[5], -a0[6], t=0, wavelength=750e-9)
    tf = tel.traceFull(rv)
    by_name = {}
    for name, v in tf.items():
        r = v["out"].toCoordSys(bt.CoordSys())
        assert_rays_match(r, g, f"hsc{k}_{name}", label=name)
        by_name[name] = tuple(getattr(r, c)[0] for c in ("x", "y", "z", "vx", "vy", "vz"))
    check_hsc(by_name, g[f"hsc{k}_zemax"])
