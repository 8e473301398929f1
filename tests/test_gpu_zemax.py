"""CUDA path vs the Zemax golden traces of the reference's tests
(tests/test_zemax.py) and vs the reference's own traces of the same rays:
LSST, HSC, DECam, CBP and ComCam traces from their YAML prescriptions, the
DECam exit pupil, the LSST wavefronts and the HSC Zernike decomposition."""
import numpy as np
import pytest

import batoid_gb300 as bt
from _helpers import golden, assert_rays_match, FIELDS
from _zemax import (optic, check_lsst, check_hsc, check_decam, check_cbp, check_comcam, cbp_start, comcam_start,
                    srt)

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


def _glob(v):
    r = v["out"].toCoordSys(bt.CoordSys())
    return r, tuple(getattr(r, c)[0] for c in ("x", "y", "z", "vx", "vy", "vz"))


@pytest.mark.parametrize("k", [0, 1, 2])
def test_decam_zemax(k):
    """tests/test_zemax.py:466-520: 1e-9 against Zemax; the reference's own
    trace of the same ray at the parity tolerances."""
    g = golden("zemax_more")
    tel = optic("decam", "zemax_more")
    Hx, Hy, Px, Py = g[f"decam{k}_hp"]
    ray = bt.RayVector.fromStop(Px * 2.005, Py * 2.005, optic=tel, stopSurface=tel['PM'], wavelength=700e-9,
                                theta_x=np.deg2rad(Hx * 1.1), theta_y=np.deg2rad(Hy * 1.1), projection='zemax')
    assert_rays_match(ray, g, f"decam{k}_in", label="fromStop")
    tf = tel.traceFull(ray)
    assert list(tf.keys()) == list(g[f"decam{k}_names"])
    glob_rays = []
    for name, v in tf.items():
        r, row = _glob(v)
        assert_rays_match(r, g, f"decam{k}_{name}", label=name)
        glob_rays.append(row)
    check_decam(glob_rays, g[f"decam{k}_zemax"])


def test_decam_exit_pupil():
    """tests/test_zemax.py:522-534: 4275.016 mm in front of the focal plane
    (1 mm), and the reference's own exitPupilPos."""
    g = golden("zemax_more")
    tel = optic("decam", "zemax_more")
    tel.stopSurface = tel['PM']
    epp = np.asarray(bt.exitPupilPos(tel, wavelength=700e-9))
    np.testing.assert_allclose(epp, (0, 0, float(g["decam_D_z"]) + 4275.016 / 1e3), rtol=0, atol=1e-3)
    np.testing.assert_allclose(epp, g["decam_epp_ref"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("i", [1, 2, 3, 4])
def test_cbp_zemax(i):
    """tests/test_zemax.py:536-612: positions and directions at 1e-10."""
    g = golden("zemax_more")
    tel = optic("cbp", "zemax_more")
    x, y, z, vx, vy, vz, _, wl = cbp_start(g, i)
    ray = bt.RayVector(x + 0.1 * vx, y + 0.1 * vy, z + 0.1 * vz, vx, vy, vz, t=0, wavelength=wl)
    ray.propagate(-0.1)
    by_name = {name: _glob(v)[1] for name, v in tel.traceFull(ray).items()}
    check_cbp(by_name, g, i)


@pytest.mark.parametrize("band", list("ugrizy"))
def test_comcam_zemax(band):
    """tests/test_zemax.py:614-700: positions at 1e-9 on two rays per band,
    and a spot smaller than a pixel (10 um) at the first ray's field."""
    g = golden("zemax_more")
    tel = optic(f"comcam_{band}", "zemax_more")
    for i in (1, 2):
        x, y, z, vx, vy, vz, t, wl = comcam_start(g, band, i)
        ray = bt.RayVector(x, y, z, vx, vy, vz, t=t, wavelength=wl)
        by_name = {name: _glob(v)[1][:3] for name, v in tel.traceFull(ray).items()}
        check_comcam(by_name, g, band, i)
        _, Hx, Hy, _, _ = srt(g, f"comcam_{band}{i}")
        sx, sy = bt.spot(tel, np.deg2rad(Hx), np.deg2rad(Hy), wl, nx=128)
        assert np.sqrt(np.nanvar(sx) + np.nanvar(sy)) < 10e-6
