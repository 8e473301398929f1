"""Ray factories with device-generated stop points (asGrid, asPolar,
asSpokes) and fromStop against the reference's own outputs
(tests/golden/factories.npz, made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads as W
from _helpers import golden
import _factories as F

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "t", "wavelength", "flux", "vignetted", "failed")


@pytest.fixture(scope="module")
def optic():
    return W.tma_optic(bt)


@pytest.mark.parametrize("name,kind,kw", F.cases(), ids=[c[0] for c in F.cases()])
def test_factory_matches_reference(optic, name, kind, kw):
    g = golden("factories")
    rv = F.make(bt, optic, kind, kw)
    assert len(rv) == len(g[f"{name}_x"])
    for k in FIELDS:
        got = np.asarray(getattr(rv, k))
        want = g[f"{name}_{k}"]
        if k in ("vignetted", "failed"):
            np.testing.assert_array_equal(got, want, err_msg=f"{name}_{k}")
        else:
            # stop points: device cos/sin against numpy's (a few ulp of 4 m);
            # z and t follow through the stop sag and the back-propagation
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-12, err_msg=f"{name}_{k}")


def test_factory_traces_like_host_points(optic):
    """The device-generated grid traced through the optic equals a trace of
    the same points supplied from the host (fromStop)."""
    rv = bt.RayVector.asGrid(optic=optic, nx=24, wavelength=620e-9, **F.TH)
    x = np.asarray(rv.x)
    assert np.isfinite(x).all()
    nx = 24
    xx = np.fft.fftshift(np.fft.fftfreq(nx, (nx - 2) / nx)) * optic.pupilSize
    px, py = np.meshgrid(xx, xx)
    ref = bt.RayVector.fromStop(px.ravel(), py.ravel(), optic=optic, wavelength=620e-9, **F.TH)
    a = optic.trace(rv)
    b = optic.trace(ref)
    np.testing.assert_allclose(a.r, b.r, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(a.vignetted, b.vignetted)
