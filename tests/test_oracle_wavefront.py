"""The oracle's wavefront restatement (oracle/wavefront.py) against the
reference's own batoid.wavefront (batoid/analysis.py:308-388, run by
tests/golden/make_golden.py) and against Zemax's LSST wavefronts
(tests/test_zemax.py:224-270 of the reference, 10 pm).  CPU only: this pins
the checker that the batched wavefront kernel is compared with."""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads as W
from batoid_gb300.utils import fieldToDirCos
import wavefront as owf
from _helpers import golden
from _zemax import optic


def _match(opd, vig, want, want_mask, wavelength, atol=1e-11):
    opd = np.asarray(opd).reshape(want.shape)
    vig = np.asarray(vig).reshape(want.shape)
    np.testing.assert_array_equal(vig, want_mask)
    w = ~want_mask
    np.testing.assert_allclose(opd[w] * wavelength, want[w] * wavelength, rtol=0, atol=atol)


@pytest.mark.parametrize("f", [0, 1, 2])
@pytest.mark.parametrize("nx", [32, 33])
def test_oracle_wavefront_vs_reference(f, nx):
    g = golden("wavefront")
    tx, ty = g["fields"][f]
    opd, vig = owf.wavefront(W.tma_optic(bt), fieldToDirCos(tx, ty), 620e-9, nx)
    _match(opd, vig, g[f"wf_{f}_{nx}_chief"], g[f"wf_{f}_{nx}_chief_mask"], 620e-9)


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_oracle_lsst_wavefront_zemax(k):
    g = golden("zemax_more")
    tel = optic("lsst", "zemax_more")
    thx, thy = np.deg2rad(g[f"lsstwf{k}_field_deg"])
    opd, vig = owf.wavefront(tel, fieldToDirCos(thx, thy, projection='zemax'), 500e-9, 32)
    _match(opd, vig, g[f"lsstwf{k}_ref"], g[f"lsstwf{k}_ref_mask"], 500e-9)
    Z = g[f"lsstwf{k}_zemax"]
    w = (Z != 0) & ~np.asarray(vig).reshape(32, 32)
    np.testing.assert_allclose(Z[w] * 500e-9, np.asarray(opd).reshape(32, 32)[w] * 500e-9, rtol=0, atol=1e-11)


def test_oracle_hsc_wavefront_vs_reference():
    g = golden("zemax_more")
    tel = optic("hsc_no_obsc", "zemax_more")
    opd, vig = owf.wavefront(tel, fieldToDirCos(0.0, np.deg2rad(0.75), projection='zemax'), 750e-9, 64)
    _match(opd, vig, g["hsc_wf64_ref"], g["hsc_wf64_ref_mask"], 750e-9)


def test_oracle_hsc_zernike_zemax():
    """Zemax's jmax 37 Zernike decomposition of the HSC wavefront
    (tests/test_zemax.py:189-221 of the reference): pins the annular basis
    (batoid_gb300/zpoly.py) that the oracle and the device fits share."""
    g = golden("zemax_more")
    tel = optic("hsc_no_obsc", "zemax_more")
    z = owf.zernike(tel, fieldToDirCos(0.0, np.deg2rad(0.75), projection='zemax'), 750e-9, 256, 37, 0.0)
    zz = g["hsc_zernike_zemax"]
    np.testing.assert_allclose(zz[4:], z[4:], rtol=0, atol=1e-2)
    np.testing.assert_allclose(zz[11:], z[11:], rtol=0, atol=3e-3)
