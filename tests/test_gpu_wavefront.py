"""wavefront, zernike and huygensPSF through the CUDA path against the
reference's own outputs (batoid/analysis.py:17-56, 181-388, generated by
tests/golden/make_golden.py) and against Zemax (the reference's
tests/test_zemax.py:189-270: LSST wavefronts at 10 pm, the HSC Zernike
decomposition at 1e-2 / 3e-3 waves)."""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads as W
from _helpers import golden
from _zemax import optic

pytestmark = pytest.mark.gpu

WL = 620e-9


def _wf_match(wf, want, want_mask, wavelength, atol=1e-11):
    arr = wf.array
    np.testing.assert_array_equal(np.ma.getmaskarray(arr), want_mask)
    w = ~want_mask
    np.testing.assert_allclose(np.asarray(arr.data)[w] * wavelength, want[w] * wavelength, rtol=0, atol=atol)


@pytest.mark.parametrize("f", [0, 1, 2])
@pytest.mark.parametrize("nx", [32, 33])
@pytest.mark.parametrize("ref", ["chief", "mean"])
def test_wavefront_vs_reference(f, nx, ref):
    g = golden("wavefront")
    tx, ty = g["fields"][f]
    wf = bt.wavefront(W.tma_optic(bt), tx, ty, WL, nx=nx, reference=ref)
    _wf_match(wf, g[f"wf_{f}_{nx}_{ref}"], g[f"wf_{f}_{nx}_{ref}_mask"], WL)
    np.testing.assert_allclose(wf.primitiveVectors, g[f"wf_{f}_{nx}_{ref}_prim"], rtol=1e-15, atol=0)


@pytest.mark.parametrize("f", [0, 1, 2])
def test_dkdu_vs_reference(f):
    g = golden("wavefront")
    tx, ty = g["fields"][f]
    np.testing.assert_allclose(bt.analysis.dkdu(W.tma_optic(bt), tx, ty, WL), g[f"dkdu_{f}"], rtol=1e-9,
                               atol=1e-9 * np.abs(g[f"dkdu_{f}"]).max())


def _psf_match(psf, want, prim, rel=1e-5):
    a = np.asarray(psf.array)
    assert a.shape == want.shape
    assert np.abs(a - want).max() <= rel * want.max()
    np.testing.assert_allclose(psf.primitiveVectors, prim, rtol=1e-9, atol=1e-9 * np.abs(prim).max())


@pytest.mark.parametrize("f", [1, 2])
@pytest.mark.parametrize("nx", [32, 33])
@pytest.mark.parametrize("ref", ["chief", "mean"])
def test_huygens_psf_vs_reference(f, nx, ref):
    """Lattice given by dx; |A|^2 within 1e-5 of the peak."""
    g = golden("wavefront")
    tx, ty = g["fields"][f]
    psf = bt.huygensPSF(W.tma_optic(bt), tx, ty, WL, nx=nx, dx=1.5e-6, nxOut=20, reference=ref)
    _psf_match(psf, g[f"hpsf_{f}_{nx}_{ref}_dx"], g[f"hpsf_{f}_{nx}_{ref}_dx_prim"])


@pytest.mark.parametrize("f", [1, 2])
def test_huygens_psf_dkdu_lattice_vs_reference(f):
    """dx None: the fftPSF lattice from dkdu, padded twice."""
    g = golden("wavefront")
    tx, ty = g["fields"][f]
    psf = bt.huygensPSF(W.tma_optic(bt), tx, ty, WL, nx=24, reference="chief")
    _psf_match(psf, g[f"hpsf_{f}_24_chief_dkdu"], g[f"hpsf_{f}_24_chief_dkdu_prim"])


@pytest.mark.parametrize("ref", ["chief", "mean"])
def test_huygens_psfs_vs_reference(ref):
    """Both fields in one call."""
    g = golden("wavefront")
    f = np.array([1, 2])
    psfs = bt.analysis.huygensPSFs(W.tma_optic(bt), g["fields"][f, 0], g["fields"][f, 1], WL, nx=33, dx=1.5e-6,
                                   nxOut=20, reference=ref)
    for k, fi in enumerate(f):
        _psf_match(psfs[k], g[f"hpsf_{fi}_33_{ref}_dx"], g[f"hpsf_{fi}_33_{ref}_dx_prim"])


def test_reference_point_must_be_known():
    with pytest.raises(ValueError):
        bt.huygensPSF(W.tma_optic(bt), 0.0, 0.0, WL, nx=16, dx=1e-6, reference='Mean')
    with pytest.raises(ValueError):
        bt.wavefront(W.tma_optic(bt), 0.0, 0.0, WL, nx=16, reference='centroid')


@pytest.mark.parametrize("k", [0, 1, 2, 3])
def test_lsst_wavefront_zemax(k):
    """tests/test_zemax.py:224-270: Zemax and batoid agree to 10 pm."""
    g = golden("zemax_more")
    tel = optic("lsst", "zemax_more")
    thx, thy = np.deg2rad(g[f"lsstwf{k}_field_deg"])
    wf = bt.wavefront(tel, thx, thy, 500e-9, nx=32, reference='chief', projection='zemax')
    _wf_match(wf, g[f"lsstwf{k}_ref"], g[f"lsstwf{k}_ref_mask"], 500e-9)
    Z = np.ma.MaskedArray(data=g[f"lsstwf{k}_zemax"], mask=g[f"lsstwf{k}_zemax"] == 0)
    np.testing.assert_allclose(Z * 500e-9, wf.array * 500e-9, rtol=0, atol=1e-11)


def test_hsc_wavefront_vs_reference():
    g = golden("zemax_more")
    tel = optic("hsc_no_obsc", "zemax_more")
    wf = bt.wavefront(tel, 0.0, np.deg2rad(0.75), 750e-9, nx=64, reference='chief', projection='zemax')
    _wf_match(wf, g["hsc_wf64_ref"], g["hsc_wf64_ref_mask"], 750e-9)


def test_hsc_zernike_zemax():
    """tests/test_zemax.py:189-221: Zemax's jmax 37 decomposition of the HSC
    wavefront at 0.75 deg, 750 nm, nx 256; piston, tip and tilt excluded."""
    g = golden("zemax_more")
    tel = optic("hsc_no_obsc", "zemax_more")
    z = bt.zernike(tel, 0.0, np.deg2rad(0.75), 750e-9, jmax=37, nx=256, projection='zemax', reference='chief')
    zz = g["hsc_zernike_zemax"]
    np.testing.assert_allclose(zz[4:], z[4:], rtol=0, atol=1e-2)
    np.testing.assert_allclose(zz[11:], z[11:], rtol=0, atol=3e-3)
