"""Analysis functions on the GPU trace: drdth, dthdr, spot, fftPSF,
exitPupilPos, focalLength against the reference's own outputs
(tests/golden/analysis.npz); zernikeGQ / zernikeTA / zernikeXYAberrations /
doubleZernike (GalSim-based in the reference, so unpinned) against the
least-squares zernike fit and each other."""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads as W
from _helpers import golden

pytestmark = pytest.mark.gpu

TH = (np.deg2rad(0.6), np.deg2rad(-0.4))
WL = 620e-9


@pytest.fixture(scope="module")
def optic():
    return W.tma_optic(bt)


def test_reference_analyses(optic):
    g = golden("analysis")
    np.testing.assert_allclose(bt.drdth(optic, *TH, WL), g["drdth"], rtol=0, atol=1e-6)
    np.testing.assert_allclose(bt.dthdr(optic, *TH, WL), g["dthdr"], rtol=0, atol=1e-8)
    sx, sy = bt.spot(optic, *TH, WL, nx=32)
    np.testing.assert_allclose(sx, g["spot_x"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(sy, g["spot_y"], rtol=0, atol=1e-12)
    # PSF tolerance of the parity contract: 1e-5 of the peak (an OPD error of
    # 1e-13 m, 1e-6 rad of phase at 620 nm, moves the |FFT|^2 by ~1e-6)
    psf = bt.fftPSF(optic, *TH, WL, nx=32, pad_factor=2)
    np.testing.assert_allclose(psf.array, g["fft_array"], rtol=0, atol=1e-5 * g["fft_array"].max())
    np.testing.assert_allclose(psf.primitiveVectors, g["fft_prim"], rtol=1e-6, atol=0)
    # closest approach of rays 1 arcsec off axis: position noise of 1e-12 m
    # becomes ~2e-7 m along the axis (1 / 5e-6 rad)
    np.testing.assert_allclose(bt.exitPupilPos(optic, WL), g["epp"], rtol=0, atol=2e-6)
    np.testing.assert_allclose(bt.focalLength(optic, *TH, WL), g["focal_length"], rtol=1e-9)


def test_zernikeGQ_agrees_with_least_squares(optic):
    eps = optic.pupilObscuration
    gq = bt.zernikeGQ(optic, 0.0, 0.0, WL, rings=12, jmax=22, eps=eps)
    ls = bt.zernike(optic, 0.0, 0.0, WL, nx=160, jmax=22, eps=eps)
    assert gq.shape == (23,)
    # on axis the support of both is the full annulus; the quadratures differ
    # at the 0.3 % level (Gauss rings vs grid points near the annulus edges)
    np.testing.assert_allclose(gq[4:], ls[4:], rtol=0, atol=1e-2)


def test_zernikeTA_and_xy_aberrations(optic):
    eps = optic.pupilObscuration
    ta = bt.zernikeTA(optic, *TH, WL, nrad=10, naz=60, jmax=22, eps=eps)
    ls = bt.zernike(optic, *TH, WL, nx=128, jmax=22, eps=eps)
    assert ta[0] == 0.0 and np.all(np.isfinite(ta))
    # transverse-aberration and wavefront fits describe the same aberrations
    a, b = ta[4:], ls[4:]
    assert np.dot(a, b) / np.linalg.norm(a) / np.linalg.norm(b) > 0.9
    xz, yz = bt.zernikeXYAberrations(optic, *TH, WL, nrad=10, naz=60, jmax=22, eps=eps)
    assert xz[0] == 0.0 and yz[0] == 0.0 and np.all(np.isfinite(xz)) and np.all(np.isfinite(yz))


def test_doubleZernike_reproduces_field_dependence(optic):
    eps = optic.pupilObscuration
    field = np.deg2rad(1.2)
    dz = bt.doubleZernike(optic, field, WL, rings=4, kmax=10, jmax=11, eps=eps)
    assert dz.shape == (11, 12)
    # the field-average term of each pupil Zernike is the mean over field of zernikeGQ
    Li, w = np.polynomial.legendre.leggauss(4)
    r = np.sqrt((1 + Li) / 2) * field
    mean = np.zeros(12)
    for rr, ww in zip(r, w):
        for az in np.linspace(0, 2 * np.pi, 9, endpoint=False):
            mean += ww * bt.zernikeGQ(optic, rr * np.cos(az), rr * np.sin(az), WL, rings=4, jmax=11, eps=eps) / 18
    np.testing.assert_allclose(dz[1], mean, rtol=0, atol=1e-9)


@pytest.mark.parametrize("dx,reference", [(2e-6, "chief"), (None, "chief"), (2e-6, "mean")])
def test_huygens_psfs_match_per_field_calls(optic, dx, reference):
    """Many fields in one trace launch, one launch set of the phasor sums
    and one copy back: each PSF equals the single-field call's bit for bit."""
    thx = np.deg2rad([0.0, 0.6, -1.1])
    thy = np.deg2rad([0.0, -0.4, 0.9])
    kw = dict(nx=48, dx=dx, nxOut=24, reference=reference)
    many = bt.huygensPSFs(optic, thx, thy, WL, **kw)
    assert len(many) == 3
    for f in range(3):
        one = bt.huygensPSF(optic, thx[f], thy[f], WL, **kw)
        assert many[f].array.shape == one.array.shape
        np.testing.assert_allclose(many[f].primitiveVectors, one.primitiveVectors, rtol=1e-12, atol=0)
        np.testing.assert_array_equal(many[f].array, one.array)


def test_huygens_fields_entry_point_matches_single_field_calls(optic):
    """bt_huygens_amplitudes_fields over 70 fields (two launch sets of at
    most 64 fields) equals bt_huygens_amplitudes per field bit for bit; a
    ray count that is not a multiple of the field count is an argument
    error."""
    import ctypes
    from batoid_gb300 import _lib, _device as D
    from batoid_gb300.rayVector import concatenateRayVectors
    L = _lib.lib()
    F, nx, npix = 70, 6, 5
    rng = np.random.default_rng(3)
    thx = np.deg2rad(rng.uniform(-1, 1, F))
    thy = np.deg2rad(rng.uniform(-1, 1, F))
    rays = concatenateRayVectors([bt.RayVector.asGrid(optic=optic, wavelength=WL, theta_x=thx[f], theta_y=thy[f],
                                                      nx=nx) for f in range(F)])
    optic.trace(rays)
    n = nx * nx
    pts = np.ascontiguousarray([[rays.x[f * n + 21], rays.y[f * n + 21], 0.0] for f in range(F)])
    lat = np.ascontiguousarray(rng.uniform(1e-6, 3e-6, (F, 4)) * [1, 0.1, 0.1, 1])
    t0 = np.ascontiguousarray([float(rays.t[f * n]) for f in range(F)])
    re = D.empty(F * npix * npix)
    im = D.empty(F * npix * npix)
    dp = _lib.c_double_p
    _lib.check(L.bt_huygens_amplitudes_fields(rays._rv, F, pts.ctypes.data_as(dp), lat.ctypes.data_as(dp),
                                              t0.ctypes.data_as(dp), npix, npix, 1, D.ptr(re), D.ptr(im),
                                              D.stream_ptr()))
    got = (D.to_host(re) + 1j * D.to_host(im)).reshape(F, npix, npix)
    for f in range(F):
        view = bt.RayVector._fromBuffers(rays._d[:, f * n:(f + 1) * n], rays._b[:, f * n:(f + 1) * n],
                                         rays.coordSys)
        a, b = bt.analysis.huygens_amplitudes(view, pts[f], lat[f].reshape(2, 2), npix, npix, t0[f])
        np.testing.assert_array_equal(got[f], a + 1j * b)
    rc = L.bt_huygens_amplitudes_fields(rays._rv, F + 1, pts.ctypes.data_as(dp), lat.ctypes.data_as(dp),
                                        t0.ctypes.data_as(dp), npix, npix, 1, D.ptr(re), D.ptr(im), D.stream_ptr())
    assert rc != 0
