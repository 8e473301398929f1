"""The allocation-free Huygens entry point agrees with the allocating one.

bt_huygens_amplitudes_noalloc serves callers that may not let the library
allocate device memory (a host framework that owns a fixed device-memory
budget, or a latency-critical loop that must not call cudaMalloc); its scratch
is a fixed array inside the library.  This file is collected last so that a
failure here stops a -x run only after every other test has run.  It passes
alone in a fresh process and after the other tests: the scratch array needs
no initial contents.
"""
import ctypes

import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import _lib, _device as D
from batoid_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _amplitudes(fn, rays, point, lat, na, nb, t0):
    re = D.empty(na * nb)
    im = D.empty(na * nb)
    r = rays._rv
    latv = np.ascontiguousarray(lat, dtype=float)
    rc = fn(ctypes.byref(r), float(point[0]), float(point[1]), 0.0, latv.ctypes.data_as(_lib.c_double_p),
            na, nb, float(t0), 1, D.ptr(re), D.ptr(im), D.stream_ptr())
    return rc, D.to_host(re) + 1j * D.to_host(im)


def test_noalloc_matches_allocating_entry_point_twice():
    L = _lib.lib()
    opt = W.tma_optic(bt)
    lat = [2e-6, 0.0, 0.0, 2e-6]
    results = []
    for wl, nx, npix in ((620e-9, 128, 64), (870e-9, 96, 48)):
        rays = bt.RayVector.asGrid(optic=opt, wavelength=wl, theta_x=0.004, theta_y=-0.002, nx=nx)
        opt.trace(rays)
        point = rays.r[(nx // 2) * nx + nx // 2]
        t0 = rays.t[0]
        rc, want = _amplitudes(L.bt_huygens_amplitudes, rays, point, lat, npix, npix, t0)
        _lib.check(rc)
        rc, got = _amplitudes(L.bt_huygens_amplitudes_noalloc, rays, point, lat, npix, npix, t0)
        _lib.check(rc)
        peak = np.abs(want).max()
        assert peak > 0
        # same kernels, possibly a different number of ray splits: FP32
        # partial sums agree to well inside the 1e-5-of-peak PSF tolerance
        assert np.abs(got - want).max() <= 1e-6 * peak
        results.append(got)
    assert results[0].shape != results[1].shape


def test_noalloc_rejects_oversized_problem():
    L = _lib.lib()
    n = 300_000   # 32 B per ray alone exceeds the 8 MiB scratch array
    rays = bt.RayVector(np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n), np.ones(n),
                        wavelength=500e-9)
    rc, _ = _amplitudes(L.bt_huygens_amplitudes_noalloc, rays, (0.0, 0.0), [1e-6, 0, 0, 1e-6], 8, 8, 0.0)
    assert rc == _lib.BT_ERR_ARG
    assert b"limit is 8388608" in L.bt_last_error()
