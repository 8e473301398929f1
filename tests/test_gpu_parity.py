"""CUDA path vs the reference's golden vectors and vs the oracle.

Tolerances (the parity contract): positions and directions 1e-12, path
length t 1e-11 m (0.01 nm OPD), vignetted/failed bit-identical.
"""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads as W
import oracle as ora
from _helpers import golden, assert_rays_match, ray_inputs, FIELDS
from _prims import SURFACES, make_surfaces, make_obscurations, make_media, cs_from

pytestmark = pytest.mark.gpu


def rv_from(arrs, coordSys=None):
    rv = bt.RayVector(*arrs)
    if coordSys is not None:
        rv.coordSys = coordSys
    return rv


@pytest.fixture(scope="module")
def surfs():
    return make_surfaces(bt)


@pytest.mark.parametrize("name", SURFACES)
def test_surface_sag_normal(name, surfs):
    g = golden("primitives")
    s = surfs[name]
    x, y = g[f"surf_{name}_xy"]
    np.testing.assert_allclose(s.sag(x, y), g[f"surf_{name}_sag"], rtol=0, atol=1e-13, equal_nan=True)
    np.testing.assert_allclose(s.normal(x, y), g[f"surf_{name}_normal"], rtol=0, atol=1e-13, equal_nan=True)


@pytest.mark.parametrize("name", SURFACES)
@pytest.mark.parametrize("op", ["intersect", "reflect", "refract", "reflect_coated", "refract_rev"])
def test_surface_ops_vs_reference(name, op, surfs):
    g = golden("primitives")
    s = surfs[name]
    origin, rot = cs_from(g[f"surf_{name}_cs"])
    cs = bt.CoordSys(origin, rot)
    arrs = list(ray_inputs(g, f"surf_{name}_in"))
    silica = bt.SellmeierMedium(*W.SILICA)
    vac = bt.ConstMedium(1.0)
    if op == "refract_rev":
        for k in (3, 4, 5):
            arrs[k] = arrs[k] / 1.45
    rv = rv_from(arrs)
    if op == "intersect":
        s.intersect(rv, coordSys=cs)
    elif op == "reflect":
        s.reflect(rv, coordSys=cs)
    elif op == "reflect_coated":
        s.reflect(rv, coordSys=cs, coating=bt.SimpleCoating(0.2, 0.7))
    elif op == "refract":
        s.refract(rv, vac, silica, coordSys=cs)
    else:
        s.refract(rv, silica, vac, coordSys=cs)
    assert rv.coordSys == cs
    assert_rays_match(rv, g, f"surf_{name}_{op}", label=f"{name} {op}")


def test_obscurations_vs_reference():
    g = golden("primitives")
    pts = g["obsc_pts"]
    for k, o in make_obscurations(bt).items():
        np.testing.assert_array_equal(o.contains(pts[0], pts[1]), g[f"obsc_{k}"], err_msg=k)


def test_media_vs_reference():
    g = golden("primitives")
    wl = g["media_wavelengths"]
    for k, m in make_media(bt, g).items():
        np.testing.assert_allclose(m.getN(wl), g[f"media_{k}"], rtol=1e-15, atol=0, equal_nan=True, err_msg=k)
    csv = golden("sellmeier_csv")
    silica = bt.SellmeierMedium(0.6961663, 0.4079426, 0.8974794, 0.00467914825849, 0.013512063073959999,
                                97.93400253792099)
    np.testing.assert_allclose(silica.getN(csv["csv_wmicron"] * 1e-6), csv["csv_n"], atol=0, rtol=1e-13)


def test_paraboloid_workload_vs_reference():
    g = golden("workloads")
    opt = W.paraboloid_optic(bt)
    arrs = W.paraboloid_rays(4096, seed=57721)
    rv = rv_from(arrs)
    tf = opt.traceFull(rv)
    assert list(tf.keys()) == ["M1", "D"]
    for k, v in tf.items():
        assert_rays_match(v["out"], g, f"paraboloid_{k}", label=k)
    np.testing.assert_array_equal(rv.x, arrs[0])   # traceFull leaves its input alone
    opt.trace(rv)
    assert_rays_match(rv, g, "paraboloid_final", label="trace")
    assert rv.coordSys == opt["D"].coordSys


def test_tma_workload_vs_reference():
    g = golden("workloads")
    opt = W.tma_optic(bt)
    rv = rv_from(W.tma_rays(2048, seed=8675309))
    tf = opt.traceFull(rv)
    assert list(tf.keys()) == list(g["tma_names"])
    for k, v in tf.items():
        assert_rays_match(v["out"], g, f"tma_{k}", label=k)
    opt.trace(rv)
    assert_rays_match(rv, g, "tma_Detector", label="trace")


@pytest.mark.parametrize("workload,n", [("paraboloid", 1 << 20), ("tma_corrector", 1 << 18)])
def test_workload_vs_oracle_at_scale(workload, n):
    build_optic, make_rays, _ = W.WORKLOADS[workload]
    opt = build_optic(bt)
    arrs = make_rays(n, seed=4242)
    rv = rv_from(arrs)
    opt.trace(rv)
    rays = ora.Rays(*arrs)
    ora.trace(opt, rays)
    assert_rays_match(rv, rays, label=workload)
    assert rv.vignetted.sum() < n  # not everything vignetted


def test_rayvector_methods_vs_reference():
    g = golden("workloads")
    rv = rv_from(ray_inputs(g, "paraboloid_final"))
    t0 = float(g["paraboloid_amp_t0"])
    pts = g["paraboloid_amp_points"]
    for p, want, want_all in zip(pts, g["paraboloid_sumamp"], g["paraboloid_sumamp_all"]):
        assert abs(rv.sumAmplitude(p, t0) - want) <= 1e-9 * max(1.0, abs(want))
        assert abs(rv.sumAmplitude(p, t0, ignoreVignetted=False) - want_all) <= 1e-9 * max(1.0, abs(want_all))
    np.testing.assert_allclose(rv.phase(pts[1], t0), g["paraboloid_phase"], rtol=1e-13, atol=1e-6)
    np.testing.assert_allclose(rv.amplitude(pts[1], t0), g["paraboloid_amplitude"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(rv.positionAtTime(t0 + 0.01), g["paraboloid_pos_at_time"], rtol=0, atol=1e-12)


def test_huygens_vs_reference():
    """Phasor sums relative to the peak amplitude: PSF within 1e-5 of peak."""
    g = golden("huygens")
    for case in (0, 1):
        p = f"huy{case}"
        tx, ty, w, nx, npix = g[f"{p}_params"]
        npix = int(npix)
        rays = rv_from(ray_inputs(g, f"{p}_rays"))
        point = g[f"{p}_point"]
        re, im = bt.analysis.huygens_amplitudes(rays, (point[0], point[1], 0.0),
                                                 np.array([[2e-6, 0.0], [0.0, 2e-6]]), npix, npix,
                                                 float(g[f"{p}_t0"]))
        amp = re + 1j * im
        want = g[f"{p}_amps"]
        peak = np.abs(want).max()
        assert np.abs(amp - want).max() <= 1e-5 * peak
        psf, psf_want = np.abs(amp) ** 2, np.abs(want) ** 2
        assert np.abs(psf - psf_want).max() <= 1e-5 * psf_want.max()


def test_huygens_psf_api():
    opt = W.tma_optic(bt)
    psf = bt.huygensPSF(opt, 0.0, 0.0, 620e-9, nx=64, dx=2e-6, dy=2e-6, nxOut=32)
    assert psf.array.shape == (32, 32)
    assert np.isfinite(psf.array).all()
    assert psf.array.max() > 0


def test_empty_and_single_ray():
    opt = W.paraboloid_optic(bt)
    empty = bt.RayVector(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))
    opt.trace(empty)
    assert len(empty) == 0
    tf = opt.traceFull(empty)
    assert len(tf["D"]["out"]) == 0
    arrs = [a[:1] for a in W.paraboloid_rays(1, seed=1)]
    rv = rv_from(arrs)
    opt.trace(rv)
    rays = ora.Rays(*arrs)
    ora.trace(opt, rays)
    assert_rays_match(rv, rays, label="single")


def test_failed_inputs_and_nan_rays():
    """Failed rays are skipped but still obscured; NaN rays fail cleanly."""
    opt = W.tma_optic(bt)
    arrs = list(W.tma_rays(4096, seed=99))
    arrs[10] = np.zeros(4096, bool)
    arrs[10][::7] = True             # failed on input
    arrs[0] = arrs[0].copy()
    arrs[0][::11] = np.nan           # NaN positions
    arrs[3] = arrs[3].copy()
    arrs[3][::13] = np.inf
    rv = rv_from(arrs)
    opt.trace(rv)
    rays = ora.Rays(*arrs)
    ora.trace(opt, rays)
    assert_rays_match(rv, rays, label="failed/nan")


def test_niter_zero_and_reverse():
    import batoid_gb300.global_vars as gv
    opt = W.tma_optic(bt)
    arrs = W.tma_rays(4096, seed=5)
    old = gv._batoid_niter
    try:
        gv._batoid_niter = 0
        rv = rv_from(arrs)
        opt.trace(rv)
        rays = ora.Rays(*arrs)
        ora.trace(opt, rays, niter=0)
        assert_rays_match(rv, rays, label="niter0")
    finally:
        gv._batoid_niter = old
    # reverse trace of the forward output returns through the system
    rv = rv_from(arrs)
    opt.trace(rv)
    rev = bt.RayVector(rv.x, rv.y, rv.z, -rv.vx, -rv.vy, -rv.vz, rv.t, rv.wavelength, rv.flux, rv.vignetted,
                       rv.failed, coordSys=rv.coordSys)
    rays = ora.Rays(rev.x, rev.y, rev.z, rev.vx, rev.vy, rev.vz, rev.t, rev.wavelength, rev.flux, rev.vignetted,
                    rev.failed, origin=rv.coordSys.origin, rot=rv.coordSys.rot)
    opt.trace(rev, reverse=True)
    ora.trace(opt, rays, reverse=True)
    assert_rays_match(rev, rays, label="reverse")


def test_trace_host_matches_device():
    """The host-buffer end-to-end entry point gives the device trace's result."""
    import ctypes
    import torch
    from batoid_gb300 import _lib
    opt = W.tma_optic(bt)
    n = 100_003
    arrs = W.tma_rays(n, seed=17)
    rv = rv_from(arrs)
    opt.trace(rv)
    host = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).pin_memory() for a in arrs[:9]]
    flags = [torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint8)).pin_memory() for a in arrs[9:]]
    h = _lib.BtRayVector(*[t.data_ptr() for t in host], *[t.data_ptr() for t in flags], n)
    prog = opt._program(bt.globalCoordSys)
    prog.trace_host(h, chunk=32768)
    got = dict(zip(FIELDS, [t.numpy() for t in host] + [t.numpy().astype(bool) for t in flags]))
    for k in FIELDS:
        np.testing.assert_array_equal(got[k], getattr(rv, k), err_msg=k)


def test_device_status_clean():
    from batoid_gb300 import _lib, _device as D
    _lib.check(_lib.lib().bt_check_device_status(D.stream_ptr()))


def test_zernike_fit_matches_lstsq():
    from batoid_gb300 import zpoly
    from batoid_gb300.analysis import fit_zernike
    rng = np.random.default_rng(3)
    r = np.sqrt(rng.uniform(0.6 ** 2, 1.0, 5000)) * 4.18
    th = rng.uniform(0, 2 * np.pi, 5000)
    x, y = r * np.cos(th), r * np.sin(th)
    truth = rng.normal(0, 0.1, 23)
    truth[0] = 0
    basis = zpoly.basis_xy(22, 4.18, 4.18 * 0.61)
    B = np.stack([zpoly.horner2d_host(x, y, basis[j]) for j in range(22)])
    vals = truth[1:] @ B + rng.normal(0, 1e-3, 5000)
    got = fit_zernike(x, y, vals, 22, 4.18, 4.18 * 0.61)
    want = np.linalg.lstsq(B.T, vals, rcond=None)[0]
    np.testing.assert_allclose(got[1:], want, rtol=0, atol=1e-10)
    with pytest.raises(RuntimeError):
        fit_zernike(x[:10], y[:10], vals[:10], 22, 4.18, 4.18 * 0.61)
