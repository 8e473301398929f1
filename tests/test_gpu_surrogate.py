"""Learned wavefront surrogate, end to end on a small problem: data from the
batched tracer, linear sensitivity model, MLP trained by the tensor-core
kernels, error-head calibration and the trace fallback."""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads
from batoid_gb300.batch import PerturbedTelescope
from batoid_gb300.modes import ModeSet
from batoid_gb300.surrogate import WavefrontSurrogate, rms_nm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    modes = ModeSet(nmodes=8, n=128, seed=5)
    optic = workloads.tma_optic(bt)
    fields = np.deg2rad([[0.0, 0.0], [0.8, -0.5], [-1.0, 0.9]])
    pt = PerturbedTelescope(optic, modes=modes, fields=fields)
    sur = WavefrontSurrogate(pt, wavelengths=[500e-9, 800e-9], nx=24, hidden=256, layers=2, seed=1)
    dofs, widx = sur.sample_states(6000, seed=1)
    coefs = sur.trace(dofs, widx, threads=128, ctas_per_sm=3)
    feat, grp, w = sur.features(dofs, widx)
    losses = []
    sur.train(feat, grp, w, coefs, epochs=40, batch=2048, lr=2e-3, log=lambda e, a, b: losses.append(a))
    vd, vw = sur.sample_states(600, seed=2)
    vc = sur.trace(vd, vw, threads=128, ctas_per_sm=3)
    vf, vg, vwl = sur.features(vd, vw)
    sur.calibrate(vf, vg, vwl, vc)
    return sur, losses


def test_training_converges(trained):
    sur, losses = trained
    assert losses[-1] < 0.2 * losses[0]


def test_network_improves_on_linear_model(trained):
    sur, _ = trained
    d, wi = sur.sample_states(600, seed=3)
    truth = sur.trace(d, wi, threads=128, ctas_per_sm=3).reshape(-1, sur.J + 1)
    feat, grp, w = sur.features(d, wi)
    lin = np.concatenate([np.zeros((len(feat), 1)), sur.linear(feat, grp)], axis=1)
    pred, _ = sur.predict(feat, grp, w)
    e_lin = rms_nm(lin, truth, w)
    e_net = rms_nm(pred, truth, w)
    print(f"held-out RMS wavefront error: linear {np.mean(e_lin):.3f} nm, linear + MLP {np.mean(e_net):.3f} nm")
    assert np.mean(e_net) < 0.7 * np.mean(e_lin)


def test_fallback_rows_are_the_trace(trained):
    sur, _ = trained
    d, wi = sur.sample_states(200, seed=4)
    truth = sur.trace(d, wi, threads=128, ctas_per_sm=3)
    feat, grp, w = sur.features(d, wi)
    _, err = sur.predict(feat, grp, w)
    thr = float(np.median(sur.kappa * err))  # about half the samples fall back
    out, fb = sur.with_fallback(d, wi, threshold_nm=thr, threads=128, ctas_per_sm=3)
    assert 0 < fb.sum() < fb.size
    np.testing.assert_array_equal(out[fb], truth[fb])
    acc = ~fb.ravel()
    e = rms_nm(out.reshape(-1, sur.J + 1)[acc], truth.reshape(-1, sur.J + 1)[acc], w[acc])
    # the calibrated estimate bounds most accepted errors
    assert np.mean(e <= thr) > 0.9


def test_combine_linear_model_matches_fp64(trained):
    """The device's float-float linear model against the host's FP64 one:
    with a zero network output the coefficients are the linear model."""
    import torch
    from batoid_gb300 import _device as D, _lib
    from batoid_gb300.surrogate import PAD
    sur, _ = trained
    d, wi = sur.sample_states(300, seed=6)
    feat, grp, w = sur.features(d, wi)
    n = len(feat)
    sur.predict(feat[:1], grp[:1], w[:1])  # builds the device theta
    y = torch.zeros((n, PAD), dtype=torch.float32, device=D.device())
    out = torch.empty((n, sur.J + 1), dtype=torch.float64, device=D.device())
    fd = torch.from_numpy(np.ascontiguousarray(feat)).to(D.device())
    gd = torch.from_numpy(np.ascontiguousarray(grp)).to(D.device())
    wd = D.to_device(w)
    _lib.check(_lib.lib().bt_surrogate_combine(fd.data_ptr(), feat.shape[1], sur.pt.ndof, gd.data_ptr(),
                                               sur._theta_d.data_ptr(), y.data_ptr(), PAD, wd.data_ptr(), sur.scale,
                                               sur.J, sur.J, out.data_ptr(), None, n, D.stream_ptr()))
    got = D.to_host(out)
    want = sur.linear(feat, grp)
    assert np.all(got[:, 0] == 0.0)
    scale = np.abs(want).max()
    np.testing.assert_allclose(got[:, 1:], want, rtol=0, atol=1e-12 * scale)


def test_graph_captured_training_matches_launch_by_launch():
    """A training run whose steps are replayed from one captured CUDA graph
    (device-side minibatch gather, learning-rate schedule and Adam bias
    corrections) ends at the weights of the same run issued launch by
    launch, to float32 rounding."""
    import torch
    from batoid_gb300 import _device as D
    rng = np.random.default_rng(11)
    n, nd = 4096, 7
    feat = rng.uniform(-1, 1, (n, nd + 3)).astype(np.float32)
    grp = np.zeros(n, dtype=np.int32)
    w = np.full(n, 600e-9)

    class _PT:
        ndof, nmodes, jmax = nd, 2, 5
        rigid = [0]
        fields = np.zeros((1, 2))
    coefs = np.concatenate([np.zeros((n, 1)), np.sin(feat[:, :5] * 3.0) * 1e-2], axis=1)
    runs = []
    for graph in (True, False):
        sur = WavefrontSurrogate(_PT(), wavelengths=[600e-9], nx=16, hidden=256, layers=2, seed=3)
        sur.F = 1
        sur.train(feat, grp, w, coefs, epochs=3, batch=1024, lr=2e-3, seed=5, graph=graph)
        runs.append([D.to_host(x) for x in sur.net.W])
    for a, b in zip(*runs):
        np.testing.assert_allclose(a, b, rtol=1e-4, atol=1e-6 * np.abs(b).max())


def test_vignetting_guard_flags_every_aperture_crossing():
    """The guard's first-order aperture margins (vignetting.py) predict most
    traced margins of the kept (surface, ray) pairs within their band, and
    every (state, field, wavelength) sample whose traced grid vignetting
    differs from the nominal one is flagged (before pruning): states at the
    corners of the rigid-dof box (the largest beam shifts) and typical
    states; dofs outside the box are flagged as such."""
    modes = ModeSet(nmodes=8, n=128, seed=5)
    optic = workloads.tma_optic(bt)
    fields = np.deg2rad([[0.0, 0.0], [0.8, -0.5], [-1.0, 0.9]])
    pt = PerturbedTelescope(optic, modes=modes, fields=fields)
    sur = WavefrontSurrogate(pt, wavelengths=[500e-9, 800e-9], nx=24, hidden=256, layers=2, seed=1)
    guard = sur.build_guard()
    assert guard.nkept.max() > 0
    rays = guard._grid_rays()
    N = guard.nx ** 2
    nominal = pt.perturbed(np.zeros(pt.ndof)).trace(rays.copy()).vignetted.reshape(guard.G, N)
    nr = 5 * len(pt.rigid)
    typical, widx_t = sur.sample_states(60, seed=7)
    corner, widx_c = sur.sample_states(60, seed=8)
    sign = np.where(np.random.default_rng(9).uniform(size=(60, nr)) < 0.5, -1.0, 1.0)
    corner[:, :nr] = 0.999 * sign * sur.dof_scale[:nr]
    nflips = 0
    for dofs, widx in ((typical, widx_t), (corner, widx_c)):
        feat, grp, w = sur.features(dofs, widx)
        flags = sur.guard_flags(feat, grp).reshape(len(dofs), len(fields))
        host = guard.flags_host(np.repeat(dofs, len(fields), axis=0), grp).reshape(flags.shape)
        assert np.mean(flags != host) <= 0.01
        flips = np.zeros_like(flags)
        ratios = []
        for s in range(len(dofs)):
            opt = pt.perturbed(dofs[s])
            vig = opt.trace(rays.copy()).vignetted.reshape(guard.G, N)
            marg = guard._margins(opt, rays)
            for f in range(len(fields)):
                g = f * 2 + widx[s]
                flips[s, f] = np.any(vig[g] != nominal[g])
                k = guard.nkept[g]
                if k == 0:
                    continue
                si, ri = guard.where[g]
                z = dofs[s] / guard.dof_scale
                pred = guard.m0[g, :k] + z @ guard.jac[g, :, :k]
                actual = marg[si, g * N + ri]
                band = guard.band_abs + guard.band_rel * np.abs(pred - guard.m0[g, :k])
                ratios.append(np.abs(pred - actual) / band)
        # most margins are predicted inside their band (second-order terms
        # can exceed it where the first-order change nearly cancels)
        assert np.median(np.concatenate(ratios)) < 0.5
        assert np.all(flags[flips])
        nflips += int(flips.sum())
    assert nflips > 0
    out = typical[:1].copy()
    out[0, 0] = 1.5 * sur.dof_scale[0]
    feat, grp, w = sur.features(out, widx_t[:1])
    assert np.all(sur.guard_flags(feat, grp))
