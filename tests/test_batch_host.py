"""Host side of the batched wavefront path (no GPU): per-state stage
transforms against the reference-API optic builder, bending-mode tables,
and the oracle's zernike fit."""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads
from batoid_gb300.batch import PerturbedTelescope
from batoid_gb300.coordTransform import CoordTransform
from batoid_gb300.modes import ModeSet


@pytest.fixture(scope="module")
def modes():
    return ModeSet(nmodes=8, n=64, seed=7)


@pytest.fixture(scope="module")
def telescope(modes):
    optic = workloads.tma_optic(bt)
    fields = np.deg2rad([[0.0, 0.0], [0.9, -0.6]])
    return PerturbedTelescope(optic, modes=modes, fields=fields)


def _dofs(pt, seed):
    rng = np.random.default_rng(seed)
    scale = np.concatenate([np.tile([1e-3, 1e-3, 1e-3, 4.8e-5, 4.8e-5], 2), np.full(pt.nmodes, 1e-7)])
    return rng.uniform(-1, 1, (4, pt.ndof)) * scale


def test_stage_plan(telescope):
    # M1, M2, M3, camera entrance vary; nothing else
    assert telescope.var_stages == [1, 2, 3]
    assert telescope.bend_stage == 0
    assert telescope.ndof == 18


def test_state_tables_match_optic_builder(telescope):
    pt = telescope
    dofs = _dofs(pt, 1)
    xf, det, amps = pt.state_tables(dofs)
    for s in range(len(dofs)):
        o = pt.perturbed(dofs[s])
        prog = o._program(o.coordSys)
        ifaces = [info[0] for info in prog.stage_info]
        prev = o.coordSys
        for k, it in enumerate(ifaces):
            ct = CoordTransform(prev, it.coordSys)
            if k in pt.var_stages:
                v = pt.var_stages.index(k)
                np.testing.assert_allclose(xf[s, v, :3], ct.dr, rtol=0, atol=1e-14)
                np.testing.assert_allclose(xf[s, v, 3:], ct.drot.ravel(), rtol=0, atol=1e-15)
            else:
                # members of one rigid group keep their nominal relative transform
                nom = pt.prog.arrays
                np.testing.assert_allclose(nom["dr"][k], ct.dr, rtol=0, atol=1e-14)
                np.testing.assert_allclose(nom["drot"][k], ct.drot.ravel(), rtol=0, atol=1e-15)
            prev = it.coordSys
        np.testing.assert_allclose(det[s, :3], prev.origin, rtol=0, atol=1e-14)
        np.testing.assert_allclose(det[s, 3:], prev.rot.ravel(), rtol=0, atol=1e-15)
        np.testing.assert_array_equal(amps[s], dofs[s, 10:])


def test_zero_dofs_reproduce_nominal(telescope):
    xf, det, _ = telescope.state_tables(np.zeros((1, telescope.ndof)))
    nom = telescope.prog.arrays
    for v, k in enumerate(telescope.var_stages):
        np.testing.assert_array_equal(xf[0, v, :3], nom["dr"][k])
        np.testing.assert_array_equal(xf[0, v, 3:], nom["drot"][k])


def test_mode_tables(modes):
    # unit RMS over the aperture, FP32 storage, derivatives consistent with
    # finite differences of the height
    t = modes.tables
    assert t.dtype == np.float32 and t.shape == (64, 64, 4, 8)
    X, Y = np.meshgrid(modes.xs, modes.ys)
    inside = X ** 2 + Y ** 2 <= 4.18 ** 2
    rms = np.sqrt(np.mean(t[..., 0, :][inside].astype(float) ** 2, axis=0))
    np.testing.assert_allclose(rms, 1.0, rtol=1e-6)
    z = t[..., 0, 0].astype(float)
    fd = (z[:, 2:] - z[:, :-2]) / (2 * modes.dx)
    np.testing.assert_allclose(fd, t[:, 1:-1, 1, 0], rtol=0, atol=0.05 * np.abs(fd).max())
    a = np.linspace(-1, 1, 8) * 1e-7
    zs = modes.summed(a)
    np.testing.assert_allclose(zs[0], t[..., 0, :].astype(float) @ a, rtol=1e-15, atol=0)


def test_oracle_zernike_nominal_and_perturbed(telescope):
    import wavefront as owf
    from batoid_gb300.utils import fieldToDirCos
    pt = telescope
    dirCos = fieldToDirCos(*pt.fields[1])
    c0 = owf.zernike(pt.optic, dirCos, 620e-9, 24, pt.jmax, pt.eps)
    assert c0.shape == (29,) and c0[0] == 0.0 and np.all(np.isfinite(c0))
    c1 = owf.zernike(pt.perturbed(_dofs(pt, 2)[0]), dirCos, 620e-9, 24, pt.jmax, pt.eps)
    # a 1 mm / 10 arcsec perturbation moves the wavefront by many waves
    assert np.abs(c1 - c0).max() > 0.1
    with pytest.raises(RuntimeError, match="Rank"):
        owf.zernike(pt.optic, dirCos, 620e-9, 4, pt.jmax, pt.eps)
