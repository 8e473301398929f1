"""Batched wavefronts + Zernike fits on the GPU against the oracle.

Each (state, field) fit of the batched kernel is compared with the CPU
restatement of batoid.zernike (reference='chief') run on the state's optic
built through the reference API.  Tolerance: |coefficient difference| x
wavelength <= 1e-11 m (0.01 nm of wavefront per Zernike term)."""
import numpy as np
import pytest
import torch

import batoid_gb300 as bt
from batoid_gb300 import _device as D
from batoid_gb300 import _lib, workloads
from batoid_gb300.batch import PerturbedTelescope
from batoid_gb300.modes import ModeSet
from batoid_gb300.utils import fieldToDirCos

pytestmark = pytest.mark.gpu

TOL_M = 1e-11


@pytest.fixture(scope="module")
def pt():
    modes = ModeSet(nmodes=20, n=256, seed=11)
    optic = workloads.tma_optic(bt)
    fields = np.deg2rad([[0.0, 0.0], [0.9, -0.6], [-1.2, 1.1]])
    return PerturbedTelescope(optic, modes=modes, fields=fields)


def _dofs(pt, n, seed):
    rng = np.random.default_rng(seed)
    scale = np.concatenate([np.tile([1e-3, 1e-3, 1e-3, 4.85e-5, 4.85e-5], 2), np.full(pt.nmodes, 1.0)])
    d = rng.uniform(-1, 1, (n, pt.ndof)) * scale
    d[:, 10:] = rng.normal(0.0, 100e-9, (n, pt.nmodes))
    return d


def _oracle(pt, dofs, nx, wl):
    import wavefront as owf
    out = np.empty((len(dofs), len(pt.fields), pt.jmax + 1))
    for s in range(len(dofs)):
        optic = pt.perturbed(dofs[s])
        for f, (tx, ty) in enumerate(pt.fields):
            out[s, f] = owf.zernike(optic, fieldToDirCos(tx, ty), wl[s], int(nx[s]), pt.jmax, pt.eps)
    return out


def test_batch_matches_oracle(pt):
    dofs = _dofs(pt, 4, 1)
    nx = np.array([24, 31, 40, 33])
    wl = np.array([350e-9, 620e-9, 1000e-9, 480e-9])
    got = pt.zernike(dofs, nx, wl, threads=128, ctas_per_sm=2)
    want = _oracle(pt, dofs, nx, wl)
    err_m = np.abs(got - want) * wl[:, None, None]
    print("max |dc| * wavelength = %.3e m" % err_m.max())
    assert err_m.max() <= TOL_M
    # the perturbations are large: the fits are far from the nominal
    nominal = pt.zernike(np.zeros((1, pt.ndof)), [24], [350e-9], threads=128, ctas_per_sm=2)
    assert np.abs(got[0] - nominal[0]).max() > 0.1


def test_batch_large_grid_and_vignetting_edge(pt):
    dofs = _dofs(pt, 1, 5)
    nx, wl = np.array([128]), np.array([700e-9])
    got = pt.zernike(dofs, nx, wl, threads=128, ctas_per_sm=3)
    want = _oracle(pt, dofs, nx, wl)
    assert (np.abs(got - want) * wl[:, None, None]).max() <= TOL_M


def test_batch_matches_single_state_gpu_path(pt):
    dofs = _dofs(pt, 2, 3)
    nx, wl = np.array([36, 37]), np.array([500e-9, 800e-9])
    got = pt.zernike(dofs, nx, wl, threads=64, ctas_per_sm=4)
    for s in range(2):
        optic = pt.perturbed(dofs[s])
        for f, (tx, ty) in enumerate(pt.fields):
            c = bt.zernike(optic, tx, ty, wl[s], nx=int(nx[s]), jmax=pt.jmax, eps=pt.eps)
            assert np.abs(got[s, f] - c).max() * wl[s] <= TOL_M


def test_launch_shapes_agree_and_graph_replay_is_exact(pt):
    dofs = _dofs(pt, 6, 9)
    nx = np.array([32, 45, 64, 50, 33, 40])
    wl = np.full(6, 550e-9)
    pt.prepare(nx)
    inp = pt.device_inputs(dofs, nx, wl)
    S, F, J = 6, len(pt.fields), pt.jmax

    def run(threads, ctas, graph):
        coefs = torch.empty(S * F * (J + 1), dtype=torch.float64, device=D.device())
        status = torch.empty(S * F, dtype=torch.int32, device=D.device())
        pt.launch(inp, coefs, status, threads, ctas, graph=graph)
        torch.cuda.synchronize()
        assert np.all(D.to_host(status) == 0)
        return D.to_host(coefs)

    a = run(128, 3, False)
    b = run(64, 6, False)
    c = run(64, 4, False)
    d = run(256, 2, False)
    np.testing.assert_allclose(b, a, rtol=0, atol=1e-9)
    np.testing.assert_allclose(c, a, rtol=0, atol=1e-9)
    np.testing.assert_allclose(d, a, rtol=0, atol=1e-9)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g1 = run(128, 3, True)
        g2 = run(128, 3, True)  # replay of the captured graph
    np.testing.assert_array_equal(g1, a)
    np.testing.assert_array_equal(g2, a)


def test_unprepared_grid_and_rank_deficient_fit(pt):
    # a grid size without fit tables: that job reports BT_ERR_ARG and NaN,
    # the others still run
    pt.prepare([30])
    dofs = _dofs(pt, 2, 4)
    nx = np.array([30, 77 if 77 not in pt._prepared else 79])
    inp = pt.device_inputs(dofs, nx, [600e-9, 600e-9])
    F, J = len(pt.fields), pt.jmax
    coefs = torch.empty(2 * F * (J + 1), dtype=torch.float64, device=D.device())
    status = torch.empty(2 * F, dtype=torch.int32, device=D.device())
    pt.launch(inp, coefs, status, 128, 2)
    st = D.to_host(status).reshape(2, F)
    cf = D.to_host(coefs).reshape(2, F, J + 1)
    assert np.all(st[0] == 0) and np.all(st[1] == _lib.BT_ERR_ARG)
    assert np.all(np.isfinite(cf[0])) and np.all(np.isnan(cf[1]))
    # too few rays for 28 terms
    with pytest.raises(RuntimeError, match="Rank"):
        pt.zernike(dofs[:1], [4], [600e-9], threads=128, ctas_per_sm=2)


def test_autotuner_picks_a_valid_shape(pt, tmp_path, monkeypatch):
    from batoid_gb300 import autotune
    monkeypatch.setenv("BATOID_GB300_CACHE", str(tmp_path))
    autotune._memo.clear()
    cfg = autotune.batch_config(pt, nstates=8)
    assert cfg in autotune.CANDIDATES
    assert (tmp_path / "autotune.json").exists()


def test_split_jobs_match_whole_jobs(pt):
    """Fewer jobs than blocks splits each job's rays over several blocks (the
    last one to finish fits); more jobs than blocks gives each job to one
    block.  Both schedules give the same fits."""
    S = 120  # 360 jobs > 152 blocks at 256 threads x 1 per SM: whole jobs
    dofs = _dofs(pt, S, 17)
    rng = np.random.default_rng(4)
    nx = rng.integers(24, 61, S)
    wl = rng.choice([400e-9, 650e-9, 900e-9], S)
    pt.prepare(nx)
    inp = pt.device_inputs(dofs, nx, wl)
    F, J = len(pt.fields), pt.jmax
    coefs = torch.empty(S * F * (J + 1), dtype=torch.float64, device=D.device())
    status = torch.empty(S * F, dtype=torch.int32, device=D.device())
    pt.launch(inp, coefs, status, 256, 1)
    torch.cuda.synchronize()
    assert np.all(D.to_host(status) == 0)
    whole = D.to_host(coefs).reshape(S * F, J + 1)
    # 10 of the jobs on their own: split over ~15 blocks each
    sub = np.array([0, 7, 33, 58, 101, 150, 222, 299, 300, 359], dtype=np.int32)
    order = torch.from_numpy(sub).to(D.device())
    c2 = torch.full((S * F * (J + 1),), float("nan"), dtype=torch.float64, device=D.device())
    s2 = torch.empty(S * F, dtype=torch.int32, device=D.device())
    pt.launch(inp, c2, s2, 256, 1, order=order)
    torch.cuda.synchronize()
    st = D.to_host(s2)
    assert np.all(st[sub] == 0)
    got = D.to_host(c2).reshape(S * F, J + 1)[sub]
    np.testing.assert_allclose(got, whole[sub], rtol=0, atol=1e-9)
