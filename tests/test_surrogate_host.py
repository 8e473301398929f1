"""Host logic of the surrogate: the vignetting guard (batoid_gb300/vignetting.py:
aperture margins against the oracle's obscuration test, the choice and the
pruning of the margins to keep) and the linear model's fit."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))


def _obscurations():
    import batoid_gb300 as bt
    c = bt.ObscCircle(0.4, 0.05, -0.02)
    a = bt.ObscAnnulus(0.2, 0.6, -0.03, 0.01)
    return [c, a, bt.ObscNegation(c), bt.ObscNegation(a),
            bt.ObscUnion(bt.ObscCircle(0.1), bt.ObscNegation(bt.ObscCircle(0.5))),
            bt.ObscIntersection(bt.ObscNegation(bt.ObscCircle(0.1, 0.3, 0.0)), bt.ObscAnnulus(0.05, 0.7))]


@pytest.mark.parametrize("k", range(6))
def test_margin_sign_matches_oracle_obscuration(k):
    """margin < 0 exactly where the oracle's restatement of the reference's
    obscuration test (src/obscuration.cpp) obscures, away from the edge."""
    import oracle as ora
    from batoid_gb300.vignetting import obscuration_margin
    ob = _obscurations()[k]
    rng = np.random.default_rng(k)
    x, y = rng.uniform(-0.8, 0.8, (2, 4000))
    m = obscuration_margin(ob, x, y)
    far = np.abs(m) > 1e-9
    obscured = ora.contains(ob, x, y)
    assert np.array_equal(obscured[far], (m < 0)[far])


def test_margin_is_distance_to_edge():
    import batoid_gb300 as bt
    from batoid_gb300.vignetting import obscuration_margin
    ob = bt.ObscNegation(bt.ObscAnnulus(1.0, 2.0))
    m = obscuration_margin(ob, np.array([1.5, 1.1, 2.3, 0.0]), np.zeros(4))
    np.testing.assert_allclose(m, [0.5, 0.1, -0.3, -1.0], atol=1e-15)
    assert np.all(np.isinf(obscuration_margin(None, np.zeros(3), np.zeros(3))))
    with pytest.raises(NotImplementedError):
        obscuration_margin(bt.ObscRectangle(1.0, 1.0), np.zeros(2), np.zeros(2))


def test_select_constraints():
    """Kept: margins that can reach zero in the dof box; dropped: rays
    vignetted for sure elsewhere, failed rays, far margins, no aperture."""
    from batoid_gb300.vignetting import select_constraints
    S, N, nd = 2, 5, 2
    m0 = np.array([[1e-3, -2e-4, 5e-2, 1e-4, np.inf],
                   [3e-2, 4e-2, -1e-1, np.nan, 2e-4]])
    jac = np.zeros((S, N, nd))
    jac[0, :, 0] = 1e-3      # reach 1e-3 m per unit of dof 0 at surface 0
    jac[1, :, 1] = 1e-4
    s, i = select_constraints(m0, jac, scale=np.array([1.0, 1.0]), widen=1.2, band_abs=0.0)
    kept = set(zip(s.tolist(), i.tolist()))
    # ray 0: surface 0 margin 1e-3 < 1.2e-3 -> kept; surface 1 far
    # ray 1: surface 0 margin -2e-4 (near) -> kept
    # ray 2: surface 1 margin -0.1 (sure vignetting) -> nothing kept
    # ray 3: failed -> nothing kept
    # ray 4: no aperture at surface 0; surface 1 margin 2e-4 > 1.2e-4 -> not kept
    assert kept == {(0, 0), (0, 1)}
    s, i = select_constraints(m0, jac, scale=np.array([1.0, 3.0]), widen=1.2, band_abs=0.0)
    assert (1, 4) in set(zip(s.tolist(), i.tolist()))


def test_guard_prune_drops_margins_without_errors():
    """prune keeps a margin whose triggers coincide with errors and drops one
    that triggers on every sample without them (a ray on an aperture edge)."""
    from batoid_gb300.vignetting import VignettingGuard
    g = VignettingGuard.__new__(VignettingGuard)
    g.G, g.K = 1, 32
    g.dof_scale = np.ones(2)
    g.band_abs, g.band_rel = 1e-6, 0.05
    g.m0 = np.full((1, 32), np.inf)
    g.jac = np.zeros((1, 2, 32))
    g.m0[0, 0], g.jac[0, 0, 0] = 1e-3, -1e-3     # crosses when z0 > 1
    g.m0[0, 1], g.jac[0, 1, 1] = 1e-9, 1e-9      # on the edge: triggers always
    g.nkept = np.array([2])
    g._dev = None
    rng = np.random.default_rng(0)
    dofs = rng.uniform(-1.5, 1.5, (400, 2))
    group = np.zeros(400, dtype=int)
    h = g.hits(dofs, group)
    assert h[:, 1].mean() > 0.3 and 0 < h[:, 0].mean() < 0.5
    bad = dofs[:, 0] > 1.35  # 5 % of the samples, all past the crossing of margin 0
    assert g.prune(dofs, group, bad) == 1
    assert np.isfinite(g.m0[0, 0]) and np.isinf(g.m0[0, 1])


def test_sorted_linear_fit_equals_per_group_fit(monkeypatch):
    """The surrogate's linear model fitted over samples sorted by group
    (WavefrontSurrogate._fit_linear_sorted) equals the per-group fit and its
    residuals (fit_linear, residual_targets) to rounding."""
    from batoid_gb300 import _device
    from batoid_gb300.surrogate import WavefrontSurrogate
    monkeypatch.setattr(_device, "device", lambda: "cpu")
    rng = np.random.default_rng(3)
    n, nd, J, G = 4000, 6, 5, 6
    feat = rng.uniform(-1, 1, (n, nd + 3)).astype(np.float32)
    grp = rng.integers(0, G, n).astype(np.int32)
    coefs = np.concatenate([np.zeros((n, 1)), rng.normal(size=(n, J))], axis=1)
    w = np.full(n, 6e-7)

    class _PT:
        ndof = nd

    sur = WavefrontSurrogate.__new__(WavefrontSurrogate)
    sur.pt, sur.F, sur.wavelengths, sur.J = _PT(), G, np.ones(1), J
    r = sur._fit_linear_sorted(feat, grp, w, coefs).numpy()
    theta = sur.theta.copy()
    sur.fit_linear(feat, grp, coefs)
    r_ref = sur.residual_targets(feat, grp, w, coefs)
    np.testing.assert_allclose(theta, sur.theta, rtol=0, atol=1e-12)
    np.testing.assert_allclose(r, r_ref, rtol=0, atol=1e-9 * np.abs(r_ref).max())
