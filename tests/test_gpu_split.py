"""rSplit and traceSplit (ghost tracing) on the GPU against the reference's
own outputs (tests/golden/split.npz, made by tests/golden/make_golden.py)."""
import numpy as np
import pytest

import batoid_gb300 as bt
from _helpers import golden
import _split_optic as S

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "t", "wavelength", "flux", "vignetted", "failed")


def _match(rv, g, prefix):
    for k in FIELDS:
        got = np.asarray(getattr(rv, k))
        want = g[f"{prefix}_{k}"]
        if k in ("vignetted", "failed"):
            np.testing.assert_array_equal(got, want, err_msg=f"{prefix}_{k}")
        else:
            tol = 1e-11 if k == "t" else 1e-12
            np.testing.assert_allclose(got, want, rtol=0, atol=tol, equal_nan=True, err_msg=f"{prefix}_{k}")


@pytest.mark.parametrize("case", [0, 1, 2])
def test_rsplit_matches_reference(case):
    g = golden("split")
    surf, m1, m2, coat, cs, speed = S.rsplit_cases(bt)[case]
    rv = bt.RayVector(*S.rsplit_rays(speed=speed))
    refr, refl = bt.trace.rSplit(surf, rv, m1, m2, coat, coordSys=cs)
    _match(refr, g, f"rs{case}_refr")
    _match(refl, g, f"rs{case}_refl")
    assert refr.coordSys == cs and refl.coordSys == cs


def test_tracesplit_matches_reference():
    g = golden("split")
    optic = S.split_optic(bt)
    fwd, rev = optic.traceSplit(bt.RayVector(*S.split_rays()), minFlux=1e-4)
    for tag, lst in (("F", fwd), ("R", rev)):
        assert len(lst) == int(g[f"{tag}_n"])
        assert ["|".join(r.path) for r in lst] == list(g[f"{tag}_paths"])
        for k, r in enumerate(lst):
            _match(r, g, f"{tag}{k}")
    # flux bookkeeping: the direct path keeps 0.98^4 of the flux
    direct = [r for r in fwd if r.path == ["L1_entrance", "L1_exit", "L2_entrance", "L2_exit", "D"]]
    assert len(direct) == 1
    np.testing.assert_allclose(direct[0].flux, 0.98 ** 4, rtol=1e-14)


@pytest.mark.parametrize("case", [0, 1])
def test_refract_screen_matches_reference(case):
    g = golden("split")
    surf, screen, cs = S.screen_cases(bt)[case]
    rv = bt.trace.refractScreen(surf, bt.RayVector(*S.rsplit_rays()), screen, coordSys=cs)
    _match(rv, g, f"scr{case}")


def test_opd_screen_in_fused_optic_trace():
    g = golden("split")
    out = S.screen_optic(bt).trace(bt.RayVector(*S.split_rays()))
    _match(out, g, "scr_optic")
