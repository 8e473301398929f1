"""YAML-subset reader, optic builder, and the oracle against the Zemax golden
traces of the reference's tests (CPU only)."""
import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300.parse import yaml_load, parse_optic
import oracle as ora
from _helpers import golden, assert_rays_match, FIELDS
from _zemax import (optic, check_lsst, check_hsc, check_decam, check_cbp, check_comcam, cbp_start, comcam_start,
                    HSC_NAMES)

DOC = """
top:
  a: &anch 1.5   # comment
  b: *anch
  s: 'quoted # not a comment'
  flow: [1, -2.5e-3,
         3.0, abc]
  seq:
    - type: One
      v: 1
    -
      type: Two
    - 7
  med: &m
    type: X
    k: 2
  med2: *m
  flag: true
  none: null
"""


def test_yaml_subset():
    d = yaml_load(DOC)["top"]
    assert d["a"] == 1.5 and d["b"] == 1.5
    assert d["s"] == "quoted # not a comment"
    assert d["flow"] == [1, -2.5e-3, 3.0, "abc"]
    assert d["seq"] == [{"type": "One", "v": 1}, {"type": "Two"}, 7]
    assert d["med2"] == {"type": "X", "k": 2}
    assert d["flag"] is True and d["none"] is None


def test_parse_builds_lsst_and_hsc():
    lsst = optic("lsst")
    assert [i.name for i in lsst._interfaces()] == list(golden("zemax")["lsst0_names"])
    assert lsst["L1_entrance"].outMedium == lsst["L1"].medium
    hsc = optic("hsc")
    names = [i.name for i in hsc._interfaces()]
    for n in HSC_NAMES:
        assert n in names


def _global(r):
    """Oracle rays (frame = origin, rot) to global coordinates."""
    R, o = r.rot, r.origin
    pos = (R @ np.stack([r.x, r.y, r.z])).T + o
    vel = (R @ np.stack([r.vx, r.vy, r.vz])).T
    return pos, vel


@pytest.mark.parametrize("k", [0, 1, 2])
def test_oracle_lsst_zemax(k):
    g = golden("zemax")
    tel = optic("lsst")
    rays = ora.Rays(*[g[f"lsst{k}_in_{f}"] for f in FIELDS])
    outs = ora.trace(tel, rays, full=True)
    glob_rays = []
    for name, r in outs:
        pos, vel = _global(r)
        glob_rays.append((pos[0, 0], pos[0, 1], pos[0, 2], vel[0, 0], vel[0, 1], vel[0, 2]))
        # and the reference's own trace of the same ray, surface by surface
        np.testing.assert_allclose(pos[0], [g[f"lsst{k}_{name}_{c}"][0] for c in "xyz"], rtol=0, atol=1e-12)
    check_lsst(glob_rays, g[f"lsst{k}_zemax"])


@pytest.mark.parametrize("k", [1, 2, 3])
def test_oracle_hsc_zemax(k):
    g = golden("zemax")
    tel = optic("hsc")
    a0 = g[f"hsc{k}_zemax"][0]
    rays = ora.Rays([a0[1] / 1000], [a0[2] / 1000], [16.0], [a0[4]], [a0[5]], [-a0[6]], [0.0], [750e-9], [1.0],
                    [False], [False])
    outs = dict(ora.trace(tel, rays, full=True))
    by_name = {}
    for name, r in outs.items():
        pos, vel = _global(r)
        by_name[name] = (pos[0, 0], pos[0, 1], pos[0, 2], vel[0, 0], vel[0, 1], vel[0, 2])
    check_hsc(by_name, g[f"hsc{k}_zemax"])


def _by_name(outs):
    by_name = {}
    for name, r in outs:
        pos, vel = _global(r)
        by_name[name] = (pos[0, 0], pos[0, 1], pos[0, 2], vel[0, 0], vel[0, 1], vel[0, 2])
    return by_name


def _one_ray(x, y, z, vx, vy, vz, t, wl):
    return ora.Rays([x], [y], [z], [vx], [vy], [vz], [t], [wl], [1.0], [False], [False])


@pytest.mark.parametrize("k", [0, 1, 2])
def test_oracle_decam_zemax(k):
    g = golden("zemax_more")
    tel = optic("decam", "zemax_more")
    rays = ora.Rays(*[g[f"decam{k}_in_{f}"] for f in FIELDS])
    outs = ora.trace(tel, rays, full=True)
    assert [n for n, _ in outs] == list(g[f"decam{k}_names"])
    for name, r in outs:
        pos, _ = _global(r)
        np.testing.assert_allclose(pos[0], [g[f"decam{k}_{name}_{c}"][0] for c in "xyz"], rtol=0, atol=1e-12)
    by_name = _by_name(outs)
    check_decam([by_name[n] for n, _ in outs], g[f"decam{k}_zemax"])


@pytest.mark.parametrize("i", [1, 2, 3, 4])
def test_oracle_cbp_zemax(i):
    g = golden("zemax_more")
    check_cbp(_by_name(ora.trace(optic("cbp", "zemax_more"), _one_ray(*cbp_start(g, i)), full=True)), g, i)


@pytest.mark.parametrize("band", list("ugrizy"))
def test_oracle_comcam_zemax(band):
    g = golden("zemax_more")
    tel = optic(f"comcam_{band}", "zemax_more")
    for i in (1, 2):
        by_name = _by_name(ora.trace(tel, _one_ray(*comcam_start(g, band, i)), full=True))
        check_comcam({k: v[:3] for k, v in by_name.items()}, g, band, i)
