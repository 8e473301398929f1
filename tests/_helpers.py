"""Shared test helpers: golden fixtures and ray comparisons."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = ("x", "y", "z", "vx", "vy", "vz", "t", "wavelength", "flux", "vignetted", "failed")

# Tolerances of the parity contract: positions 1e-12 m, optical path
# (t) 1e-11 m (0.01 nm), directions 1e-12, flags bit-identical.
ATOL = {"x": 1e-12, "y": 1e-12, "z": 1e-12, "vx": 1e-12, "vy": 1e-12, "vz": 1e-12, "t": 1e-11,
        "wavelength": 0.0, "flux": 1e-15}

_cache = {}


def golden(name):
    if name not in _cache:
        _cache[name] = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return _cache[name]


def get_field(rv, k):
    return np.asarray(getattr(rv, k))


def assert_rays_match(got, want, prefix="", atol=None, label=""):
    """``got``: object with field attributes (RayVector or oracle Rays);
    ``want``: dict of arrays keyed f"{prefix}_{field}" or a second object."""
    atol = dict(ATOL, **(atol or {}))
    for k in FIELDS:
        g = get_field(got, k)
        w = want[f"{prefix}_{k}"] if isinstance(want, dict) else get_field(want, k)
        if k in ("vignetted", "failed"):
            bad = np.nonzero(np.asarray(g, bool) != np.asarray(w, bool))[0]
            assert bad.size == 0, f"{label} {k}: {bad.size} flags differ, first at {bad[:5]}"
        else:
            np.testing.assert_allclose(g, w, rtol=0, atol=atol[k], equal_nan=True,
                                       err_msg=f"{label} field {k}")


def ray_inputs(d, prefix):
    return tuple(d[f"{prefix}_{k}"] for k in FIELDS)
