"""The fused trace's float-float form (the default for niter >= 3) against
its FP64 form (BATOID_GB300_TRACE_FORM=fp64, read once per process, so that
form runs in a child process): same flags, positions and directions within
1e-12, path within 1e-11 -- on both benchmark workloads, including
per-surface snapshots of traceFull."""
import os
import subprocess
import sys

import numpy as np
import pytest

import batoid_gb300 as bt
from batoid_gb300 import workloads as W
from _helpers import assert_rays_match, FIELDS

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import batoid_gb300 as bt
from batoid_gb300 import workloads as W
out = {}
for name in ("paraboloid", "tma_corrector"):
    build, make, _ = W.WORKLOADS[name]
    opt = build(bt)
    rv = bt.RayVector(*make(20000, seed=99))
    tf = opt.traceFull(rv)
    for k, v in tf.items():
        for f in %r:
            out[f"{name}|{k}|{f}"] = np.asarray(getattr(v["out"], f))
np.savez(sys.argv[2], **out)
""" % (FIELDS,)


@pytest.fixture(scope="module")
def fp64_form(tmp_path_factory):
    path = str(tmp_path_factory.mktemp("forms") / "fp64.npz")
    env = dict(os.environ, BATOID_GB300_TRACE_FORM="fp64")
    r = subprocess.run([sys.executable, "-c", CHILD, os.path.dirname(HERE), path], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return dict(np.load(path))


@pytest.mark.parametrize("name", ["paraboloid", "tma_corrector"])
def test_float_float_form_matches_fp64_form(fp64_form, name):
    build, make, _ = W.WORKLOADS[name]
    opt = build(bt)
    rv = bt.RayVector(*make(20000, seed=99))
    tf = opt.traceFull(rv)
    for k, v in tf.items():
        want = {f"x_{f}": fp64_form[f"{name}|{k}|{f}"] for f in FIELDS}
        assert_rays_match(v["out"], want, "x", label=f"{name}/{k}")
