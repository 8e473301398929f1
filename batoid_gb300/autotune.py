"""Launch-shape autotuner for the batched wavefront kernel.

The kernel's block size sets its per-block shared memory (per-thread
caches and accumulators) and so how many blocks share an SM; the number of
resident blocks per SM sets the persistent grid.  ``batch_config`` times a
few candidates on a sample batch drawn like the caller's (random states,
uneven pupil grids) and keeps the fastest, per device and plan shape, in
memory and in a small JSON file (``$BATOID_GB300_CACHE`` or
``~/.cache/batoid_gb300/autotune.json``).  ``BATOID_GB300_AUTOTUNE=0``
skips tuning and uses the default shape.
"""
import json
import os

import numpy as np
import torch

from . import _device as D
from . import _lib

DEFAULT = (256, 2)
CANDIDATES = [(128, 3), (128, 4), (256, 1), (256, 2)]
_memo = {}


def _cache_path():
    base = os.environ.get("BATOID_GB300_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "batoid_gb300")
    return os.path.join(base, "autotune.json")


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(table):
    try:
        p = _cache_path()
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
    except OSError:
        pass


def _key(pt):
    name = torch.cuda.get_device_name(D.device())
    return (f"{name}|k2|stages={pt.prog.nstages}|var={len(pt.var_stages)}|modes={pt.nmodes}|"
            f"fields={len(pt.fields)}|jmax={pt.jmax}")


def sample_batch(pt, nstates, nx_range=(32, 128), seed=0, scale=None):
    """Random states (dofs ~ U(-1,1) x scale), grid sizes and wavelengths."""
    rng = np.random.default_rng(seed)
    if scale is None:
        scale = np.concatenate([np.tile([1e-4, 1e-4, 1e-4, 1e-5, 1e-5], len(pt.rigid)),
                                np.full(pt.nmodes, 1e-8)])
    dofs = rng.uniform(-1.0, 1.0, (nstates, pt.ndof)) * scale
    nx = rng.integers(nx_range[0], nx_range[1] + 1, nstates)
    wl = rng.choice(np.linspace(350e-9, 1000e-9, 6), nstates)
    return dofs, nx, wl


def time_config(pt, inp, threads, ctas, reps=2):
    S, F, J = inp["nstates"], len(pt.fields), pt.jmax
    coefs = torch.empty(S * F * (J + 1), dtype=torch.float64, device=D.device())
    status = torch.empty(S * F, dtype=torch.int32, device=D.device())
    pt.launch(inp, coefs, status, threads, ctas)  # warm-up
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        pt.launch(inp, coefs, status, threads, ctas)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def batch_config(pt, nstates=384, force=False):
    """(threads, ctas_per_sm) for this plan on this device.  The sample must
    give every block many jobs (384 states x 9 fields: ~11 per block at 2
    blocks per SM); with only one or two jobs per block the makespan is the
    tail and favours fewer, longer-running blocks."""
    if os.environ.get("BATOID_GB300_AUTOTUNE", "1") == "0":
        return DEFAULT
    key = _key(pt)
    if not force and key in _memo:
        return _memo[key]
    table = _load()
    if not force and key in table:
        _memo[key] = tuple(table[key]["config"])
        return _memo[key]
    dofs, nx, wl = sample_batch(pt, nstates)
    pt.prepare(nx)
    inp = pt.device_inputs(dofs, nx, wl)
    timings = {}
    for threads, ctas in CANDIDATES:
        try:
            timings[(threads, ctas)] = time_config(pt, inp, threads, ctas)
        except _lib.BatoidError:
            continue
    if not timings:
        return DEFAULT
    best = min(timings, key=timings.get)
    _memo[key] = best
    table[key] = {"config": list(best), "ms": {f"{t}x{c}": v for (t, c), v in timings.items()}}
    _store(table)
    return best
