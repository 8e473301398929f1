"""Device accumulation of least-squares normal equations (fit.cu)."""
import numpy as np
import torch

from . import _device as D
from . import _lib


def normal_equations(x, y, values, basis, offsets=None):
    """B^T B and B^T v for basis arrays ``basis`` (jmax, side, side).

    With ``offsets`` (nfits+1 int64) the points are split into independent
    fits and G, b gain a leading fit axis.
    """
    jmax, side, _ = basis.shape
    dx = D.to_device(np.asarray(x, dtype=float).ravel())
    dy = D.to_device(np.asarray(y, dtype=float).ravel())
    dv = D.to_device(np.asarray(values, dtype=float).ravel())
    single = offsets is None
    if single:
        offsets = np.array([0, dx.numel()], dtype=np.int64)
    doff = torch.as_tensor(np.asarray(offsets, dtype=np.int64), device=D.device())
    nfits = len(offsets) - 1
    dbasis = D.to_device(np.ascontiguousarray(basis, dtype=float).ravel())
    G = D.empty(nfits * jmax * jmax)
    b = D.empty(nfits * jmax)
    _lib.check(_lib.lib().bt_zernike_normal_equations(
        D.ptr(dx), D.ptr(dy), D.ptr(dv), doff.data_ptr(), nfits, D.ptr(dbasis), jmax, side,
        D.ptr(G), D.ptr(b), D.stream_ptr()))
    G = D.to_host(G).reshape(nfits, jmax, jmax)
    b = D.to_host(b).reshape(nfits, jmax)
    if single:
        return G[0], b[0]
    return G, b
