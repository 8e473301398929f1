"""ORACLE — test infrastructure only.

numpy restatement of the surrogate MLP's forward and backward passes, for
the gradient check of the tensor-core kernels.  It rounds to bf16 exactly
where the device path stores bf16 (inputs, weights, hidden activations and
back-propagated gradients) and computes everything else in FP64, so its
results differ from the device's only by FP32 accumulation order.

Network: h_0 = x; z_l = h_{l-1} W_l^T + b_l; h_l = gelu(z_l) for the hidden
layers; y = h_L W_out^T + b_out.  Loss: mean over rows of
sum_j w_j (y_j - t_j)^2 over the target columns, plus err_weight times the
squared error of the error column against log ||y - t|| (detached).
"""
import numpy as np


def bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


S2PI = np.sqrt(2.0 / np.pi)


def gelu(z):
    """GELU, tanh form: 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))."""
    return 0.5 * z * (1.0 + np.tanh(S2PI * (z + 0.044715 * z ** 3)))


def dgelu(z):
    t = np.tanh(S2PI * (z + 0.044715 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * S2PI * (1.0 + 3 * 0.044715 * z * z)


def forward(x16, Ws, bs):
    """x16: bf16-valued inputs [B][in]; Ws: bf16-valued weights [out][in]."""
    hs, zs = [x16], []
    h = x16
    for W, b in zip(Ws[:-1], bs[:-1]):
        z = h @ W.T + b
        zs.append(z)
        h = bf16(gelu(z))
        hs.append(h)
    y = h @ Ws[-1].T + bs[-1]
    return y, zs, hs


def backward(y, t, w, zs, hs, Ws, ncols, err_col=-1, err_weight=0.0, rows_valid=None):
    """Gradients (dW, db) of every layer, same order as Ws."""
    B = y.shape[0] if rows_valid is None else rows_valid
    r = np.zeros_like(y)
    r[:B, :ncols] = y[:B, :ncols] - t[:B, :ncols]
    dy = np.zeros_like(y)
    dy[:B, :ncols] = 2.0 / B * w[:ncols] * r[:B, :ncols]
    if err_col >= 0:
        target = 0.5 * np.log(np.sum(r[:B, :ncols] ** 2, axis=1) + 1e-12)
        dy[:B, err_col] = 2.0 / B * err_weight * (y[:B, err_col] - target)
    dz = bf16(dy)
    dWs, dbs = [], []
    L = len(Ws)
    for l in range(L - 1, -1, -1):
        dWs.append(dz.T @ hs[l])
        dbs.append(dz.sum(axis=0))
        if l > 0:
            dh = dz @ Ws[l]
            dz = bf16(dh * dgelu(zs[l - 1]))
    return dWs[::-1], dbs[::-1]
