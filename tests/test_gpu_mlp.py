"""Tensor-core MLP kernels: GEMM epilogues against PyTorch FP32 references,
gradients against the numpy oracle, and a short training run."""
import numpy as np
import pytest
import torch

from batoid_gb300 import _device as D
from batoid_gb300 import _lib
from batoid_gb300.surrogate import MLP

pytestmark = pytest.mark.gpu

BF = torch.bfloat16


def _gemm(A, B, M, N, K, bn, mode, splitk=1, bias=None, out32=None, zs=None, h16=None, h16t=None):
    p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    _lib.check(_lib.lib().bt_mlp_gemm(p(A), p(B), M, N, K, bn, splitk, mode, p(bias), p(out32), p(zs), p(h16),
                                      p(h16t), D.stream_ptr()))
    torch.cuda.synchronize()


S2PI = np.sqrt(2.0 / np.pi)


def _gelu(z):
    return 0.5 * z * (1 + torch.tanh(S2PI * (z + 0.044715 * z ** 3)))


def _dgelu(z):
    t = torch.tanh(S2PI * (z + 0.044715 * z ** 3))
    return 0.5 * (1 + t) + 0.5 * z * (1 - t * t) * S2PI * (1 + 3 * 0.044715 * z * z)


@pytest.mark.parametrize("N,bn", [(256, 128), (512, 256)])
def test_gemm_epilogues(N, bn):
    dev = D.device()
    g = torch.Generator(device="cpu").manual_seed(N)
    M, K = 384, 192
    A = torch.randn(M, K, generator=g).to(dev).to(BF)
    B = torch.randn(N, K, generator=g).to(dev).to(BF)
    bias = torch.randn(N, generator=g).to(dev)
    ref = A.float() @ B.float().T
    tol = 1e-4 * ref.abs().max().item()
    out = torch.empty(M, N, device=dev)
    _gemm(A, B, M, N, K, bn, 0, out32=out)
    assert (out - ref).abs().max().item() <= tol
    parts = torch.empty(3, M, N, device=dev)
    _gemm(A, B, M, N, K, bn, 0, splitk=3, out32=parts)
    assert (parts.sum(0) - ref).abs().max().item() <= tol
    _gemm(A, B, M, N, K, bn, 1, bias=bias, out32=out)
    assert (out - (ref + bias)).abs().max().item() <= tol
    zs = torch.empty(M, N, device=dev)
    h16 = torch.empty(M, N, device=dev, dtype=BF)
    h16t = torch.empty(N, M, device=dev, dtype=BF)
    _gemm(A, B, M, N, K, bn, 2, bias=bias, zs=zs, h16=h16, h16t=h16t)
    assert (zs - (ref + bias)).abs().max().item() <= tol
    torch.testing.assert_close(h16, _gelu(zs).to(BF), rtol=1.6e-2, atol=1e-2)
    torch.testing.assert_close(h16t, h16.t().contiguous(), rtol=0, atol=0)
    zin = torch.randn(M, N, generator=g).to(dev)
    _gemm(A, B, M, N, K, bn, 3, zs=zin, h16=h16, h16t=h16t)
    torch.testing.assert_close(h16.float(), (ref * _dgelu(zin)), rtol=1.6e-2, atol=1e-2 * ref.abs().max().item())
    torch.testing.assert_close(h16t, h16.t().contiguous(), rtol=0, atol=0)


@pytest.mark.parametrize("bn", [128, 256])
def test_gemm_persistent_many_tiles(bn):
    """More tiles than SMs: every CTA walks several tiles, so both TMEM
    accumulators and the epilogue's staging tiles are reused."""
    dev = D.device()
    g = torch.Generator(device="cpu").manual_seed(bn + 7)
    M, N, K = 128 * 200, 512, 192
    A = torch.randn(M, K, generator=g).to(dev).to(BF)
    B = torch.randn(N, K, generator=g).to(dev).to(BF)
    bias = torch.randn(N, generator=g).to(dev)
    z = A.float() @ B.float().T + bias
    tol = 1e-4 * z.abs().max().item()
    zs = torch.empty(M, N, device=dev)
    h16 = torch.empty(M, N, device=dev, dtype=BF)
    h16t = torch.empty(N, M, device=dev, dtype=BF)
    _gemm(A, B, M, N, K, bn, 2, bias=bias, zs=zs, h16=h16, h16t=h16t)
    assert (zs - z).abs().max().item() <= tol
    torch.testing.assert_close(h16, _gelu(zs).to(BF), rtol=1.6e-2, atol=1e-2)
    torch.testing.assert_close(h16t, h16.t().contiguous(), rtol=0, atol=0)
    # inference form: no pre-activations, no transposed copy
    h2 = torch.zeros(M, N, device=dev, dtype=BF)
    _gemm(A, B, M, N, K, bn, 2, bias=bias, h16=h2)
    torch.testing.assert_close(h2, h16, rtol=0, atol=0)
    out = torch.empty(M, N, device=dev)
    _gemm(A, B, M, N, K, bn, 1, bias=bias, out32=out)
    assert (out - z).abs().max().item() <= tol


def test_gemm_rejects_bad_shapes():
    dev = D.device()
    A = torch.zeros(100, 64, device=dev, dtype=BF)
    B = torch.zeros(128, 64, device=dev, dtype=BF)
    out = torch.empty(100, 128, device=dev)
    with pytest.raises(_lib.BatoidError):
        _gemm(A, B, 100, 128, 64, 128, 0, out32=out)
    # split K only for the FP32 partials
    A = torch.zeros(128, 128, device=dev, dtype=BF)
    bias = torch.zeros(128, device=dev)
    out = torch.empty(128, 128, device=dev)
    with pytest.raises(_lib.BatoidError):
        _gemm(A, torch.zeros(128, 128, device=dev, dtype=BF), 128, 128, 128, 128, 1, splitk=2, bias=bias, out32=out)


def test_gradients_match_numpy_oracle():
    import mlp as omlp
    net = MLP(n_in=33, n_out=29, hidden=256, layers=2, seed=3)
    B = 256
    rng = np.random.default_rng(1)
    x = torch.from_numpy(rng.uniform(-1, 1, (B, 33)).astype(np.float32)).to(D.device())
    t = torch.from_numpy(rng.normal(0, 1, (B, 28)).astype(np.float32)).to(D.device())
    bf = net.pack(x, B, True)
    y = net.forward(bf, B, True)
    net.backward(bf, B, t, B, err_col=28, err_weight=0.1)
    torch.cuda.synchronize()
    dW, db = net.gradients(bf)
    # oracle on the same bf16 values
    x16 = omlp.bf16(np.pad(D.to_host(x), ((0, 0), (0, 128 - 33))))
    Ws = [D.to_host(w.float()) for w in net.W16]
    bs = [D.to_host(b) for b in net.b]
    yo, zs, hs = omlp.forward(x16, Ws, bs)
    np.testing.assert_allclose(D.to_host(y), yo, rtol=0, atol=2e-2 * np.abs(yo).max())
    tp = np.pad(D.to_host(t).astype(np.float64), ((0, 0), (0, 100)))
    gW, gb = omlp.backward(D.to_host(y).astype(np.float64), tp, np.ones(128), zs, hs, Ws, 28, 28, 0.1)
    for l in range(len(Ws)):
        err = np.linalg.norm(dW[l] - gW[l]) / np.linalg.norm(gW[l])
        errb = np.linalg.norm(db[l] - gb[l]) / np.linalg.norm(gb[l])
        print(f"layer {l}: dW rel err {err:.2e}, db rel err {errb:.2e}")
        assert err < 2e-2 and errb < 2e-2


def test_training_reduces_loss():
    net = MLP(n_in=8, n_out=4, hidden=256, layers=2, seed=0)
    B = 1024
    rng = np.random.default_rng(2)
    xs = rng.uniform(-1, 1, (B, 8)).astype(np.float32)
    ts = np.stack([np.sin(2 * xs[:, 0]) + xs[:, 1] * xs[:, 2], xs[:, 3] ** 2, np.cos(xs[:, 4] + xs[:, 5]),
                   xs[:, 6] - xs[:, 7]], axis=1).astype(np.float32)
    x = torch.from_numpy(xs).to(D.device())
    t = torch.from_numpy(ts).to(D.device())
    losses = []
    for it in range(300):
        bf = net.pack(x, B, True)
        net.forward(bf, B, True)
        net.backward(bf, B, t, B)
        net.adam(bf, 2e-3)
        if it in (0, 299):
            torch.cuda.synchronize()
            losses.append(float(bf["loss"][0].item()))
    assert losses[1] < 0.05 * losses[0]
    pred = D.to_host(net.predict(x))
    assert np.sqrt(np.mean((pred - ts) ** 2)) < 0.1

