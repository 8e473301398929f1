"""Learned wavefront surrogate.

``MLP`` is a fully connected network trained and evaluated entirely by this
package's kernels: BF16 tensor-core GEMMs with FP32 accumulation
(tcgen05, ``bt_mlp_gemm``) with fused bias / GELU / GELU' epilogues, a fused
loss gradient, bias reductions and Adam.  Dimensions are padded to the
GEMM tiles: inputs and outputs to 128 columns, the batch to a multiple of
128 rows.

``WavefrontSurrogate`` maps perturbation dofs, field position and wavelength
to the 28 Zernike coefficients of ``PerturbedTelescope.zernike`` (no
counterpart in the reference): a linear sensitivity model per (field,
wavelength) plus the MLP on its residual, with an error head whose
prediction decides when to fall back to the batched trace.
"""
import numpy as np
import torch

from . import _device as D
from . import _lib

PAD = 128


def _bf16(shape):
    return torch.empty(shape, dtype=torch.bfloat16, device=D.device())


def _f32(shape, zero=False):
    f = torch.zeros if zero else torch.empty
    return f(shape, dtype=torch.float32, device=D.device())


def _p(t):
    return None if t is None else t.data_ptr()


class MLP:
    """n_in -> hidden x layers (GELU) -> n_out, BF16 weights/activations with
    FP32 accumulation; FP32 master weights and Adam moments."""

    def __init__(self, n_in=33, n_out=29, hidden=512, layers=4, seed=0):
        if hidden % 256:
            raise ValueError("hidden width must be a multiple of 256")
        if n_in > PAD or n_out > PAD:
            raise ValueError("at most 128 inputs and outputs")
        self.n_in, self.n_out, self.hidden, self.layers = n_in, n_out, hidden, layers
        rng = np.random.default_rng(seed)
        dims = [PAD] + [hidden] * layers + [PAD]
        self.shapes = [(dims[i + 1], dims[i]) for i in range(len(dims) - 1)]
        self.W, self.b, self.W16, self.W16t, self.mW, self.vW, self.mb, self.vb = ([] for _ in range(8))
        for li, (o, i) in enumerate(self.shapes):
            fan_in = n_in if li == 0 else i
            w = rng.normal(0.0, np.sqrt(2.0 / fan_in), (o, i)).astype(np.float32)
            if li == 0:
                w[:, n_in:] = 0.0
            if li == len(self.shapes) - 1:
                w *= 0.1
                w[n_out:, :] = 0.0
            self.W.append(torch.from_numpy(w).to(D.device()))
            self.W16.append(self.W[-1].to(torch.bfloat16).contiguous())
            self.W16t.append(self.W[-1].t().contiguous().to(torch.bfloat16))
            self.mW.append(_f32((o, i), zero=True))
            self.vW.append(_f32((o, i), zero=True))
        # biases, their moments (and, per buffer set, their gradients) are
        # views of one flat array each: one Adam launch updates all biases
        self._boff = [0] + [int(x) for x in np.cumsum([o for o, _ in self.shapes])]
        self.b_flat, self.mb_flat, self.vb_flat = (_f32(self._boff[-1], zero=True) for _ in range(3))
        self.b, self.mb, self.vb = ([f[self._boff[l]:self._boff[l + 1]] for l in range(len(self.shapes))]
                                    for f in (self.b_flat, self.mb_flat, self.vb_flat))
        self.step_count = 0
        self._bufs = {}

    # -- buffers ---------------------------------------------------------------
    def _buffers(self, B, train):
        key = (B, train)
        if key not in self._bufs:
            H = self.hidden
            bf = {"x16": _bf16((B, PAD)), "y": _f32((B, PAD)),
                  "h16": [_bf16((B, H)) for _ in range(self.layers)]}
            if train:
                bf["x16t"] = _bf16((PAD, B))
                bf["zs"] = [_f32((B, H)) for _ in range(self.layers)]
                bf["h16t"] = [_bf16((H, B)) for _ in range(self.layers)]
                bf["dz"] = [_bf16((B, H)) for _ in range(self.layers)] + [_bf16((B, PAD))]
                bf["dzt"] = [_bf16((H, B)) for _ in range(self.layers)] + [_bf16((PAD, B))]
                bf["db_flat"] = _f32(self._boff[-1])
                bf["db"] = [bf["db_flat"][self._boff[l]:self._boff[l + 1]] for l in range(len(self.shapes))]
                bf["loss"] = _f32(2, zero=True)
                splits = [self._splitk(o, i, B) for o, i in self.shapes]
                bf["splits"] = splits
                bf["ws"] = [_f32((s, o, i)) for s, (o, i) in zip(splits, self.shapes)]
            self._bufs[key] = bf
        return self._bufs[key]

    @staticmethod
    def _bn(n):
        return 256 if n % 256 == 0 else 128

    def _splitk(self, o, i, B):
        tiles = (o // 128) * (i // self._bn(i))
        s = 1
        while tiles * s * 2 <= 160 and B % (64 * s * 2) == 0 and B // (s * 2) >= 128:
            s *= 2
        return s

    def _gemm(self, A, Bm, M, N, K, mode, bias=None, out32=None, zs=None, h16=None, h16t=None, splitk=1):
        _lib.check(_lib.lib().bt_mlp_gemm(_p(A), _p(Bm), M, N, K, self._bn(N), splitk, mode, _p(bias), _p(out32),
                                          _p(zs), _p(h16), _p(h16t), D.stream_ptr()))

    # -- passes --------------------------------------------------------------------
    def pack(self, x, B, train):
        """x: FP32 device tensor [n <= B][n_in] -> padded bf16 inputs."""
        bf = self._buffers(B, train)
        _lib.check(_lib.lib().bt_mlp_pack(_p(x), x.shape[0], x.shape[1], PAD, B, _p(bf["x16"]),
                                          _p(bf.get("x16t")), D.stream_ptr()))
        return bf

    def forward(self, bf, B, train):
        h = bf["x16"]
        for l in range(self.layers):
            o, i = self.shapes[l]
            self._gemm(h, self.W16[l], B, o, i, 2, bias=self.b[l], zs=bf["zs"][l] if train else None,
                       h16=bf["h16"][l], h16t=bf["h16t"][l] if train else None)
            h = bf["h16"][l]
        o, i = self.shapes[-1]
        self._gemm(h, self.W16[-1], B, o, i, 1, bias=self.b[-1], out32=bf["y"])
        return bf["y"]

    def backward(self, bf, B, t, rows_valid, wt=None, err_col=-1, err_weight=0.0):
        """Gradients of the loss into the split-K workspaces and bias buffers."""
        L = _lib.lib()
        s = D.stream_ptr()
        bf["loss"].zero_()
        ncols = t.shape[1]
        _lib.check(L.bt_mlp_loss(_p(bf["y"]), PAD, _p(t), _p(wt), B, rows_valid, ncols, err_col, float(err_weight),
                                 PAD, _p(bf["dz"][-1]), _p(bf["dzt"][-1]), _p(bf["loss"]), s))
        nl = len(self.shapes)
        for l in range(nl - 1, -1, -1):
            o, i = self.shapes[l]
            hin_t = bf["x16t"] if l == 0 else bf["h16t"][l - 1]
            # dW_l = dz_l^T . h_{l-1}
            self._gemm(bf["dzt"][l], hin_t, o, i, B, 0, out32=bf["ws"][l], splitk=bf["splits"][l])
            _lib.check(L.bt_mlp_colsum(_p(bf["dzt"][l]), o, B, _p(bf["db"][l]), s))
            if l > 0:
                # dz_{l-1} = (dz_l . W_l) * gelu'(z_{l-1})
                self._gemm(bf["dz"][l], self.W16t[l], B, i, o, 3, zs=bf["zs"][l - 1], h16=bf["dz"][l - 1],
                           h16t=bf["dzt"][l - 1])

    def adam(self, bf, lr, b1=0.9, b2=0.999, eps=1e-8, hyper=None):
        """One Adam step.  hyper: optional device FP32 tensor {lr, bc1, bc2}
        read by the kernels when they run (a captured step then follows a
        schedule computed on the device); lr is ignored then."""
        L = _lib.lib()
        s = D.stream_ptr()
        if hyper is not None:
            for l, (o, i) in enumerate(self.shapes):
                _lib.check(L.bt_mlp_adam_dev(_p(bf["ws"][l]), bf["splits"][l], None, o * i, _p(self.W[l]),
                                             _p(self.mW[l]), _p(self.vW[l]), _p(hyper), b1, b2, eps, o, i,
                                             _p(self.W16[l]), _p(self.W16t[l]), s))
            nb = self._boff[-1]
            _lib.check(L.bt_mlp_adam_dev(None, 0, _p(bf["db_flat"]), nb, _p(self.b_flat), _p(self.mb_flat),
                                         _p(self.vb_flat), _p(hyper), b1, b2, eps, 1, nb, None, None, s))
            return
        self.step_count += 1
        bc1 = 1.0 - b1 ** self.step_count
        bc2 = 1.0 - b2 ** self.step_count
        for l, (o, i) in enumerate(self.shapes):
            _lib.check(L.bt_mlp_adam(_p(bf["ws"][l]), bf["splits"][l], None, o * i, _p(self.W[l]), _p(self.mW[l]),
                                     _p(self.vW[l]), lr, b1, b2, eps, bc1, bc2, o, i, _p(self.W16[l]),
                                     _p(self.W16t[l]), s))
        nb = self._boff[-1]
        _lib.check(L.bt_mlp_adam(None, 0, _p(bf["db_flat"]), nb, _p(self.b_flat), _p(self.mb_flat), _p(self.vb_flat),
                                 lr, b1, b2, eps, bc1, bc2, 1, nb, None, None, s))

    def gradients(self, bf):
        """(dW, db) lists as host arrays (split-K partials summed)."""
        dW = [D.to_host(w.sum(dim=0)) for w in bf["ws"]]
        db = [D.to_host(b) for b in bf["db"]]
        return dW, db

    def predict(self, x, B=None):
        """FP32 outputs [n][n_out] for FP32 inputs x [n][n_in] (device)."""
        n = x.shape[0]
        Bp = B or ((n + 127) // 128) * 128
        bf = self.pack(x, Bp, False)
        y = self.forward(bf, Bp, False)
        return y[:n, :self.n_out]


class WavefrontSurrogate:
    """Zernike coefficients of a ``PerturbedTelescope`` from its dofs, field
    and wavelength, with the batched trace as fallback and ground truth.

    Model: c = c_lin + r, with c_lin a least-squares linear model in the
    normalised dofs per (field, wavelength) and r (in nm / scale) predicted
    by the MLP from all 33 normalised inputs.  The MLP's extra output
    predicts log of the residual norm; ``calibrate`` turns it into a
    conservative error estimate, and samples whose estimate exceeds the
    threshold are traced instead.
    """

    DOF_SCALE_RIGID = np.array([1e-3, 1e-3, 1e-3, np.deg2rad(10 / 3600), np.deg2rad(10 / 3600)])

    def __init__(self, pt, wavelengths, nx=32, hidden=512, layers=4, seed=0):
        self.pt = pt
        self.wavelengths = np.asarray(wavelengths, dtype=float)
        self.nx = int(nx)
        self.J = pt.jmax
        self.F = len(pt.fields)
        self.dof_scale = np.concatenate([np.tile(self.DOF_SCALE_RIGID, len(pt.rigid)), np.full(pt.nmodes, 100e-9)])
        self.field_scale = max(np.abs(pt.fields).max(), 1e-12)
        self.net = MLP(n_in=pt.ndof + 3, n_out=self.J + 1, hidden=hidden, layers=layers, seed=seed)
        self.theta = None
        self.scale = 1.0
        self.kappa = 1.0
        self.guard = None

    # -- data ----------------------------------------------------------------------
    def sample_states(self, nstates, seed, widen=1.0):
        """Seeded states: rigid dofs uniform within +-1 mm / +-10 arcsec,
        bending amplitudes N(0, 100 nm), wavelength index uniform.  `widen`
        scales both ranges (training on a wider distribution than the one
        evaluated keeps its tails inside the training support)."""
        rng = np.random.default_rng(seed)
        nr = 5 * len(self.pt.rigid)
        dofs = np.empty((nstates, self.pt.ndof))
        dofs[:, :nr] = rng.uniform(-widen, widen, (nstates, nr)) * self.dof_scale[:nr]
        dofs[:, nr:] = rng.normal(0.0, 100e-9 * widen, (nstates, self.pt.nmodes))
        widx = rng.integers(0, len(self.wavelengths), nstates)
        return dofs, widx

    def trace(self, dofs, widx, chunk=16384, threads=None, ctas_per_sm=None):
        """Batched-trace coefficients (S, F, J+1) of states (the ground truth)."""
        out = []
        for a in range(0, len(dofs), chunk):
            out.append(self.pt.zernike(dofs[a:a + chunk], self.nx, self.wavelengths[widx[a:a + chunk]],
                                       threads=threads, ctas_per_sm=ctas_per_sm))
        return np.concatenate(out)

    def features(self, dofs, widx):
        """Per-(state, field) network inputs (S*F, ndof+3), group ids and
        wavelengths, state-major."""
        S, F = len(dofs), self.F
        d = np.repeat(dofs / self.dof_scale, F, axis=0)
        fxy = np.tile(self.pt.fields / self.field_scale, (S, 1))
        w = np.repeat(self.wavelengths[widx], F)
        wn = (w - self.wavelengths.mean()) / max(np.ptp(self.wavelengths) / 2, 1e-30)
        feat = np.concatenate([d, fxy, wn[:, None]], axis=1).astype(np.float32)
        grp = (np.tile(np.arange(F), S) * len(self.wavelengths) + np.repeat(widx, F)).astype(np.int32)
        return feat, grp, w

    # -- fit -------------------------------------------------------------------------
    def fit_linear(self, feat, grp, coefs):
        """Least-squares linear model per (field, wavelength) group."""
        nd = self.pt.ndof
        G = self.F * len(self.wavelengths)
        c = coefs.reshape(-1, self.J + 1)[:, 1:]
        self.theta = np.zeros((G, nd + 1, self.J))
        self._theta_d = None  # device copy rebuilt on the next prediction
        for g in range(G):
            sel = grp == g
            if not np.any(sel):
                continue
            A = np.concatenate([np.ones((sel.sum(), 1)), feat[sel, :nd].astype(np.float64)], axis=1)
            # normal equations: the scaled features keep A^T A well
            # conditioned (ones column and unit-range inputs)
            try:
                self.theta[g] = np.linalg.solve(A.T @ A, A.T @ c[sel])
            except np.linalg.LinAlgError:
                self.theta[g] = np.linalg.lstsq(A, c[sel], rcond=None)[0]

    def linear(self, feat, grp):
        nd = self.pt.ndof
        out = np.empty((len(grp), self.J))
        for g in np.unique(grp):
            sel = grp == g
            out[sel] = self.theta[g, 0, :] + feat[sel, :nd].astype(np.float64) @ self.theta[g, 1:, :]
        return out

    def residual_targets(self, feat, grp, w, coefs):
        """Residual of the linear model in nm / scale."""
        r = (coefs.reshape(-1, self.J + 1)[:, 1:] - self.linear(feat, grp)) * w[:, None] * 1e9
        return r

    def _fit_linear_sorted(self, feat, grp, w, coefs):
        """fit_linear and residual_targets in one pass over the samples
        sorted by group (contiguous slices instead of a mask per group):
        each group's normal equations by one FP64 product, the
        (ndof+1)-sized systems solved directly.  Returns the residuals (nm)
        as a device tensor."""
        nd = self.pt.ndof
        G = self.F * len(self.wavelengths)
        order = np.argsort(grp, kind="stable")
        counts = np.bincount(grp, minlength=G)
        starts = np.concatenate([[0], np.cumsum(counts)])
        A = np.empty((len(feat), nd + 1))
        A[:, 0] = 1.0
        A[:, 1:] = feat[order, :nd]
        C = coefs.reshape(-1, self.J + 1)[order, 1:]
        self.theta = np.zeros((G, nd + 1, self.J))
        self._theta_d = None
        R = np.empty_like(C)
        for k in range(G):
            if not counts[k]:
                continue
            sl = slice(starts[k], starts[k + 1])
            a, c = A[sl], C[sl]
            try:
                self.theta[k] = np.linalg.solve(a.T @ a, a.T @ c)
            except np.linalg.LinAlgError:
                self.theta[k] = np.linalg.lstsq(a, c, rcond=None)[0]
            R[sl] = (c - a @ self.theta[k]) * w[order[sl], None] * 1e9
        r = np.empty_like(R)
        r[order] = R
        return torch.from_numpy(r).to(D.device())

    def train(self, feat, grp, w, coefs, epochs=30, batch=8192, lr=1e-3, lr_min=1e-5, err_weight=0.05, seed=0,
              log=None, graph=True):
        """Fits the linear model, then trains the MLP on its residuals.

        graph: each training step (minibatch gather, forward, loss,
        backward, Adam with the cosine learning-rate schedule and bias
        corrections computed on the device) is captured once in a CUDA
        graph and replayed; the step's ~30 launches then cost one graph
        launch.  graph=False issues them one by one (same arithmetic).

        Minibatches are drawn from a device permutation per epoch (seeded
        generator).  self.timing afterwards holds the wall time of the
        linear fit (host, samples sorted by group) and of the network
        training (device steps)."""
        import time
        t0 = time.perf_counter()
        r = self._fit_linear_sorted(feat, grp, w, coefs)
        self.scale = float(torch.sqrt(torch.mean(r * r)).item())
        t_all = (r / self.scale).float().contiguous()
        del r
        x_all = torch.from_numpy(feat).to(D.device())
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        n = len(feat)
        steps_per_epoch = n // batch
        total = epochs * steps_per_epoch
        gen = torch.Generator(device=D.device())
        gen.manual_seed(seed)

        def perm_of_epoch():
            return torch.randperm(n, generator=gen, device=D.device())[:steps_per_epoch * batch]

        if graph and steps_per_epoch > 0:
            self._train_graph(x_all, t_all, epochs, steps_per_epoch, batch, lr, lr_min, err_weight, perm_of_epoch,
                              log)
        else:
            self._train_eager(x_all, t_all, epochs, steps_per_epoch, batch, lr, lr_min, err_weight, perm_of_epoch,
                              log)
        self.timing = {"linear_fit_s": t1 - t0, "network_s": time.perf_counter() - t1,
                       "steps": total, "samples": total * batch}

    def _train_eager(self, x_all, t_all, epochs, steps_per_epoch, batch, lr, lr_min, err_weight, perm_of_epoch, log):
        total = epochs * steps_per_epoch
        step = 0
        for ep in range(epochs):
            perm = perm_of_epoch()
            for k in range(steps_per_epoch):
                idx = perm[k * batch:(k + 1) * batch]
                x = x_all.index_select(0, idx)
                t = t_all.index_select(0, idx)
                bf = self.net.pack(x, batch, True)
                self.net.forward(bf, batch, True)
                self.net.backward(bf, batch, t, batch, err_col=self.J, err_weight=err_weight)
                cur = lr_min + 0.5 * (lr - lr_min) * (1 + np.cos(np.pi * step / max(total, 1)))
                self.net.adam(bf, float(cur))
                step += 1
            if log is not None:
                torch.cuda.synchronize()
                log(ep, float(bf["loss"][0].item()), float(bf["loss"][1].item()))
        torch.cuda.synchronize()

    def _train_graph(self, x_all, t_all, epochs, steps_per_epoch, batch, lr, lr_min, err_weight, perm_of_epoch, log,
                     b1=0.9, b2=0.999):
        net, dev = self.net, D.device()
        total = epochs * steps_per_epoch
        perm = torch.empty((steps_per_epoch, batch), dtype=torch.int64, device=dev)
        k_in_epoch = torch.zeros(1, dtype=torch.int64, device=dev)
        step = torch.zeros(1, dtype=torch.int64, device=dev)
        # {lr, bc1, bc2} of every step, as the launch-by-launch path computes them
        g = np.arange(max(total, 1), dtype=np.float64)
        table = np.stack([lr_min + 0.5 * (lr - lr_min) * (1.0 + np.cos(np.pi * g / max(total, 1))),
                          1.0 - b1 ** (g + 1), 1.0 - b2 ** (g + 1)], axis=1).astype(np.float32)
        table_d = torch.from_numpy(table.ravel()).to(dev)
        hyper = torch.empty(3, dtype=torch.float32, device=dev)
        xb = torch.empty((batch, x_all.shape[1]), dtype=torch.float32, device=dev)
        tb = torch.empty((batch, t_all.shape[1]), dtype=torch.float32, device=dev)

        L = _lib.lib()
        nxc, ntc = x_all.shape[1], t_all.shape[1]

        def body():
            # minibatch gather, network step, then this step's learning rate
            # and Adam bias corrections from the table (advancing both step
            # counters) and Adam
            _lib.check(L.bt_mlp_gather(perm.data_ptr(), k_in_epoch.data_ptr(), x_all.data_ptr(), nxc, t_all.data_ptr(),
                                       ntc, batch, xb.data_ptr(), tb.data_ptr(), D.stream_ptr()))
            bf = net.pack(xb, batch, True)
            net.forward(bf, batch, True)
            net.backward(bf, batch, tb, batch, err_col=self.J, err_weight=err_weight)
            _lib.check(L.bt_mlp_schedule(k_in_epoch.data_ptr(), step.data_ptr(), table_d.data_ptr(), max(total, 1),
                                         hyper.data_ptr(), D.stream_ptr()))
            net.adam(bf, 0.0, b1=b1, b2=b2, hyper=hyper)
            return bf

        stream = torch.cuda.Stream()
        stream.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            done = 0
            for ep in range(epochs):
                perm.copy_(perm_of_epoch().view(steps_per_epoch, batch))
                k_in_epoch.zero_()
                for k in range(steps_per_epoch):
                    if done == 0:
                        bf = body()  # eager first step: buffers, kernel attributes
                        stream.synchronize()
                        with torch.cuda.graph(g, stream=stream):
                            body()
                        # the capture queued no work: undo nothing, count the eager step
                    else:
                        g.replay()
                    done += 1
                if log is not None:
                    stream.synchronize()
                    log(ep, float(bf["loss"][0].item()), float(bf["loss"][1].item()))
        net.step_count += done
        torch.cuda.current_stream().wait_stream(stream)
        torch.cuda.synchronize()

    # -- inference ------------------------------------------------------------------------
    def predict_device(self, feat_d, grp_d, w_d, out=None, err=None):
        """Device path: coefficients (n, J+1) in waves and predicted error
        in nm (before calibration), all on the device."""
        n = feat_d.shape[0]
        y = self.net.predict(feat_d)
        if out is None:
            out = torch.empty((n, self.J + 1), dtype=torch.float64, device=D.device())
        if err is None:
            err = torch.empty(n, dtype=torch.float32, device=D.device())
        if not hasattr(self, "_theta_d") or self._theta_d is None:
            # float-float pairs (hi, lo) of the FP64 linear model
            th = np.ascontiguousarray(self.theta.ravel(), dtype=np.float64)
            hi = th.astype(np.float32)
            lo = (th - hi.astype(np.float64)).astype(np.float32)
            self._theta_d = torch.from_numpy(np.stack([hi, lo], axis=1).ravel()).to(D.device())
        _lib.check(_lib.lib().bt_surrogate_combine(_p(feat_d), feat_d.shape[1], self.pt.ndof, _p(grp_d),
                                                   _p(self._theta_d), y.data_ptr(), PAD, _p(w_d), self.scale, self.J,
                                                   self.J, _p(out), _p(err), n, D.stream_ptr()))
        return out, err

    def predict(self, feat, grp, w):
        feat_d = torch.from_numpy(feat).to(D.device())
        grp_d = torch.from_numpy(grp).to(D.device())
        w_d = D.to_device(w)
        out, err = self.predict_device(feat_d, grp_d, w_d)
        return D.to_host(out), D.to_host(err)

    def build_guard(self, **kw):
        """The vignetting guard of this surrogate's pupil grid, fields and
        wavelengths (vignetting.VignettingGuard): samples whose dofs may
        move a grid ray across an aperture edge fall back to the trace."""
        from .vignetting import VignettingGuard
        self.guard = VignettingGuard(self.pt, self.wavelengths, self.nx, self.dof_scale, **kw)
        return self.guard

    def guard_flags(self, feat, grp):
        """Host bool flags of the vignetting guard (all False without one)."""
        if self.guard is None:
            return np.zeros(len(feat), dtype=bool)
        f = self.guard.flags_device(torch.from_numpy(feat).to(D.device()), torch.from_numpy(grp).to(D.device()))
        return D.to_host(f).astype(bool)

    def calibrate(self, feat, grp, w, coefs, quantile=0.99, threshold_nm=2.0):
        """Safety factor on the predicted error: the given quantile of
        actual / predicted over a validation set (the samples the vignetting
        guard does not already send to the trace).  With a guard, its
        margins whose crossings do not coincide with errors above
        threshold_nm on this set are pruned first (VignettingGuard.prune)."""
        pred, err = self.predict(feat, grp, w)
        actual = rms_nm(pred, coefs.reshape(-1, self.J + 1), w)
        if self.guard is not None:
            dofs = feat[:, :self.pt.ndof].astype(np.float64) * self.dof_scale
            self.guard.prune(dofs, grp, actual > threshold_nm)
        keep = ~self.guard_flags(feat, grp)
        if not np.any(keep):
            keep[:] = True
        self.kappa = float(np.quantile(actual[keep] / np.maximum(err[keep], 1e-6), quantile))
        return self.kappa

    def with_fallback(self, dofs, widx, threshold_nm=2.0, threads=None, ctas_per_sm=None):
        """(coefs (S, F, J+1), traced mask (S, F)): surrogate where its
        calibrated error estimate is within the threshold and the vignetting
        guard (when built) sees no aperture crossing, batched trace
        elsewhere."""
        feat, grp, w = self.features(dofs, widx)
        pred, err = self.predict(feat, grp, w)
        S, F = len(dofs), self.F
        fb = ((self.kappa * err > threshold_nm) | self.guard_flags(feat, grp)).reshape(S, F)
        out = pred.reshape(S, F, self.J + 1)
        if np.any(fb):
            traced = self.trace_jobs(dofs, widx, np.flatnonzero(fb.ravel()), threads, ctas_per_sm)
            out = out.copy()
            out.reshape(S * F, -1)[fb.ravel()] = traced.reshape(S * F, -1)[fb.ravel()]
        return out, fb

    def trace_jobs(self, dofs, widx, jobs, threads=None, ctas_per_sm=None):
        """Batched trace of only the given (state * F + field) jobs; other
        rows of the result are NaN."""
        pt = self.pt
        S, F, J = len(dofs), self.F, self.J
        pt.prepare([self.nx])
        if threads is None or ctas_per_sm is None:
            from .autotune import batch_config
            threads, ctas_per_sm = batch_config(pt)
        inp = pt.device_inputs(dofs, self.nx, self.wavelengths[widx])
        order = torch.from_numpy(np.asarray(jobs, dtype=np.int32)).to(D.device())
        coefs = torch.full((S * F * (J + 1),), float("nan"), dtype=torch.float64, device=D.device())
        status = torch.empty(S * F, dtype=torch.int32, device=D.device())
        pt.launch(inp, coefs, status, threads, ctas_per_sm, order=order)
        return D.to_host(coefs).reshape(S, F, J + 1)


def rms_nm(pred, truth, w):
    """RMS wavefront difference (nm) of coefficient rows (waves), piston
    excluded: the basis is orthonormal over the annulus."""
    d = (pred[:, 2:] - truth[:, 2:]) * w[:, None] * 1e9
    return np.sqrt(np.sum(d ** 2, axis=1))
