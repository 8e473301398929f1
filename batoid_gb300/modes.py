"""Seeded smooth bending modes of a mirror, as bicubic height tables.

A mode is a sum of three seeded plane waves c cos(a x + b y + phi), sampled
with its analytic derivatives (z, dz/dx, dz/dy, d2z/dxdy) on a uniform grid
and normalised to unit RMS height over the mirror's clear aperture.  The
sampled values are rounded to FP32 once; those FP32 numbers define the
mode, for the device kernel and for every FP64 reference alike.

A bent surface z = sum_m a_m mode_m is the reference's Bicubic
(batoid/surface.py:521-663) of the summed tables; the batched kernel
evaluates the same patch from the weighted corner values.
"""
import numpy as np


class ModeSet:
    """``nmodes`` bending modes on an ``n`` x ``n`` grid over
    [-half_width, half_width]^2 (metres)."""

    def __init__(self, nmodes=20, n=512, half_width=4.4, r_aperture=4.18, seed=20240601):
        if nmodes % 4 != 0:
            raise ValueError("nmodes must be a multiple of 4")
        self.nmodes = nmodes
        self.n = n
        self.xs = np.linspace(-half_width, half_width, n)
        self.ys = self.xs.copy()
        self.x0 = self.xs[0]
        self.y0 = self.ys[0]
        # the grid step exactly as Bicubic derives it
        self.dx = (self.xs[-1] - self.xs[0]) / (n - 1)
        self.dy = (self.ys[-1] - self.ys[0]) / (n - 1)
        rng = np.random.default_rng(seed)
        X, Y = np.meshgrid(self.xs, self.ys)
        inside = X ** 2 + Y ** 2 <= r_aperture ** 2
        # [iy][ix][q][mode], q = z, dz/dx, dz/dy, d2z/dxdy
        tab = np.empty((n, n, 4, nmodes), dtype=np.float32)
        for m in range(nmodes):
            z = np.zeros_like(X)
            zx = np.zeros_like(X)
            zy = np.zeros_like(X)
            zxy = np.zeros_like(X)
            for _ in range(3):
                k = rng.uniform(0.3, 2.5)
                th = rng.uniform(0.0, 2 * np.pi)
                a, b = k * np.cos(th), k * np.sin(th)
                phi = rng.uniform(0.0, 2 * np.pi)
                c = rng.normal()
                arg = a * X + b * Y + phi
                co, si = np.cos(arg), np.sin(arg)
                z += c * co
                zx -= c * a * si
                zy -= c * b * si
                zxy -= c * a * b * co
            norm = 1.0 / np.sqrt(np.mean(z[inside] ** 2))
            for q, arr in enumerate((z, zx, zy, zxy)):
                tab[:, :, q, m] = arr * norm
        self.tables = tab
        self._device = None

    def device_tables(self):
        """The FP32 tables as a device tensor (kept by this object)."""
        if self._device is None:
            from . import _device as D
            import torch
            self._device = torch.from_numpy(np.ascontiguousarray(self.tables)).to(D.device())
        return self._device

    def summed(self, amps):
        """(z, dzdx, dzdy, d2zdxdy) of sum_m amps[m] * mode_m, in FP64."""
        amps = np.asarray(amps, dtype=np.float64)
        if amps.shape != (self.nmodes,):
            raise ValueError(f"expected {self.nmodes} amplitudes")
        return tuple(self.tables[:, :, q, :].astype(np.float64) @ amps for q in range(4))

    def bicubic(self, amps, bt=None):
        """The bent-surface term as a reference-API Bicubic (zero outside
        the grid)."""
        if bt is None:
            from . import surface as bt
        z, zx, zy, zxy = self.summed(amps)
        return bt.Bicubic(self.xs, self.ys, z, zx, zy, zxy, nanpolicy='zero')
