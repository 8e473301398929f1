"""First-order model of the vignetting of a pupil grid under small
perturbations: the surrogate's guard against vignetting changes.

The batched wavefront fit (``PerturbedTelescope.zernike``) uses the pupil
rays that are not vignetted.  When a perturbation moves one grid ray across
an aperture edge, that ray joins or leaves the fit and the coefficients
jump; a smooth surrogate cannot follow the jump.  A ray's vignetting by an
aperture depends on its signed distance to the aperture's edge on that
surface (its margin: positive when clear), and the margin is a smooth
function of the perturbation.  ``VignettingGuard`` traces the nominal grid
of every (field, wavelength) group once and with each dof stepped both ways
(central differences), and keeps, per group, the (surface, ray) margins
that could cross zero inside the dof ranges: m(d) = m0 + J d.  A sample is
flagged when any of its group's kept margins, predicted at its dofs, has
changed sign or lies within a band of zero (band_abs, 1 nm, plus band_rel
of the predicted change: the model's second-order error scales with the
change), or when a dof
lies outside the ranges the margins were chosen for
(``bt_surrogate_guard``, one warp per sample on the device).

Not every crossing matters: a grid ray that sits on an aperture edge in the
nominal state (a grid point at the pupil's rim) flips with nanometre
motions in almost every state, and the training data already sample both
of its states.  ``prune`` drops the margins whose crossings, over a
validation set, almost never coincide with a surrogate error above the
threshold, as the error head's safety factor is calibrated on the same set.

Margins follow the obscuration tree: a circle obscures its inside (margin
r - R), an annulus obscures inner <= r < outer (margin max(inner - r,
r - outer)), a negation flips the sign, a union takes the minimum (clear
only where every part is), an intersection the maximum.  Rectangles, rays
and polygons are not modelled (``NotImplementedError``).
"""
import numpy as np

from . import _device as D
from . import _lib


def obscuration_margin(obsc, x, y):
    """Signed distance to the edge of the clear region (m; > 0 clear) of an
    obscuration at local points (x, y); +inf where there is no obscuration."""
    from .obscuration import ObscAnnulus, ObscCircle, ObscIntersection, ObscNegation, ObscUnion
    if obsc is None:
        return np.full(np.shape(x), np.inf)
    if isinstance(obsc, ObscCircle):
        return np.hypot(x - obsc.x, y - obsc.y) - obsc.radius
    if isinstance(obsc, ObscAnnulus):
        r = np.hypot(x - obsc.x, y - obsc.y)
        return np.maximum(obsc.inner - r, r - obsc.outer)
    if isinstance(obsc, ObscNegation):
        return -obscuration_margin(obsc.original, x, y)
    if isinstance(obsc, ObscUnion):
        return np.min([obscuration_margin(o, x, y) for o in obsc.items], axis=0)
    if isinstance(obsc, ObscIntersection):
        return np.max([obscuration_margin(o, x, y) for o in obsc.items], axis=0)
    raise NotImplementedError(f"no margin model for {type(obsc).__name__}")


def select_constraints(m0, jac, scale, widen=1.2, band_abs=2e-6):
    """Margins that can cross zero inside the dof ranges.

    m0 : (S, N) nominal margins of S surfaces x N rays (inf: no aperture,
        NaN: the ray failed); jac : (S, N, ndof) their derivatives per unit
        of each normalised dof; scale : (ndof,) the reach of each dof
        (e.g. 1 for uniform dofs on [-1, 1], several sigma for Gaussian
        ones).  A (surface, ray) margin is kept when |m0| < widen * sum |J|
        scale + band_abs, unless the ray is vignetted for sure by another
        surface (a negative margin that cannot cross zero) or failed.
    Returns (surface index, ray index) arrays of the kept margins."""
    m0 = np.asarray(m0, dtype=float)
    reach = np.abs(jac) @ np.asarray(scale, dtype=float)
    finite = np.isfinite(m0)
    near = finite & (np.abs(np.where(finite, m0, 0.0)) < widen * reach + band_abs)
    sure_vig = np.any(finite & ~near & (m0 < 0), axis=0)
    failed = np.any(np.isnan(m0), axis=0)
    keep = near & ~sure_vig[None, :] & ~failed[None, :]
    s, i = np.nonzero(keep)
    return s, i


class VignettingGuard:
    """Kept margins of every (field, wavelength) group of a
    ``PerturbedTelescope`` pupil grid and their dof derivatives.

    groups follow the surrogate's numbering g = field * nwavelengths +
    wavelength index.  dof_scale converts dofs to the surrogate's
    normalised features; reach gives each normalised dof's range for the
    selection (defaults: 1 for rigid dofs, uniform on [-1, 1]; 5 for
    bending amplitudes, Gaussian with unit sigma)."""

    def __init__(self, pt, wavelengths, nx, dof_scale, reach=None, band_abs=1e-9, band_rel=0.05, widen=1.2):
        self.pt = pt
        self.wavelengths = np.asarray(wavelengths, dtype=float)
        self.nx = int(nx)
        self.dof_scale = np.asarray(dof_scale, dtype=float)
        nd = pt.ndof
        if reach is None:
            reach = np.concatenate([np.ones(5 * len(pt.rigid)), np.full(pt.nmodes, 5.0)])
        self.reach = np.asarray(reach, dtype=float)
        self.band_abs, self.band_rel = float(band_abs), float(band_rel)
        F, Wn = len(pt.fields), len(self.wavelengths)
        self.G = F * Wn
        rays = self._grid_rays()
        m0 = self._margins(pt.perturbed(np.zeros(nd)), rays)  # (S, G*N)
        jac = np.empty(m0.shape + (nd,))
        for d in range(nd):
            step = np.zeros(nd)
            step[d] = self.dof_scale[d]
            mp = self._margins(pt.perturbed(step), rays)
            mm = self._margins(pt.perturbed(-step), rays)
            with np.errstate(invalid="ignore"):
                jac[..., d] = np.where(np.isfinite(m0), 0.5 * (mp - mm), 0.0)
        # a ray that fails under a step: no first-order model; its margins
        # keep their nominal value (such rays are rejected by the fit anyway)
        jac = np.nan_to_num(jac, nan=0.0, posinf=0.0, neginf=0.0)
        N = self.nx * self.nx
        S = m0.shape[0]
        per = []
        for g in range(self.G):
            sl = slice(g * N, (g + 1) * N)
            s, i = select_constraints(m0[:, sl], jac[:, sl, :], reach, widen=widen, band_abs=band_abs)
            per.append((m0[s, g * N + i], jac[s, g * N + i, :], s, i))
        K = max([len(p[0]) for p in per] + [1])
        self.K = ((K + 31) // 32) * 32
        self.m0 = np.full((self.G, self.K), np.inf)
        self.jac = np.zeros((self.G, nd, self.K))
        self.where = []
        for g, (mg, jg, s, i) in enumerate(per):
            self.m0[g, :len(mg)] = mg
            self.jac[g, :, :len(mg)] = jg.T
            self.where.append((s, i))
        self.nkept = np.array([len(p[0]) for p in per])
        self.nsurf = S
        self._dev = None

    # -- host side ------------------------------------------------------------------------
    def _grid_rays(self):
        """Pupil grid rays of every group, concatenated (group-major), as the
        batched kernel generates them (RayVector.asGrid on the nominal optic)."""
        from .rayVector import RayVector
        pt, o = self.pt, self.pt.optic
        parts = []
        for tx, ty in pt.fields:
            for w in self.wavelengths:
                parts.append(RayVector.asGrid(optic=o, wavelength=w, theta_x=tx, theta_y=ty,
                                              projection=pt.projection, nx=self.nx))
        cols = [np.concatenate([getattr(p, a) for p in parts]) for a in
                ("x", "y", "z", "vx", "vy", "vz", "t", "wavelength", "flux")]
        return RayVector(*cols, coordSys=parts[0].coordSys)

    def _margins(self, optic, rays):
        """(surfaces with an obscuration, rays) margins on the traced rays."""
        full = optic.traceFull(rays.copy())
        out = []
        for name, rec in full.items():
            item = optic[name]
            if getattr(item, "obscuration", None) is None:
                continue
            r = rec["out"]
            m = obscuration_margin(item.obscuration, r.x, r.y)
            m = np.where(r.failed, np.nan, m)
            out.append(m)
        if not out:
            return np.full((1, len(rays)), np.inf)
        return np.array(out)

    def predict(self, dofs, group):
        """Host evaluation of the kept margins (G groups' constraints) for
        states (S, ndof) in group ids (S,): (S, K) margins, inf padding."""
        z = np.asarray(dofs, dtype=float) / self.dof_scale
        return self.m0[group] + np.einsum('sd,sdk->sk', z, self.jac[group])

    # -- device side ----------------------------------------------------------------------
    def hits(self, dofs, group):
        """(S, K) bool: which kept margins of each sample's group trigger the
        rule (sign change or within the band of the edge)."""
        m = self.predict(dofs, group)
        m0 = self.m0[group]
        used = np.isfinite(m0)
        side = np.where(m0 >= 0, m, -m)
        with np.errstate(invalid="ignore"):
            return used & (side < self.band_abs + self.band_rel * np.abs(np.where(used, m - m0, 0.0)))

    def flags_host(self, dofs, group):
        """The device rule evaluated on the host in FP64 (for checks)."""
        z = np.asarray(dofs, dtype=float) / self.dof_scale
        out_box = np.any(np.abs(z) > self.reach, axis=1)
        return np.any(self.hits(dofs, group), axis=1) | out_box

    def prune(self, dofs, group, bad, min_bad_frac=0.1, min_hits=8):
        """Drops the kept margins whose triggers, over validation samples
        (dofs (S, ndof), group (S,), bad (S,) bool: surrogate error above
        the threshold), coincide with an error in fewer than min_bad_frac of
        at least min_hits samples.  Returns the number dropped."""
        h = self.hits(dofs, group)
        bad = np.asarray(bad, dtype=bool)
        dropped = 0
        for g in range(self.G):
            sel = group == g
            if not np.any(sel):
                continue
            hg, bg = h[sel], bad[sel]
            for k in range(int(self.nkept[g])):
                n = int(hg[:, k].sum())
                if n >= min_hits and np.mean(bg[hg[:, k]]) < min_bad_frac and np.isfinite(self.m0[g, k]):
                    self.m0[g, k] = np.inf
                    self.jac[g, :, k] = 0.0
                    dropped += 1
        self.dropped = getattr(self, "dropped", 0) + dropped
        self._dev = None
        return dropped

    def _device(self):
        import torch
        if self._dev is None:
            m0 = np.where(np.isfinite(self.m0), self.m0, np.float32(3e38)).astype(np.float32)
            f32 = (lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32).ravel()).to(D.device()))
            self._dev = (f32(m0), f32(self.jac), f32(self.reach))
        return self._dev

    def flags_device(self, feat_d, grp_d, out=None):
        """int32 device flags (n,): 1 where a kept margin of the sample's group,
        predicted at its normalised dofs (the first ndof feature columns),
        changed sign or lies within band_abs + band_rel * |J z| of zero, or
        where a normalised dof exceeds its reach."""
        import torch
        n = feat_d.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.int32, device=D.device())
        m0, jac, reach = self._device()
        _lib.check(_lib.lib().bt_surrogate_guard(feat_d.data_ptr(), feat_d.shape[1], self.pt.ndof, grp_d.data_ptr(),
                                                 m0.data_ptr(), jac.data_ptr(), reach.data_ptr(), self.K,
                                                 self.band_abs, self.band_rel, out.data_ptr(), n, D.stream_ptr()))
        return out
