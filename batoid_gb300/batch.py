"""Batched wavefronts and Zernike fits of perturbed telescope states.

A ``PerturbedTelescope`` describes a family of optics around a nominal one:
rigid-body motions (shift dx, dy, dz and tilts rx, ry) of named items and a
bending of one mirror as a weighted sum of seeded bicubic modes.  A state is
one vector of those degrees of freedom.

``zernike`` computes, for every (state, field), what ``batoid.zernike``
(batoid/analysis.py:479-573, reference='chief') computes for the state's
optic, in one persistent kernel launch (bt_batch_zernike).  ``perturbed``
builds the state's optic through the reference API
(withGloballyShiftedOptic / withLocallyRotatedOptic / withSurface,
batoid/optic.py:1380-1560), which is what the single-state path and any FP64
reference trace use.

A rigid-body motion leaves the relative transforms between members of the
moved group unchanged, so only the stages that enter or leave a moved
group, and the last stage's frame, vary per state; the kernel takes the
nominal transforms for the rest.
"""
import numpy as np
import torch

from . import _device as D
from . import _lib
from . import zpoly
from ._handle import Handle
from .coordSys import RotX, RotY
from .coordTransform import CoordTransform
from .utils import fieldToDirCos

RIGID_DOFS = ("dx", "dy", "dz", "rx", "ry")


def rigid_rotation(rx, ry):
    """Tilt of a rigid body: rotation about its own x axis, then y."""
    return RotX(rx) @ RotY(ry)


def _rot_stack(rx, ry):
    """RotX(rx) @ RotY(ry) for arrays of angles, shape (S, 3, 3)."""
    S = len(rx)
    cx, sx, cy, sy = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry)
    A = np.zeros((S, 3, 3))
    A[:, 0, 0] = 1
    A[:, 1, 1] = cx
    A[:, 1, 2] = -sx
    A[:, 2, 1] = sx
    A[:, 2, 2] = cx
    B = np.zeros((S, 3, 3))
    B[:, 0, 0] = cy
    B[:, 0, 2] = sy
    B[:, 1, 1] = 1
    B[:, 2, 0] = -sy
    B[:, 2, 2] = cy
    return A @ B


def _interfaces(item):
    if hasattr(item, "items"):
        out = []
        for it in item.items:
            out.extend(_interfaces(it))
        return out
    return [item]


class PerturbedTelescope:
    """Nominal optic plus perturbation degrees of freedom.

    Parameters
    ----------
    optic : CompoundOptic
        The nominal telescope; its stop surface must be flat and its
        entrance medium of constant index.
    rigid : sequence of str
        Items moved as rigid bodies, 5 dofs each (dx, dy, dz in m; rx, ry in
        rad: ``withGloballyShiftedOptic`` then ``withLocallyRotatedOptic``
        with RotX(rx) @ RotY(ry)).
    bend : str or None
        Item whose surface gets the bending term.
    modes : ModeSet or None
        Bending modes; their amplitudes (m) follow the rigid dofs.
    fields : array (F, 2)
        Field angles (rad).
    jmax, eps, sphereRadius, projection
        As for ``zernike``; eps defaults to the optic's pupilObscuration and
        sphereRadius to the optic's.
    """

    def __init__(self, optic, rigid=("M2", "Camera"), bend="M1", modes=None, fields=((0.0, 0.0),), jmax=28,
                 eps=None, sphereRadius=None, projection='postel'):
        self.optic = optic
        self.rigid = tuple(rigid)
        self.bend = bend if modes is not None else None
        self.modes = modes
        self.nmodes = modes.nmodes if modes is not None else 0
        self.ndof = 5 * len(self.rigid) + self.nmodes
        self.fields = np.atleast_2d(np.asarray(fields, dtype=float))
        self.jmax = int(jmax)
        self.eps = optic.pupilObscuration if eps is None else float(eps)
        self.sphereRadius = optic.sphereRadius if sphereRadius is None else float(sphereRadius)
        self.projection = projection
        self._plan = None
        self._prepared = set()
        self._analyse()

    # -- single-state optic (reference API) -----------------------------------
    def perturbed(self, dofs):
        """The state's optic, built with the reference's optic API."""
        from .surface import Sum
        dofs = np.asarray(dofs, dtype=float)
        if dofs.shape != (self.ndof,):
            raise ValueError(f"expected {self.ndof} dofs")
        o = self.optic
        for g, name in enumerate(self.rigid):
            dx, dy, dz, rx, ry = dofs[5 * g:5 * g + 5]
            o = o.withGloballyShiftedOptic(name, [dx, dy, dz])
            o = o.withLocallyRotatedOptic(name, rigid_rotation(rx, ry))
        if self.modes is not None:
            base = o[self.bend].surface
            term = self.modes.bicubic(dofs[5 * len(self.rigid):])
            parts = tuple(base.surfaces) if isinstance(base, Sum) else (base,)
            o = o.withSurface(self.bend, Sum(parts + (term,)))
        return o

    # -- static analysis of the stage list --------------------------------------
    def _analyse(self):
        optic = self.optic
        stop = optic.stopSurface
        from .surface import Plane
        if not isinstance(stop.surface, Plane):
            raise NotImplementedError("batched wavefronts need a flat stop surface")
        if optic.inMedium.getN(500e-9) != optic.inMedium.getN(1000e-9):
            raise NotImplementedError("batched wavefronts need a constant-index entrance medium")
        self.prog = optic._program(optic.coordSys)
        stages = [info[0] for info in self.prog.stage_info]
        self.ifaces = stages
        group = [-1] * len(stages)
        self.group_kind = []
        self.group_frame = []
        for g, name in enumerate(self.rigid):
            item = optic[name]
            members = {id(i) for i in _interfaces(item)}
            for k, it in enumerate(stages):
                if id(it) in members:
                    group[k] = g
            self.group_kind.append("compound" if hasattr(item, "items") else "interface")
            self.group_frame.append((np.array(item.coordSys.origin), np.array(item.coordSys.rot)))
        self.group = group
        self.var_stages = [k for k in range(len(stages))
                           if group[k] != (group[k - 1] if k > 0 else -1)]
        if len(self.var_stages) > 8:
            raise NotImplementedError("at most 8 stages may change per state")
        self.bend_stage = -1
        if self.bend is not None:
            bend_item = optic[self.bend]
            for k, it in enumerate(stages):
                if it is bend_item:
                    self.bend_stage = k
            if self.bend_stage < 0:
                raise ValueError(f"{self.bend} is not traced")
        ct = CoordTransform(stop.coordSys, optic.coordSys)
        self.stop_dr = np.array(ct.dr, dtype=float)
        self.stop_drot = np.array(ct.drot, dtype=float).ravel()
        self.field_table = np.stack([self._field_row(tx, ty) for tx, ty in self.fields])

    def _field_row(self, tx, ty):
        """Back-propagation frame of asGrid's _finish for one field
        (batoid/rayVector.py:817-846), plus the rays' velocity."""
        dirCos = fieldToDirCos(tx, ty, projection=self.projection)
        n = self.optic.inMedium.getN(500e-9)
        vv = np.array(dirCos, dtype=float, copy=True)
        vv /= n * np.sqrt(np.dot(vv, vv))
        zhat = -n * vv
        xhat = np.cross(np.array([1.0, 0.0, 0.0]), zhat)
        xhat /= np.sqrt(np.dot(xhat, xhat))
        yhat = np.cross(xhat, zhat)
        origin = zhat * self.optic.backDist
        rot = np.stack([xhat, yhat, zhat]).T
        r = rot.ravel()
        vl = [-vv[0] * r[0] - vv[1] * r[3] - vv[2] * r[6],
              -vv[0] * r[1] - vv[1] * r[4] - vv[2] * r[7],
              -vv[0] * r[2] - vv[1] * r[5] - vv[2] * r[8]]
        return np.concatenate([origin, r, vl, vv])

    # -- per-state tables (vectorised) ---------------------------------------------
    def state_tables(self, dofs):
        """(xf (S, nvar, 12), det (S, 12), amps (S, nmodes)) for dofs (S, ndof)."""
        dofs = np.atleast_2d(np.asarray(dofs, dtype=float))
        S = dofs.shape[0]
        if dofs.shape[1] != self.ndof:
            raise ValueError(f"expected {self.ndof} dofs per state")
        K = len(self.ifaces)
        O = np.empty((S, K, 3))
        R = np.empty((S, K, 3, 3))
        for k, it in enumerate(self.ifaces):
            O[:, k] = it.coordSys.origin
            R[:, k] = it.coordSys.rot
        for g in range(len(self.rigid)):
            d = dofs[:, 5 * g:5 * g + 3]
            rot = _rot_stack(dofs[:, 5 * g + 3], dofs[:, 5 * g + 4])
            ks = [k for k in range(K) if self.group[k] == g]
            if self.group_kind[g] == "interface":
                for k in ks:
                    O[:, k] = O[:, k] + d
                    R[:, k] = R[:, k] @ rot
            else:
                c, Rc = self.group_frame[g]
                center = c + d
                G = (Rc @ rot) @ Rc.T
                for k in ks:
                    O[:, k] = np.einsum('sij,sj->si', G, (O[:, k] + d) - center) + center
                    R[:, k] = G @ R[:, k]
        xf = np.empty((S, len(self.var_stages), 12))
        in_o = np.asarray(self.optic.coordSys.origin, dtype=float)
        in_r = np.asarray(self.optic.coordSys.rot, dtype=float)
        for v, k in enumerate(self.var_stages):
            if k == 0:
                o1 = np.broadcast_to(in_o, (S, 3))
                r1 = np.broadcast_to(in_r, (S, 3, 3))
            else:
                o1, r1 = O[:, k - 1], R[:, k - 1]
            r1t = np.swapaxes(r1, 1, 2)
            xf[:, v, :3] = np.einsum('sij,sj->si', r1t, O[:, k] - o1)
            xf[:, v, 3:] = (r1t @ R[:, k]).reshape(S, 9)
        det = np.concatenate([O[:, -1], R[:, -1].reshape(S, 9)], axis=1)
        amps = np.ascontiguousarray(dofs[:, 5 * len(self.rigid):])
        return np.ascontiguousarray(xf), np.ascontiguousarray(det), amps

    # -- device plan -------------------------------------------------------------------
    def plan(self):
        if self._plan is None:
            from .surface import Sphere
            a = self.prog.arrays
            desc = _lib.BtBatchDesc()
            desc.nstages = self.prog.nstages
            desc.kinds = ctypes_addr(a["kinds"])
            desc.surfaces = ctypes_addr(a["surfs"])
            desc.dr = a["dr"].ctypes.data
            desc.drot = a["drot"].ctypes.data
            desc.media = ctypes_addr(a["media"])
            desc.obscurations = ctypes_addr(a["obscs"])
            self._var = (_lib.c_int * max(len(self.var_stages), 1))(*self.var_stages)
            desc.nvar = len(self.var_stages)
            desc.var_stages = ctypes_addr(self._var)
            desc.modal_stage = self.bend_stage
            if self.modes is not None:
                m = self.modes
                desc.modal_grid[:] = [m.x0, m.y0, m.dx, m.dy]
                desc.modal_nx = m.n
                desc.modal_ny = m.n
                desc.nmodes = m.nmodes
                desc.modes = m.device_tables().data_ptr()
                desc.modal_use_nan = 0
            desc.stop_dr[:] = list(self.stop_dr)
            desc.stop_drot[:] = list(self.stop_drot)
            self._sphere = Sphere(-self.sphereRadius)
            desc.sphere = self._sphere._surface.ptr
            desc.sphere_radius = self.sphereRadius
            R_outer = self.optic.pupilSize / 2
            desc.pupil_size = self.optic.pupilSize
            desc.r_outer = R_outer
            desc.r_inner = R_outer * self.eps
            self._basis = np.ascontiguousarray(zpoly.basis_xy(self.jmax, R_outer, R_outer * self.eps))
            desc.jmax = self.jmax
            desc.basis = self._basis.ctypes.data
            desc.side = self._basis.shape[1]
            self._desc = desc
            self._plan = Handle(_lib.new_handle(_lib.lib().bt_batch_create, desc), "bt_batch_destroy")
            self._d_fields = D.to_device(self.field_table.ravel())
        return self._plan

    def prepare(self, nx_values):
        """Builds the fit tables of these pupil grid sizes."""
        want = sorted({int(n) for n in np.ravel(nx_values)} - self._prepared)
        if want:
            arr = (_lib.c_int * len(want))(*want)
            _lib.check(_lib.lib().bt_batch_prepare(self.plan().ptr, len(want), arr, D.stream_ptr()))
            self._prepared.update(want)

    def device_inputs(self, dofs, nx, wavelength):
        """Device tensors of one batch: tables, grid sizes, wavelengths and
        the job order (largest grids first)."""
        dofs = np.atleast_2d(np.asarray(dofs, dtype=float))
        S = dofs.shape[0]
        nx = np.array(np.broadcast_to(np.asarray(nx, dtype=np.int32), (S,)))
        wl = np.array(np.broadcast_to(np.asarray(wavelength, dtype=float), (S,)))
        xf, det, amps = self.state_tables(dofs)
        F = len(self.fields)
        jobs = np.arange(S * F, dtype=np.int32)
        order = jobs[np.argsort(-nx[jobs // F], kind='stable')].astype(np.int32)
        t = dict(xf=D.to_device(xf.ravel()), det=D.to_device(det.ravel()),
                 amps=D.to_device(amps.ravel() if amps.size else np.zeros(1)),
                 nx=torch.from_numpy(np.ascontiguousarray(nx)).to(D.device()),
                 wl=D.to_device(np.ascontiguousarray(wl)),
                 order=torch.from_numpy(order).to(D.device()), nstates=S)
        return t

    def launch(self, inp, coefs, status, threads=256, ctas_per_sm=2, niter=None, graph=False, order=None):
        """Stream-ordered launch on device inputs from ``device_inputs``;
        ``order`` (device int32 job ids) runs only those jobs."""
        from .global_vars import _batoid_niter
        plan = self.plan()
        fn = _lib.lib().bt_batch_zernike_graph if graph else _lib.lib().bt_batch_zernike
        order = inp["order"] if order is None else order
        _lib.check(fn(plan.ptr, inp["nstates"], D.ptr(inp["xf"]), D.ptr(inp["det"]), D.ptr(inp["amps"]),
                      inp["nx"].data_ptr(), D.ptr(inp["wl"]), len(self.fields), D.ptr(self._d_fields),
                      order.data_ptr(), int(order.numel()), coefs.data_ptr(), status.data_ptr(), int(threads),
                      int(ctas_per_sm), int(_batoid_niter if niter is None else niter), D.stream_ptr()))

    def zernike(self, dofs, nx, wavelength, threads=None, ctas_per_sm=None, errors='raise'):
        """Zernike coefficients (waves; Noll; entry 0 = 0) of every state and
        field: array (S, F, jmax + 1).  ``errors='nan'`` leaves failed fits
        as NaN rows instead of raising."""
        dofs = np.atleast_2d(np.asarray(dofs, dtype=float))
        S, F, J = dofs.shape[0], len(self.fields), self.jmax
        self.prepare(nx)
        if threads is None or ctas_per_sm is None:
            from .autotune import batch_config
            threads, ctas_per_sm = batch_config(self)
        inp = self.device_inputs(dofs, nx, wavelength)
        coefs = torch.empty(S * F * (J + 1), dtype=torch.float64, device=D.device())
        status = torch.empty(S * F, dtype=torch.int32, device=D.device())
        self.launch(inp, coefs, status, threads, ctas_per_sm)
        out = D.to_host(coefs).reshape(S, F, J + 1)
        st = D.to_host(status).reshape(S, F)
        if errors == 'raise' and np.any(st != 0):
            bad = np.argwhere(st != 0)
            s, f = bad[0]
            code = int(st[s, f])
            if code == _lib.BT_ERR_RANK:
                raise RuntimeError(f"Rank-deficient matrix found when fitting {J} Zernike coefficients "
                                   f"(state {s}, field {f}; {len(bad)} fits)")
            raise RuntimeError(f"batched fit failed with status {code} (state {s}, field {f}; {len(bad)} fits)")
        return out


def ctypes_addr(obj):
    import ctypes
    return ctypes.addressof(obj)
