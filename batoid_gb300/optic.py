"""Optic tree (batoid/optic.py) with a fused trace.

The tree API is the reference's: Interface / Mirror / RefractiveInterface /
Detector / Baffle leaves and CompoundOptic / Lens containers, name lookup,
and the perturbation builders.  Tracing differs in mechanism only: instead
of one Python call and one kernel pass per surface (batoid/optic.py:
1013-1083), the sequence of interfaces visited by a trace is compiled once
into a device program (``_Program``) and all rays go through all surfaces in
one kernel launch.  Per-ray results follow the reference's semantics.
"""
from collections import OrderedDict
from functools import cached_property

import numpy as np

from . import _device as D
from . import _lib
from .coating import SimpleCoating
from .constants import globalCoordSys, vacuum
from .coordTransform import CoordTransform
from .obscuration import ObscAnnulus, ObscCircle, ObscNegation
from .rayVector import RayVector

_CACHE_KEYS = ('itemDict', '_names', 'R_inner', 'R_outer', '_programs')


class Optic:
    """Base class of all optics (batoid/optic.py:13-95)."""

    def __init__(self, name=None, coordSys=globalCoordSys, inMedium=vacuum, outMedium=vacuum,
                 skip=False, **kwargs):
        self.name = name
        self.coordSys = coordSys
        self.inMedium = inMedium
        self.outMedium = outMedium
        self.skip = False
        for k in _CACHE_KEYS:
            kwargs.pop(k, None)
        self.__dict__.update(**kwargs)

    def _repr_helper(self):
        out = ""
        if self.name is not None:
            out += ", name={!r}".format(self.name)
        out += ", coordSys={!r}".format(self.coordSys)
        if self.inMedium != vacuum:
            out += ", inMedium={!r}".format(self.inMedium)
        if self.outMedium != vacuum:
            out += ", outMedium={!r}".format(self.outMedium)
        return out

    @classmethod
    def fromYaml(cls, filename):
        """Load an optic from a YAML file (own YAML-subset reader; see parse.py)."""
        from .parse import load_yaml_file, parse_optic
        config = load_yaml_file(filename)
        return parse_optic(config['opticalSystem'])

    # -- fused tracing ------------------------------------------------------------
    def _stages(self, reverse=False, path=None):
        """List of (interface, stage_kind, outgoing_medium) visited by a trace."""
        raise NotImplementedError

    def _program(self, coordSys, reverse=False, path=None):
        progs = self.__dict__.setdefault('_programs', {})
        key = (coordSys, reverse, None if path is None else tuple(path))
        prog = progs.get(key)
        if prog is None:
            prog = _Program(self._stages(reverse, path), coordSys)
            progs[key] = prog
        return prog

    def _trace_fused(self, rv, reverse=False, path=None):
        prog = self._program(rv.coordSys, reverse, path)
        prog.trace(rv)
        return rv

    def _traceFull_fused(self, rv, reverse=False, path=None):
        prog = self._program(rv.coordSys, reverse, path)
        outs = prog.traceFull(rv)
        result = OrderedDict()
        rv_in = rv
        for (iface, _, _, key), out in zip(prog.stage_info, outs):
            result[key] = {'name': iface.name, 'in': rv_in, 'out': out}
            rv_in = out
        return result


def _interaction(iface, reverse):
    """Stage kind and outgoing medium of one interface."""
    if isinstance(iface, Mirror):
        return _lib.STAGE_REFLECT, None
    if isinstance(iface, RefractiveInterface):
        return _lib.STAGE_REFRACT, (iface.inMedium if reverse else iface.outMedium)
    if isinstance(iface, OPDScreen):
        return _lib.STAGE_SCREEN, None
    return _lib.STAGE_INTERSECT, None


class _Program:
    """A compiled trace: device program of all stages plus the Python
    objects that must outlive it (surfaces own device tables)."""

    def __init__(self, stages, coordSys):
        self.stage_info = []
        n = len(stages)
        kinds = (_lib.c_int * max(n, 1))()
        surfs = (_lib.c_void_p * max(n, 1))()
        media = (_lib.c_void_p * max(n, 1))()
        obscs = (_lib.c_void_p * max(n, 1))()
        coats = (_lib.c_void_p * max(n, 1))()
        screens = (_lib.c_void_p * max(n, 1))()
        dr = np.zeros((max(n, 1), 3))
        drot = np.zeros((max(n, 1), 9))
        self._keep = []
        prev = coordSys
        keys = {}
        for k, (iface, kind, medium, forced_key) in enumerate(stages):
            ct = CoordTransform(prev, iface.coordSys)
            dr[k] = ct.dr
            drot[k] = ct.drot.ravel()
            kinds[k] = kind
            surfs[k] = iface.surface._surface.ptr
            media[k] = medium._medium.ptr if medium is not None else None
            obscs[k] = iface.obscuration._obsc.ptr if iface.obscuration is not None else None
            coats[k] = None
            screens[k] = iface.screen._surface.ptr if kind == _lib.STAGE_SCREEN else None
            self._keep.append((iface.surface, medium, iface.obscuration, getattr(iface, 'screen', None)))
            prev = iface.coordSys
            if forced_key is None:
                key = iface.name
            else:
                base = iface.name
                j = keys.get(base, 0)
                key = f"{base}_{j}"
                keys[base] = j + 1
            self.stage_info.append((iface, kind, iface.coordSys, key))
        self.final_coordSys = prev
        self.nstages = n
        dr = np.ascontiguousarray(dr)
        drot = np.ascontiguousarray(drot)
        # the stage arrays, also used to build batched plans of this optic
        self.arrays = dict(kinds=kinds, surfs=surfs, dr=dr, drot=drot, media=media, obscs=obscs, screens=screens)
        self._coats = coats
        self._handle = None

    @property
    def _optic(self):
        # the device program is built on first use
        if self._handle is None:
            a = self.arrays
            self._handle = _make_optic(self.nstages, a["kinds"], a["surfs"], a["dr"], a["drot"], a["media"],
                                       a["obscs"], self._coats, a["screens"])
        return self._handle

    def trace(self, rv):
        from .global_vars import _batoid_niter
        if self.nstages:
            r = rv._rv
            _lib.check(_lib.lib().bt_optic_trace(self._optic.ptr, r, _batoid_niter, D.stream_ptr()))
            rv.coordSys = self.final_coordSys
        return rv

    def traceFull(self, rv):
        from .global_vars import _batoid_niter
        n = len(rv)
        outs = []
        arr = (_lib.BtRayVector * max(self.nstages, 1))()
        for k, (_, _, cs, _) in enumerate(self.stage_info):
            out = RayVector._empty(n, cs)
            outs.append(out)
            arr[k] = out._rv
        if self.nstages and n:
            r = rv._rv
            _lib.check(_lib.lib().bt_optic_trace_full(self._optic.ptr, r, arr, _batoid_niter,
                                                      D.stream_ptr()))
        return outs

    def trace_host(self, host_rv, chunk=0):
        """End-to-end trace of host (ideally pinned) arrays; see bt_optic_trace_host."""
        from .global_vars import _batoid_niter
        _lib.check(_lib.lib().bt_optic_trace_host(self._optic.ptr, host_rv, _batoid_niter, chunk,
                                                  D.stream_ptr()))


def _make_optic(n, kinds, surfs, dr, drot, media, obscs, coats, screens=None):
    from ._handle import Handle
    h = _lib.new_handle(_lib.lib().bt_optic_create_ex, n, kinds, surfs,
                        dr.ctypes.data_as(_lib.c_double_p), drot.ctypes.data_as(_lib.c_double_p),
                        media, obscs, coats, screens)
    return Handle(h, "bt_optic_destroy")


class Interface(Optic):
    """One surface with an optional obscuration (batoid/optic.py:98-760)."""

    def __init__(self, surface, obscuration=None, **kwargs):
        Optic.__init__(self, **kwargs)
        self.path = [self.name]
        self.surface = surface
        self.obscuration = obscuration
        self.inRadius = self.R_inner
        self.outRadius = None
        if self.obscuration is not None:
            if isinstance(self.obscuration, ObscNegation):
                if isinstance(self.obscuration.original, ObscCircle):
                    self.outRadius = self.obscuration.original.radius
                elif isinstance(self.obscuration.original, ObscAnnulus):
                    self.outRadius = self.obscuration.original.outer
                    self.inRadius = self.obscuration.original.inner
            elif isinstance(self.obscuration, ObscCircle):
                self.outRadius = self.obscuration.radius
            elif isinstance(self.obscuration, ObscAnnulus):
                self.outRadius = self.obscuration.outer
                self.inRadius = self.obscuration.inner
        if self.inRadius is None:
            self.inRadius = self.R_inner
        if self.outRadius is None:
            self.outRadius = self.R_outer

    def __hash__(self):
        return hash((self.__class__.__name__, self.surface, self.obscuration, self.name,
                     self.inMedium, self.outMedium, self.coordSys))

    def _stages(self, reverse=False, path=None):
        kind, medium = _interaction(self, reverse)
        return [(self, kind, medium, None)]

    def trace(self, rv, reverse=False):
        """interact + obscure, in place (batoid/optic.py:391-424)."""
        return self._trace_fused(rv, reverse)

    def traceFull(self, rv, reverse=False):
        result = OrderedDict()
        if not self.skip:
            result[self.name] = {'name': self.name, 'in': rv, 'out': self.trace(rv.copy(), reverse=reverse)}
        return result

    def traceSplit(self, rv, minFlux=1e-3, reverse=False, _verbose=False):
        """(forward, reverse) lists of rays after splitting at this surface
        (batoid/optic.py:466-536): obscuration applied to both, ``path``
        extended by this interface's name."""
        if _verbose:
            s = "forward" if not reverse else "reverse"
            print("traceSplit {}       {:30s} flux = {:18.8f}   nphot = {:10d}".format(
                s, self.name, float(np.sum(rv.flux)), len(rv)))
        if self.skip:
            return ([], [rv]) if reverse else ([rv], [])
        refracted, reflected = self.rSplit(rv, reverse=reverse)
        if self.obscuration is not None:
            if refracted is not None:
                self.obscuration.obscure(refracted)
            if reflected is not None:
                self.obscuration.obscure(reflected)
        path = list(getattr(rv, 'path', []))
        for r in (refracted, reflected):
            if r is not None:
                r.path = path + [self.name]
        rForward, rReverse = [refracted], [reflected]
        if reverse:
            rForward, rReverse = rReverse, rForward
        if isinstance(self, Mirror):
            rForward, rReverse = rReverse, rForward
        return rForward, rReverse

    def clearObscuration(self, unless=()):
        if self.name not in unless:
            self.obscuration = None
            self.__dict__.pop('_programs', None)

    def interact(self, rv, reverse=False):
        return self.surface.intersect(rv, coordSys=self.coordSys)

    def intersect(self, rv, reverse=False):
        return self.surface.intersect(rv, coordSys=self.coordSys)

    def __eq__(self, other):
        if not self.__class__ == other.__class__:
            return False
        return (self.surface == other.surface and self.obscuration == other.obscuration
                and self.name == other.name and self.inMedium == other.inMedium
                and self.outMedium == other.outMedium and self.coordSys == other.coordSys)

    def __ne__(self, other):
        return not (self == other)

    def __repr__(self):
        out = "{!s}({!r}".format(self.__class__.__name__, self.surface)
        if self.obscuration is not None:
            out += ", obscuration={!r}".format(self.obscuration)
        out += Optic._repr_helper(self)
        return out + ")"

    def _clone(self, surface, **changes):
        ret = self.__class__.__new__(self.__class__)
        newDict = {k: v for k, v in self.__dict__.items() if k not in _CACHE_KEYS}
        newDict.update(changes)
        del newDict['surface']
        ret.__init__(surface, **newDict)
        return ret

    def withGlobalShift(self, shift):
        changes = {'coordSys': self.coordSys.shiftGlobal(shift)}
        if 'stopSurface' in self.__dict__:
            changes['stopSurface'] = self.__dict__['stopSurface'].withGlobalShift(shift)
        return self._clone(self.surface, **changes)

    def withLocalShift(self, shift):
        return self.withGlobalShift(self.coordSys.rot @ shift)

    def withGlobalRotation(self, rot, rotCenter=None, coordSys=None):
        if rotCenter is None:
            rotCenter = [0, 0, 0]
        if coordSys is None:
            coordSys = globalCoordSys
        elif coordSys == 'local':
            coordSys = self.coordSys
        changes = {'coordSys': self.coordSys.rotateGlobal(rot, rotCenter, coordSys)}
        if 'stopSurface' in self.__dict__:
            changes['stopSurface'] = self.__dict__['stopSurface'].withGlobalRotation(rot, rotCenter, coordSys)
        return self._clone(self.surface, **changes)

    def withLocalRotation(self, rot, rotCenter=None, coordSys=None):
        if rotCenter is None:
            rotCenter = [0, 0, 0]
        if coordSys is None:
            coordSys = self.coordSys
        changes = {'coordSys': self.coordSys.rotateLocal(rot, rotCenter, coordSys)}
        if 'stopSurface' in self.__dict__:
            changes['stopSurface'] = self.__dict__['stopSurface'].withLocalRotation(rot, rotCenter, coordSys)
        return self._clone(self.surface, **changes)

    def withSurface(self, surface):
        return self._clone(surface)

    def withPerturbedSurface(self, perturbation):
        return self.withSurface(self.surface + perturbation)

    @cached_property
    def R_outer(self):
        obsc = self.obscuration
        if obsc is not None:
            if isinstance(obsc, ObscNegation):
                obsc = obsc.original
            if isinstance(obsc, ObscAnnulus):
                return obsc.outer
            if isinstance(obsc, ObscCircle):
                return obsc.radius
        return None

    @cached_property
    def R_inner(self):
        obsc = self.obscuration
        if obsc is not None:
            if isinstance(obsc, ObscNegation):
                obsc = obsc.original
            if isinstance(obsc, ObscAnnulus):
                return obsc.inner
            if isinstance(obsc, ObscCircle):
                return 0.0
        return None


class RefractiveInterface(Interface):
    def __init__(self, *args, **kwargs):
        Interface.__init__(self, *args, **kwargs)
        self.forwardCoating = SimpleCoating(reflectivity=0.0, transmissivity=1.0)
        self.reverseCoating = SimpleCoating(reflectivity=0.0, transmissivity=1.0)

    def interact(self, rv, reverse=False):
        m1, m2 = (self.outMedium, self.inMedium) if reverse else (self.inMedium, self.outMedium)
        return self.surface.refract(rv, m1, m2, coordSys=self.coordSys)

    def refract(self, rv, reverse=False):
        return self.interact(rv, reverse=reverse)

    def rSplit(self, rv, reverse=False):
        """(refracted, reflected); as the reference, the forward pass uses
        reverseCoating and the reverse pass forwardCoating
        (batoid/optic.py:786-797)."""
        if reverse:
            m1, m2, coating = self.outMedium, self.inMedium, self.forwardCoating
        else:
            m1, m2, coating = self.inMedium, self.outMedium, self.reverseCoating
        return self.surface.rSplit(rv, m1, m2, coating, coordSys=self.coordSys)


class Mirror(Interface):
    def __init__(self, *args, **kwargs):
        Interface.__init__(self, *args, **kwargs)
        self.forwardCoating = SimpleCoating(reflectivity=1.0, transmissivity=0.0)
        self.reverseCoating = SimpleCoating(reflectivity=1.0, transmissivity=0.0)

    def interact(self, rv, reverse=False):
        return self.surface.reflect(rv, coordSys=self.coordSys)

    def reflect(self, rv, reverse=False):
        return self.interact(rv, reverse=reverse)

    def rSplit(self, rv, reverse=False):
        # reflection only (batoid/optic.py:821-823)
        return None, self.surface.reflect(rv, coordSys=self.coordSys)


class Detector(Interface):
    def __init__(self, *args, **kwargs):
        Interface.__init__(self, *args, **kwargs)
        self.forwardCoating = SimpleCoating(reflectivity=0.0, transmissivity=1.0)
        self.reverseCoating = None

    def rSplit(self, rv, reverse=False):
        # batoid/optic.py:840-845
        assert reverse is False
        return self.surface.rSplit(rv, self.inMedium, self.outMedium, self.forwardCoating, coordSys=self.coordSys)


class Baffle(Interface):
    def __init__(self, *args, **kwargs):
        Interface.__init__(self, *args, **kwargs)
        self.forwardCoating = SimpleCoating(reflectivity=0.0, transmissivity=1.0)
        self.reverseCoating = SimpleCoating(reflectivity=0.0, transmissivity=1.0)

    def rSplit(self, rv, reverse=False):
        # straight through (batoid/optic.py:864-865)
        return self.surface.intersect(rv, self.coordSys), None


class OPDScreen(Interface):
    """Interface adding an optical path difference (the screen surface's
    sag, meters) and the matching deflection (batoid/optic.py:867-929)."""

    def __init__(self, surface, screen, **kwargs):
        Interface.__init__(self, surface, **kwargs)
        self.screen = screen
        assert self.inMedium == self.outMedium

    def interact(self, rv, reverse=False):
        return self.surface.refractScreen(rv, self.screen, coordSys=self.coordSys)

    def refract(self, rv, reverse=False):
        return self.interact(rv, reverse=reverse)


class CompoundOptic(Optic):
    """Sequence of optics traced in order (batoid/optic.py:933-1820)."""

    def __init__(self, items, **kwargs):
        Optic.__init__(self, **kwargs)
        self.items = tuple(items)
        self.path = [name for item in self.items for name in item.path]

    @cached_property
    def itemDict(self):
        out = {self.name: self}
        for item in self.items:
            out[self.name + '.' + item.name] = item
            if hasattr(item, 'itemDict'):
                for k, v in item.itemDict.items():
                    out[self.name + '.' + k] = v
        return out

    def __getitem__(self, key):
        try:
            return self.itemDict[key]
        except KeyError:
            try:
                return self.itemDict[self._names[key]]
            except KeyError:
                raise ValueError("Cannot find item {}".format(key))

    @cached_property
    def _names(self):
        nameDict = {}
        duplicates = set()
        for k in self.itemDict.keys():
            tokens = k.split('.')
            shortNames = [tokens[-1]]
            for token in reversed(tokens[:-1]):
                shortNames.append('.'.join([token, shortNames[-1]]))
            for shortName in shortNames:
                if shortName in nameDict:
                    duplicates.add(shortName)
                else:
                    nameDict[shortName] = k
        for name in duplicates:
            del nameDict[name]
        return nameDict

    def _interfaces(self, reverse=False):
        """Flattened non-skipped interfaces in trace order."""
        out = []
        for item in (self.items if not reverse else reversed(self.items)):
            if item.skip:
                continue
            if isinstance(item, CompoundOptic):
                out.extend(item._interfaces(reverse))
            else:
                out.append(item)
        return out

    def _stages(self, reverse=False, path=None):
        if path is None:
            return [(it,) + _interaction(it, reverse) + (None,) for it in self._interfaces(reverse)]
        # Ghost / explicit path (batoid/optic.py:1050-1082): a direction
        # change at an interface is a reflection off its surface.
        nominal = {}
        for name in path:
            if name not in nominal:
                nominal[name] = len(nominal)
        direction = "forward"
        stages = []
        for i in range(len(path)):
            item = self[path[i]]
            if i == len(path) - 1:
                nxt = "reverse" if nominal[path[i]] == 0 else direction
            else:
                nxt = "reverse" if nominal[path[i + 1]] < nominal[path[i]] else "forward"
            if direction == nxt:
                kind, medium = _interaction(item, direction == "reverse")
                stages.append((item, kind, medium, True))
            else:
                direction = nxt
                stages.append((item, _lib.STAGE_REFLECT, None, True))
        return stages

    def trace(self, rv, reverse=False, path=None):
        """Trace rays through all items in one kernel launch, in place."""
        return self._trace_fused(rv, reverse, path)

    def traceFull(self, rv, reverse=False, path=None):
        """Per-interface history {name: {'name', 'in', 'out'}} (batoid/optic.py:1085-1182)."""
        if self.skip and path is None:
            return OrderedDict()
        return self._traceFull_fused(rv, reverse, path)

    def traceSplit(self, rv, minFlux=1e-3, reverse=False, _verbose=False):
        """Recursive split trace with a work queue (batoid/optic.py:1184-1280):
        (forward, reverse) lists of RayVectors, one per distinct path, each
        with its ``path``; vignetted rays and rays below minFlux are dropped
        between items (stream compaction on the device)."""
        if _verbose:
            s = "reverse" if reverse else "forward"
            print("traceSplit {}       {:30s} flux = {:18.8f}   nphot = {:10d}".format(
                s, self.name, float(np.sum(rv.flux)), len(rv)))
        if self.skip:
            return ([], [rv]) if reverse else ([rv], [])
        workQueue = [(rv, "forward", 0)] if not reverse else [(rv, "reverse", len(self.items) - 1)]
        outF, outR = [], []
        while workQueue:
            rays, direction, idx = workQueue.pop()
            optic = self.items[idx]
            rF, rR = optic.traceSplit(rays, minFlux=minFlux, reverse=(direction == "reverse"), _verbose=_verbose)
            rF = [r for r in rF if r is not None]
            rR = [r for r in rR if r is not None]
            for lst in (rF, rR):
                for k, rr in enumerate(lst):
                    keep = (rr._b[0] == 0) & (rr._d[8] >= minFlux)
                    nr = RayVector._fromBuffers(rr._d[:, keep].contiguous(), rr._b[:, keep].contiguous(),
                                                rr.coordSys)
                    nr.path = rr.path
                    lst[k] = nr
            for rr in rF:
                if len(rr) > 0:
                    if idx == len(self.items) - 1:
                        outF.append(rr)
                    else:
                        workQueue.append((rr, "forward", idx + 1))
            for rr in rR:
                if len(rr) > 0:
                    if idx == 0:
                        outR.append(rr)
                    else:
                        workQueue.append((rr, "reverse", idx - 1))
        return outF, outR

    def clearObscuration(self, unless=()):
        for item in self.items:
            item.clearObscuration(unless=unless)
        self.__dict__.pop('_programs', None)

    def __eq__(self, other):
        if not self.__class__ == other.__class__:
            return False
        return (self.items == other.items and self.name == other.name
                and self.inMedium == other.inMedium and self.outMedium == other.outMedium
                and self.coordSys == other.coordSys)

    def __ne__(self, other):
        return not (self == other)

    def __repr__(self):
        out = "{!s}([".format(self.__class__.__name__)
        out += ", ".join("{!r}".format(item) for item in self.items)
        out += "]" + Optic._repr_helper(self) + ")"
        return out

    def __hash__(self):
        return hash((self.__class__.__name__, self.items, self.name, self.inMedium, self.outMedium,
                     self.coordSys))

    def _newDict(self):
        d = {k: v for k, v in self.__dict__.items() if k not in _CACHE_KEYS}
        d.pop('items', None)
        return d

    def withGlobalShift(self, shift):
        newItems = [item.withGlobalShift(shift) for item in self.items]
        newDict = self._newDict()
        newDict['coordSys'] = self.coordSys.shiftGlobal(shift)
        if 'stopSurface' in newDict:
            newDict['stopSurface'] = newDict['stopSurface'].withGlobalShift(shift)
        return self.__class__(newItems, **newDict)

    def withLocalShift(self, shift):
        return self.withGlobalShift(self.coordSys.rot @ shift)

    def _replace(self, name, fn_leaf, fn_recurse):
        """Rebuild with the item at ``name`` (relative) replaced."""
        newItems = []
        newDict = self._newDict()
        for i, item in enumerate(self.items):
            if name.startswith(item.name):
                if name == item.name:
                    newItems.append(fn_leaf(item))
                else:
                    newItems.append(fn_recurse(item, name))
                newItems.extend(self.items[i + 1:])
                return self.__class__(newItems, **newDict)
            newItems.append(item)
        raise RuntimeError("item not found while rebuilding")

    def _qualify(self, name):
        name = self._names.get(name, name)
        if name not in self.itemDict:
            raise ValueError("Optic {} not found".format(name))
        return name

    def _strip(self, name):
        leading = name[:len(self.name) + 1]
        assert leading == self.name + ".", f"{leading} != {self.name}."
        return name[len(self.name) + 1:]

    def withGloballyShiftedOptic(self, name, shift):
        name = self._qualify(name)
        if name == self.name:
            return self.withGlobalShift(shift)
        return self._replace(self._strip(name), lambda it: it.withGlobalShift(shift),
                             lambda it, nm: it.withGloballyShiftedOptic(nm, shift))

    def withLocallyShiftedOptic(self, name, shift):
        name = self._qualify(name)
        return self.withGloballyShiftedOptic(name, self.itemDict[name].coordSys.rot @ shift)

    def withGlobalRotation(self, rot, rotCenter=None, coordSys=None):
        if rotCenter is None:
            rotCenter = [0, 0, 0]
        if coordSys is None:
            coordSys = globalCoordSys
        elif coordSys == 'local':
            coordSys = self.coordSys
        newItems = [item.withGlobalRotation(rot, rotCenter, coordSys) for item in self.items]
        newDict = self._newDict()
        newDict['coordSys'] = self.coordSys.rotateGlobal(rot, rotCenter, coordSys)
        if 'stopSurface' in newDict:
            newDict['stopSurface'] = newDict['stopSurface'].withGlobalRotation(rot, rotCenter, coordSys)
        return self.__class__(newItems, **newDict)

    def withLocalRotation(self, rot, rotCenter=None, coordSys=None):
        if rotCenter is None:
            rotCenter = [0, 0, 0]
        if coordSys is None:
            coordSys = self.coordSys
        return self.withGlobalRotation(self.coordSys.rot @ rot @ self.coordSys.rot.T, rotCenter, coordSys)

    def withLocallyRotatedOptic(self, name, rot, rotCenter=None, coordSys=None):
        name = self._qualify(name)
        if rotCenter is None:
            rotCenter = [0, 0, 0]
        if coordSys is None:
            coordSys = self.itemDict[name].coordSys
        if name == self.name:
            return self.withLocalRotation(rot, rotCenter, coordSys)
        return self._replace(self._strip(name), lambda it: it.withLocalRotation(rot, rotCenter, coordSys),
                             lambda it, nm: it.withLocallyRotatedOptic(nm, rot, rotCenter, coordSys))

    def withGloballyRotatedOptic(self, name, rot, rotCenter=None, coordSys=None):
        name = self._qualify(name)
        if rotCenter is None:
            rotCenter = [0, 0, 0]
        if coordSys is None:
            coordSys = globalCoordSys
        if name == self.name:
            return self.withGlobalRotation(rot, rotCenter, coordSys)
        return self._replace(self._strip(name), lambda it: it.withGlobalRotation(rot, rotCenter, coordSys),
                             lambda it, nm: it.withGloballyRotatedOptic(nm, rot, rotCenter, coordSys))

    def withSurface(self, name, surface):
        name = self._qualify(name)
        return self._replace(self._strip(name), lambda it: it.withSurface(surface),
                             lambda it, nm: it.withSurface(nm, surface))

    def withPerturbedSurface(self, name, perturbation):
        name = self._names.get(name, name)
        return self.withSurface(name, self.itemDict[name].surface + perturbation)

    def withInsertedOptic(self, before, item):
        before = self._qualify(before)
        newItems = []
        for it in self.items:
            if self._names[it.name] == self._names[before]:
                newItems.append(item)
            newItems.append(it)
        return self.__class__(newItems, **self._newDict())

    def withRemovedOptic(self, item):
        item = self._qualify(item)
        newItems = [it for it in self.items if self._names[it.name] != self._names[item]]
        return self.__class__(newItems, **self._newDict())


class Lens(CompoundOptic):
    """A CompoundOptic of refractive interfaces sharing a medium."""

    def __init__(self, items, **kwargs):
        CompoundOptic.__init__(self, items, **kwargs)
