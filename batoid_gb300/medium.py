"""Refractive media (batoid/medium.py; src/medium.cpp).  getN runs on the GPU."""
import numpy as np

from . import _device as D
from . import _lib
from ._handle import Handle


class Medium:
    def getN(self, wavelength):
        """Refractive index at vacuum wavelength(s) in meters."""
        scalar = np.ndim(wavelength) == 0
        w = D.to_device(np.atleast_1d(np.asarray(wavelength, dtype=float)).ravel())
        out = D.empty(w.numel())
        _lib.check(_lib.lib().bt_medium_getN(self._medium.ptr, D.ptr(w), D.ptr(out), w.numel(),
                                             D.stream_ptr()))
        res = D.to_host(out)
        if scalar:
            return float(res[0])
        return res.reshape(np.shape(wavelength))

    def __ne__(self, rhs):
        return not (self == rhs)


class ConstMedium(Medium):
    def __init__(self, n):
        self.n = n
        self._medium = Handle(_lib.new_handle(_lib.lib().bt_const_medium_create, float(n)),
                              "bt_medium_destroy")

    def getN(self, wavelength):
        # a constant needs no kernel
        if np.ndim(wavelength) == 0:
            return float(self.n)
        return np.full(np.shape(wavelength), float(self.n))

    def __eq__(self, rhs):
        return type(rhs) == type(self) and self.n == rhs.n

    def __getstate__(self):
        return self.n

    def __setstate__(self, n):
        self.__init__(n)

    def __hash__(self):
        return hash(("batoid.ConstMedium", self.n))

    def __repr__(self):
        return f"ConstMedium({self.n})"


class TableMedium(Medium):
    def __init__(self, wavelengths, ns):
        self.wavelengths = np.array(wavelengths, dtype=float)
        self.ns = np.array(ns, dtype=float)
        a, pa = _lib.dptr(self.wavelengths)
        b, pb = _lib.dptr(self.ns)
        self._medium = Handle(_lib.new_handle(_lib.lib().bt_table_medium_create, pa, pb,
                                              len(self.wavelengths)), "bt_medium_destroy")

    @classmethod
    def fromTxt(cls, filename, **kwargs):
        import glob
        import os
        try:
            wavelength, n = np.loadtxt(filename, unpack=True, **kwargs)
        except IOError:
            from . import datadir
            for candidate in glob.glob(os.path.join(datadir, "**", "*.txt"), recursive=True):
                if os.path.basename(candidate) == filename:
                    wavelength, n = np.loadtxt(candidate, unpack=True, **kwargs)
                    break
            else:
                raise FileNotFoundError(filename)
        return TableMedium(wavelength * 1e-6, n)

    def __eq__(self, rhs):
        return (type(rhs) == type(self) and np.array_equal(self.wavelengths, rhs.wavelengths)
                and np.array_equal(self.ns, rhs.ns))

    def __getstate__(self):
        return self.wavelengths, self.ns

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("batoid.TableMedium", tuple(self.wavelengths), tuple(self.ns)))

    def __repr__(self):
        return f"TableMedium({self.wavelengths!r}, {self.ns!r})"


def _six(args, kwargs, names):
    if len(args) == 6:
        return tuple(float(a) for a in args)
    if len(args) == 1:
        return tuple(float(a) for a in args[0])
    if kwargs:
        return tuple(float(kwargs[k]) for k in names)
    raise ValueError("Incorrect number of arguments")


class SellmeierMedium(Medium):
    """n^2 = 1 + sum B_i x/(x - C_i), x = (lambda/um)^2 (src/medium.cpp:145-149)."""

    def __init__(self, *args, **kwargs):
        self.coefs = _six(args, kwargs, ['B1', 'B2', 'B3', 'C1', 'C2', 'C3'])
        self._medium = Handle(_lib.new_handle(_lib.lib().bt_sellmeier_medium_create, *self.coefs),
                              "bt_medium_destroy")

    def __eq__(self, rhs):
        return type(rhs) == type(self) and self.coefs == rhs.coefs

    def __getstate__(self):
        return self.coefs

    def __setstate__(self, coefs):
        self.__init__(coefs)

    def __hash__(self):
        return hash(("batoid.SellmeierMedium", self.coefs))

    def __repr__(self):
        return f"SellmeierMedium({self.coefs})"


class SumitaMedium(Medium):
    def __init__(self, *args, **kwargs):
        self.coefs = _six(args, kwargs, ['A0', 'A1', 'A2', 'A3', 'A4', 'A5'])
        self._medium = Handle(_lib.new_handle(_lib.lib().bt_sumita_medium_create, *self.coefs),
                              "bt_medium_destroy")

    def __eq__(self, rhs):
        return type(rhs) == type(self) and self.coefs == rhs.coefs

    def __getstate__(self):
        return self.coefs

    def __setstate__(self, coefs):
        self.__init__(coefs)

    def __hash__(self):
        return hash(("batoid.SumitaMedium", self.coefs))

    def __repr__(self):
        return f"SumitaMedium({self.coefs})"


class Air(Medium):
    """Edlen/Filippenko air index; SI inputs (kPa, K, kPa) (src/medium.cpp:214-245)."""

    def __init__(self, pressure=69.328, temperature=293.15, h2o_pressure=1.067):
        self.pressure = pressure
        self.temperature = temperature
        self.h2o_pressure = h2o_pressure
        self._medium = Handle(_lib.new_handle(_lib.lib().bt_air_create, float(pressure),
                                              float(temperature), float(h2o_pressure)),
                              "bt_medium_destroy")

    def __eq__(self, rhs):
        return (type(rhs) == type(self) and self.pressure == rhs.pressure
                and self.temperature == rhs.temperature and self.h2o_pressure == rhs.h2o_pressure)

    def __getstate__(self):
        return self.pressure, self.temperature, self.h2o_pressure

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("batoid.Air", self.pressure, self.temperature, self.h2o_pressure))

    def __repr__(self):
        return f"Air({self.pressure}, {self.temperature}, {self.h2o_pressure})"
