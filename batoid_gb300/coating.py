"""Coatings (batoid/coating.py; src/coating.cpp)."""
from . import _lib
from ._handle import Handle


class Coating:
    def getCoefs(self, wavelength, cosIncidenceAngle):
        return self.getReflect(wavelength, cosIncidenceAngle), self.getTransmit(wavelength, cosIncidenceAngle)

    def __ne__(self, rhs):
        return not (self == rhs)


class SimpleCoating(Coating):
    """Constant reflectivity and transmissivity (src/coating.cpp:28-39)."""

    def __init__(self, reflectivity, transmissivity):
        self.reflectivity = reflectivity
        self.transmissivity = transmissivity
        self._coating = Handle(_lib.new_handle(_lib.lib().bt_simple_coating_create, float(reflectivity),
                                               float(transmissivity)), "bt_coating_destroy")

    def getReflect(self, wavelength, cosIncidenceAngle):
        return self.reflectivity

    def getTransmit(self, wavelength, cosIncidenceAngle):
        return self.transmissivity

    def __eq__(self, rhs):
        return (isinstance(rhs, SimpleCoating) and self.reflectivity == rhs.reflectivity
                and self.transmissivity == rhs.transmissivity)

    def __getstate__(self):
        return self.reflectivity, self.transmissivity

    def __setstate__(self, args):
        self.__init__(*args)

    def __hash__(self):
        return hash(("SimpleCoating", self.reflectivity, self.transmissivity))

    def __repr__(self):
        return f"SimpleCoating({self.reflectivity}, {self.transmissivity})"
