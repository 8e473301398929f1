"""batoid_gb300: GB300-native sequential ray tracing behind batoid's Python API.

Rays live in device memory; every per-ray computation runs in the CUDA
library libbatoid_gb300.so (C-ABI: include/batoid_gb300.h).  The public names
mirror jmeyers314/batoid (batoid/__init__.py).
"""
__version__ = "0.1.0"

from .rayVector import RayVector, concatenateRayVectors
from .coordSys import CoordSys, RotX, RotY, RotZ
from .coordTransform import CoordTransform
from .surface import (
    Surface, Plane, Paraboloid, Sphere, Quadric, Asphere, Bicubic, Sum, Tilted, Zernike,
    PolynomialSurface,
)
from .trace import intersect, applyForwardTransform, applyReverseTransform, obscure, reflect, refract
from .medium import Medium, ConstMedium, TableMedium, SellmeierMedium, SumitaMedium, Air
from .obscuration import (
    Obscuration, ObscCircle, ObscAnnulus, ObscRectangle, ObscRay, ObscPolygon, ObscNegation,
    ObscUnion, ObscIntersection,
)
from .coating import Coating, SimpleCoating
from .optic import Optic, CompoundOptic, Lens
from .optic import Interface, RefractiveInterface, Mirror, Detector, Baffle, OPDScreen
from .lattice import Lattice
from . import utils
from .constants import globalCoordSys, vacuum
from .analysis import (huygensPSF, huygensPSFs, wavefront, zernike, dkdu, drdth, dthdr, spot, fftPSF, zernikeGQ, zernikeTA,
                       zernikeXYAberrations, doubleZernike, exitPupilPos, focalLength)
from . import global_vars

import os
datadir = os.path.join(os.path.dirname(__file__), "data")
