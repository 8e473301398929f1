from .coordSys import CoordSys
from .medium import ConstMedium

globalCoordSys = CoordSys()
vacuum = ConstMedium(1.0)
