"""Ray-factory cases shared by tests/golden/make_golden.py (reference
outputs) and tests/test_gpu_factories.py (this package): the factory name
and its keyword arguments, for the 12-surface system."""
import numpy as np

TH = dict(theta_x=np.deg2rad(0.35), theta_y=np.deg2rad(-0.2))


def cases():
    return [
        ("grid_even", "asGrid", dict(nx=16, wavelength=620e-9, **TH)),
        ("grid_odd", "asGrid", dict(nx=15, wavelength=500e-9, **TH)),
        ("grid_nxny", "asGrid", dict(nx=10, ny=7, wavelength=700e-9, **TH)),
        ("grid_dx", "asGrid", dict(dx=0.55, lx=8.36, wavelength=620e-9, **TH)),
        ("grid_rot", "asGrid", dict(nx=12, lx=(8.0, 1.5), wavelength=620e-9, **TH)),
        ("grid_1", "asGrid", dict(nx=1, wavelength=620e-9, **TH)),
        ("polar", "asPolar", dict(nrad=6, naz=30, wavelength=620e-9, **TH)),
        ("polar_inner0", "asPolar", dict(nrad=5, naz=24, inner=0.0, wavelength=400e-9, **TH)),
        ("polar_k4", "asPolar", dict(nrad=7, naz=40, kfold=4, outer=4.0, inner=1.0, wavelength=900e-9, **TH)),
        ("spokes", "asSpokes", dict(spokes=7, rings=5, wavelength=620e-9, **TH)),
        ("spokes_gq", "asSpokes", dict(rings=4, spacing="GQ", inner=2.558, wavelength=620e-9, **TH)),
        ("spokes_arrays", "asSpokes", dict(rings=np.array([1.0, 2.5, 4.0]),
                                           spokes=np.array([0.1, 1.7, 3.3, 5.0]), wavelength=620e-9, **TH)),
        ("fromstop", "fromStop", dict(x=np.array([0.0, 1.0, -3.2]), y=np.array([0.0, -2.0, 0.5]),
                                      wavelength=620e-9, **TH)),
    ]


def make(bt, optic, kind, kw):
    kw = dict(kw)
    if kind == "fromStop":
        return bt.RayVector.fromStop(kw.pop("x"), kw.pop("y"), optic=optic, **kw)
    return getattr(bt.RayVector, kind)(optic=optic, **kw)
