"""Zemax golden-trace helpers (reference tests/test_zemax.py:16-63, 413-462)."""
import copy
import json

import numpy as np

from _helpers import golden

LSST_ZSURF = [4, 5, 7, 9, 10, 11, 12, 13, 14, 15, 16, 17]
HSC_SURF = [3, 6, 7, 8, 9, 11, 12, 13, 14, 16, 17, 18, 19, 20, 21, 24, 25, 28, 29, 31]
HSC_NAMES = ['PM', 'G1_entrance', 'G1_exit', 'G2_entrance', 'G2_exit', 'ADC1_entrance', 'ADC1_exit',
             'ADC2_entrance', 'ADC2_exit', 'G3_entrance', 'G3_exit', 'G4_entrance', 'G4_exit', 'G5_entrance',
             'G5_exit', 'F_entrance', 'F_exit', 'W_entrance', 'W_exit', 'D']


def optic(which):
    from batoid_gb300.parse import parse_optic
    cfg = json.loads(str(golden("zemax")[f"{which}_config"]))
    return parse_optic(copy.deepcopy(cfg["opticalSystem"]))


def check_lsst(global_rays, arr, atol=1e-10):
    """global_rays: list of (x, y, z, vx, vy, vz) per surface in trace order."""
    for (x, y, z, vx, vy, vz), iz in zip(global_rays, LSST_ZSURF):
        n = 1.0 / np.sqrt(vx * vx + vy * vy + vz * vz)
        np.testing.assert_allclose(x, arr[iz][0] / 1e3, rtol=0, atol=atol)
        np.testing.assert_allclose(y, arr[iz][1] / 1e3, rtol=0, atol=atol)
        np.testing.assert_allclose(abs(z), abs(arr[iz][2] / 1e3), rtol=0, atol=atol)
        np.testing.assert_allclose(abs(vx * n), abs(arr[iz][3]), rtol=0, atol=atol)
        np.testing.assert_allclose(abs(vy * n), abs(arr[iz][4]), rtol=0, atol=atol)
        np.testing.assert_allclose(abs(vz * n), abs(arr[iz][5]), rtol=0, atol=atol)


def check_hsc(by_name, arr, atol=1e-9):
    """by_name: name -> (x, y, z, vx, vy, vz) in global coordinates."""
    for name, iz in zip(HSC_NAMES, HSC_SURF):
        x, y, z, vx, vy, vz = by_name[name]
        np.testing.assert_allclose([x, y, z - 16.0], arr[iz - 1][1:4] / 1000, rtol=0, atol=atol, err_msg=name)
        v = np.array([vx, vy, vz])
        np.testing.assert_allclose(v / np.linalg.norm(v), arr[iz - 1][4:7], rtol=0, atol=atol, err_msg=name)
