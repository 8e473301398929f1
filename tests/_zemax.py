"""Zemax golden-trace helpers (reference tests/test_zemax.py:16-63, 413-700)."""
import copy
import json

import numpy as np

from _helpers import golden

LSST_ZSURF = [4, 5, 7, 9, 10, 11, 12, 13, 14, 15, 16, 17]
HSC_SURF = [3, 6, 7, 8, 9, 11, 12, 13, 14, 16, 17, 18, 19, 20, 21, 24, 25, 28, 29, 31]
HSC_NAMES = ['PM', 'G1_entrance', 'G1_exit', 'G2_entrance', 'G2_exit', 'ADC1_entrance', 'ADC1_exit',
             'ADC2_entrance', 'ADC2_exit', 'G3_entrance', 'G3_exit', 'G4_entrance', 'G4_exit', 'G5_entrance',
             'G5_exit', 'F_entrance', 'F_exit', 'W_entrance', 'W_exit', 'D']


DECAM_ZSURF = [2, 3, 5, 7, 9, 10, 11, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 28, 29, 30, 31, 32, 33, 34, 35,
               36, 37, 38, 39, 40]
CBP_IDX = {'Schmidt_plate_entrance': 1, 'Schmidt_plate_exit': 2, 'stop': 3, 'turning_flat': 5, 'PM': 7,
           'flat_hole': 9, 'L1_entrance': 11, 'L1_exit': 12, 'L2_entrance': 13, 'L2_exit': 14, 'L3_entrance': 15,
           'L3_exit': 16, 'Detector': 17}
COMCAM_IDX = {'M1': 5, 'M2': 6, 'M3': 8, 'L1_entrance': 10, 'L1_exit': 11, 'L2_entrance': 12, 'L2_exit': 13,
              'Filter_entrance': 14, 'Filter_exit': 15, 'L3_entrance': 16, 'L3_exit': 17, 'Detector': 18}


def optic(which, fixture="zemax"):
    from batoid_gb300.parse import parse_optic
    cfg = json.loads(str(golden(fixture)[f"{which}_config"]))
    return parse_optic(copy.deepcopy(cfg["opticalSystem"]))


def srt(g, key):
    """A Zemax single-ray trace in the reference's conventions (tests/
    test_zemax.py:560-580): x, z and their cosines flip sign, Hx too;
    wavelength in m, positions in m.  Returns (wavelength, Hx, Hy, pos
    (rows, 3), cosines (rows, 3))."""
    wl = float(g[f"{key}_wavelength_um"][0]) * 1e-6
    Hx, Hy, Px, Py = g[f"{key}_hp"]
    rows = g[f"{key}_rows"]
    pos = np.stack([-rows[:, 1], rows[:, 2], -rows[:, 3]], axis=1) * 1e-3
    cos = np.stack([-rows[:, 4], rows[:, 5], -rows[:, 6]], axis=1)
    return wl, -Hx, Hy, pos, cos


def cbp_start(g, i):
    """CBP input ray (tests/test_zemax.py:582-586): the first row's point,
    the field's Zemax direction, rewound 0.1 m.  (x, y, z, vx, vy, vz, t, wl)."""
    from batoid_gb300.utils import zemaxToDirCos
    wl, Hx, Hy, pos, _ = srt(g, f"cbp{i}")
    v = np.array(zemaxToDirCos(Hx * np.deg2rad(2.05), Hy * np.deg2rad(2.05)), dtype=float)
    r = pos[0] - 0.1 * v
    return (*r, *v, -0.1, wl)


def comcam_start(g, band, i):
    """ComCam input ray (tests/test_zemax.py:648-652): first row, direction
    towards the second.  (x, y, z, vx, vy, vz, t, wl)."""
    wl, _, _, pos, _ = srt(g, f"comcam_{band}{i}")
    dr = pos[1] - pos[0]
    v = dr / np.linalg.norm(dr)
    return (*pos[0], *v, 0.0, wl)


def check_decam(global_rays, arr, atol=1e-9):
    """As check_lsst for DECam's surface numbering (tests/test_zemax.py:466-520)."""
    check_lsst(global_rays, arr, atol=atol, zsurf=[i - 1 for i in DECAM_ZSURF])


def check_cbp(by_name, g, i, atol=1e-10):
    _, _, _, pos, cos = srt(g, f"cbp{i}")
    for name, (x, y, z, vx, vy, vz) in by_name.items():
        if name == 'flat_hole':
            continue  # the reference's test skips it (Zemax's tilt convention there)
        idx = CBP_IDX[name]
        np.testing.assert_allclose([x, y, z], pos[idx], rtol=0, atol=atol, err_msg=name)
        v = np.array([vx, vy, vz])
        v /= np.linalg.norm(v)
        if v[2] > 0:
            v = -v
        np.testing.assert_allclose(v, cos[idx], rtol=0, atol=atol, err_msg=name)


def check_comcam(by_name, g, band, i, atol=1e-9):
    _, _, _, pos, _ = srt(g, f"comcam_{band}{i}")
    for name, (x, y, z) in by_name.items():
        np.testing.assert_allclose([x, y, z], pos[COMCAM_IDX[name] - 1], rtol=0, atol=atol, err_msg=name)


def check_lsst(global_rays, arr, atol=1e-10, zsurf=None):
    """global_rays: list of (x, y, z, vx, vy, vz) per surface in trace order."""
    for (x, y, z, vx, vy, vz), iz in zip(global_rays, zsurf or LSST_ZSURF):
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
