"""Host side of the device ray factories: the hexapolar ring table handed
to the device reproduces hexapolar()'s points bit for bit (batoid/utils.py
:483-535), and the grid parameters reproduce numpy's fftfreq lattice."""
import numpy as np
import pytest

from batoid_gb300.utils import hexapolar, hexapolar_rings


@pytest.mark.parametrize("args", [(4.18, 2.5, 6, 30, 6), (4.18, 0.0, 5, 24, 6), (1.0, 0.0, 1, 30, 6),
                                  (2.0, 0.3, 10, 64, 4), (3.0, 0.0, 2, 5, 6)])
def test_ring_table_reproduces_hexapolar(args):
    rr, th = hexapolar(*args, rth=True)
    r, step, off = hexapolar_rings(*args)
    n = int(off[-1])
    assert n == len(rr) and len(off) == len(r) + 1
    k = np.searchsorted(off, np.arange(n), side="right") - 1
    # the device computes (i - off[k]) * step[k] and r[k]
    np.testing.assert_array_equal(r[k], rr)
    np.testing.assert_array_equal((np.arange(n) - off[k]) * step[k], th)


@pytest.mark.parametrize("nx", [1, 2, 7, 16, 33])
def test_grid_lattice_matches_fftfreq(nx):
    x_d = 1. if nx <= 2 else (nx - (2 if nx % 2 == 0 else 1)) / nx
    val = 1.0 / (nx * x_d)
    # the device computes (i - nx // 2) * val
    dev = (np.arange(nx) - nx // 2) * val
    np.testing.assert_array_equal(dev, np.fft.fftshift(np.fft.fftfreq(nx, x_d)))
