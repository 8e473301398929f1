"""Annular Zernike polynomials (Noll indexing) as Cartesian polynomials.

The reference obtains these from GalSim (batoid/surface.py:464-483,
batoid/analysis.py:563-566), which is not available here.  This module
builds them from the published definitions:

* Noll (1976) ordering j -> (n, m): n grows with j; within an order, |m|
  grows; even j carry cos(m theta), odd j sin(|m| theta).
* Mahajan (1981) annular polynomials: for each m the radial factors are the
  polynomials in rho of the form rho^m * P(rho^2) that are orthogonal over
  eps <= rho <= 1 with weight rho, with positive leading coefficient, and
  normalised so that (1/(pi (1 - eps^2))) * integral over the annulus of
  Z_j^2 = 1.  At eps = 0 they reduce to the circular Zernike polynomials.

The orthogonalisation is done exactly in rational arithmetic (an LDL^T
factorisation of the monomial Gram matrix), so the coefficients carry only
the final float rounding.
"""
from fractions import Fraction
from functools import lru_cache
from math import comb, sqrt

import numpy as np


def noll_to_nm(j):
    """Noll index (j >= 1) to (n, m); m < 0 denotes the sin term."""
    if j < 1:
        raise ValueError("Noll index must be >= 1")
    n = 0
    j1 = j - 1
    while j1 > n:
        n += 1
        j1 -= n
    m = (n % 2) + 2 * ((j1 + ((n + 1) % 2)) // 2)
    if m != 0 and j % 2 == 1:
        m = -m
    return n, m


def noll_nmax(jmax):
    return noll_to_nm(jmax)[0] if jmax >= 1 else 0


@lru_cache(maxsize=None)
def _radial_table(m, nmax, eps):
    """Orthonormal radial polynomials for fixed |m| and n = m, m+2, ..., nmax.

    Returns {n: [c_0, c_1, ...]} with R_n(rho) = sum_k c_k rho^(m+2k) and
    integral_eps^1 R_n^2 rho drho = 1.
    """
    e = Fraction(eps)
    e2 = e * e
    ks = list(range((nmax - m) // 2 + 1))
    size = len(ks)
    # Gram matrix of rho^(m+2a), rho^(m+2b): integral rho^(2m+2a+2b+1) = (1 - eps^p)/p
    G = [[None] * size for _ in range(size)]
    for a in ks:
        for b in ks:
            p = 2 * m + 2 * a + 2 * b + 2
            G[a][b] = (1 - e2 ** (p // 2)) / p
    # LDL^T with unit-lower L
    L = [[Fraction(0)] * size for _ in range(size)]
    Dg = [Fraction(0)] * size
    for i in range(size):
        for j in range(i + 1):
            s = G[i][j] - sum(L[i][k] * L[j][k] * Dg[k] for k in range(j))
            if i == j:
                Dg[i] = s
                L[i][i] = Fraction(1)
            else:
                L[i][j] = s / Dg[j]
    # inverse of unit-lower L (rows give orthogonal polynomials)
    Linv = [[Fraction(0)] * size for _ in range(size)]
    for i in range(size):
        Linv[i][i] = Fraction(1)
        for j in range(i - 1, -1, -1):
            Linv[i][j] = -sum(L[i][k] * Linv[k][j] for k in range(j, i))
    out = {}
    for i in range(size):
        scale = 1.0 / sqrt(float(Dg[i]))
        out[m + 2 * i] = [float(Linv[i][k]) * scale for k in range(i + 1)]
    return out


@lru_cache(maxsize=None)
def zernike_xy_unit(j, eps):
    """Cartesian coefficients C[a][b] (x^a y^b) of Z_j on the unit annulus."""
    n, m = noll_to_nm(j)
    am = abs(m)
    rad = _radial_table(am, n if (n - am) % 2 == 0 else n, float(eps))[n]
    # angular normalisation: mean of Z^2 over the annulus is 1
    area = 1.0 - float(eps) ** 2
    norm = sqrt(area / (1.0 if am != 0 else 2.0))
    C = np.zeros((n + 1, n + 1))
    # (x + i y)^am = sum_q comb(am, q) x^(am-q) (i y)^q
    ang = {}
    for q in range(am + 1):
        c = comb(am, q)
        # i^q: real part for even q, imaginary part for odd q
        if m >= 0:
            if q % 2 == 0:
                ang[(am - q, q)] = ang.get((am - q, q), 0.0) + c * (-1) ** (q // 2)
        else:
            if q % 2 == 1:
                ang[(am - q, q)] = ang.get((am - q, q), 0.0) + c * (-1) ** ((q - 1) // 2)
    for k, ck in enumerate(rad):
        # (x^2 + y^2)^k
        for r in range(k + 1):
            ckr = ck * comb(k, r)
            for (ax, ay), cang in ang.items():
                C[ax + 2 * r, ay + 2 * (k - r)] += norm * ckr * cang
    return C


def zernike_xy(coef, R_outer=1.0, R_inner=0.0):
    """Cartesian coefficient array of sum_j coef[j] Z_j(x/R_outer, y/R_outer)
    (coef[0] ignored, Noll convention), shape (n+1, n+1)."""
    coef = np.asarray(coef, dtype=float)
    jmax = len(coef) - 1
    nmax = noll_nmax(jmax)
    eps = R_inner / R_outer
    C = np.zeros((nmax + 1, nmax + 1))
    for j in range(1, jmax + 1):
        if coef[j] == 0.0:
            continue
        Cj = zernike_xy_unit(j, eps)
        C[:Cj.shape[0], :Cj.shape[1]] += coef[j] * Cj
    a = np.arange(nmax + 1)
    C /= float(R_outer) ** (a[:, None] + a[None, :])
    return C


def grad_xy(C):
    """d/dx and d/dy coefficient arrays, one smaller in each dimension
    (1x1 zero arrays for a constant)."""
    n = C.shape[0]
    if n <= 1:
        return np.zeros((1, 1)), np.zeros((1, 1))
    gx = np.zeros((n - 1, n - 1))
    gy = np.zeros((n - 1, n - 1))
    for a in range(n - 1):
        for b in range(n - 1):
            gx[a, b] = (a + 1) * C[a + 1, b]
            gy[a, b] = (b + 1) * C[a, b + 1]
    return gx, gy


def horner2d_host(x, y, C):
    """Evaluate sum C[a][b] x^a y^b (host reference for tests)."""
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    out = np.zeros(np.broadcast(x, y).shape)
    for a in range(C.shape[0] - 1, -1, -1):
        row = np.zeros_like(out)
        for b in range(C.shape[1] - 1, -1, -1):
            row = row * y + C[a, b]
        out = out * x + row
    return out


def basis_xy(jmax, R_outer=1.0, R_inner=0.0):
    """Cartesian coefficient arrays of Z_1..Z_jmax (each (n+1, n+1) padded to
    the largest n), as an array of shape (jmax, n+1, n+1)."""
    nmax = noll_nmax(jmax)
    out = np.zeros((jmax, nmax + 1, nmax + 1))
    for j in range(1, jmax + 1):
        c = np.zeros(j + 1)
        c[j] = 1.0
        Cj = zernike_xy(c, R_outer, R_inner)
        out[j - 1, :Cj.shape[0], :Cj.shape[1]] = Cj
    return out
