"""Seeded small inputs shared by the oracle and GPU parity tests."""
from __future__ import annotations

import numpy as np

import oracle as O


def F(a):
    return np.asfortranarray(a, dtype=np.float64)


def curvilinear(ni=14, nj=10, nk=8, seed=0, shear=0.1):
    """Sheared/stretched curvilinear grid on [0,1]^3 with a smooth level set
    crossing it and a smooth velocity field (all FP64, Fortran order)."""
    rng = np.random.default_rng(seed)
    xi, et, ze = np.meshgrid(np.linspace(0, 1, ni), np.linspace(0, 1, nj), np.linspace(0, 1, nk), indexing="ij")
    a = rng.uniform(-shear, shear, 3)
    x = F(xi + a[0] * et + 0.03 * np.sin(2 * np.pi * ze))
    y = F(et + a[1] * ze)
    z = F(ze ** 1.2 + a[2] * xi)
    phi = F(0.45 - z + 0.06 * np.sin(2 * np.pi * x) * np.cos(np.pi * y) + 0.01 * rng.standard_normal((ni, nj, nk)))
    q = np.zeros((4, ni, nj, nk), order="F")
    q[1] = 0.8 + 0.3 * np.sin(np.pi * y)
    q[2] = -0.4 * np.cos(np.pi * x)
    q[3] = 0.2 * np.sin(2 * np.pi * x) * np.sin(np.pi * z)
    g = O.make_grid(ni, nj, nk)
    return g, x, y, z, phi, q


def sphere(n=12):
    """Cartesian unit box with the sphere of radius 0.15 at (0.35,0.35,0.35)."""
    X, Y, Z = np.meshgrid(*(np.linspace(0, 1, n),) * 3, indexing="ij")
    phi = F(0.15 - np.sqrt((X - 0.35) ** 2 + (Y - 0.35) ** 2 + (Z - 0.35) ** 2))
    sx, sy, sz = np.sin(np.pi * X), np.sin(np.pi * Y), np.sin(np.pi * Z)
    s2x, s2y, s2z = np.sin(2 * np.pi * X), np.sin(2 * np.pi * Y), np.sin(2 * np.pi * Z)
    q = np.zeros((4, n, n, n), order="F")
    q[1] = 2.0 * sx ** 2 * s2y * s2z
    q[2] = -s2x * sy ** 2 * s2z
    q[3] = -s2x * s2y * sz ** 2
    return O.make_grid(n, n, n), F(X), F(Y), F(Z), phi, q


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = max(float(np.abs(b).max()), 1e-300)
    return float(np.abs(a - b).max()) / den
