"""Synthetic workloads of the level-set transport step (host, FP64, numpy).

The reference ships no input decks, so each workload is generated from its
analytic description: grid coordinates, initial level set phi0 (water is
phi > 0, as in AnalyticalPhiSphere, src/AdvectionMethods.F90:1733) and the
Cartesian velocity q(2:4).  Sizes are parameters so the same geometry can be
run small (parity tests) or at full size (benchmarks).

  sphere_deformation   64^3 unit box, sphere r=0.15 at (0.35,0.35,0.35), LeVeque
                       3-D deformation field, WENO3 + TVD-RK3 at CFL 0.5, 5
                       reinit pseudo-steps per step, eps = 1.5 h, 6-cell band.
  solitary_wave        256x128x96 curvilinear grid x = 8 xi + 0.05 sin(2 pi eta),
                       y = 2 eta, z = zeta^1.3, phi0 = z - (0.5 + A sech^2(k(x-2))),
                       uniform flow + solitary-wave perturbation, CFL 0.4, 10
                       reinit pseudo-steps per step.
  large_free_surface   512x256x256, the same mapping on a 16x4x2 domain, 3-D
                       free surface phi0 = z - 1 - 0.08 sech^2(k(x-4)) (1 + 0.2
                       cos(2 pi y / 4)), k = sqrt(3 A / (4 d^3)) with A = 0.08,
                       depth d = 1; velocity (1,0,0) + A sqrt(g d) sech^2 in u
                       and w; CFL 0.4, 10 reinit pseudo-steps per step.
"""
from __future__ import annotations

import dataclasses as dc
import math
from typing import Callable, Optional

import numpy as np

from .api import Grid
from .params import LsmParams


@dc.dataclass
class Case:
    name: str
    grid: Grid
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    phi0: np.ndarray
    params: LsmParams
    steps: int
    cfl: float
    velocity: Callable[[float], np.ndarray]   # t -> q (4, ni, nj, nk), Fortran order
    redistance_iters: int = 0
    h: float = 0.0

    def q(self, t: float = 0.0) -> np.ndarray:
        return self.velocity(t)

    def time_step(self, csi: np.ndarray, eta: np.ndarray, zet: np.ndarray, t: float = 0.0) -> float:
        """CFL time step in computational space: cfl / max_nodes max_m |grad xi_m . u|."""
        q = self.velocity(t)
        u = q[1:4]
        s = 0.0
        for m in (csi, eta, zet):
            U = np.abs(m[0] * u[0] + m[1] * u[1] + m[2] * u[2])
            s = max(s, float(U.max()))
        return self.cfl / s


def _fortran(a: np.ndarray) -> np.ndarray:
    return np.asfortranarray(a, dtype=np.float64)


def _mesh(ni, nj, nk):
    xi = np.arange(ni, dtype=np.float64) / (ni - 1)
    eta = np.arange(nj, dtype=np.float64) / (nj - 1)
    zeta = np.arange(nk, dtype=np.float64) / (nk - 1)
    return np.meshgrid(xi, eta, zeta, indexing="ij")


def sphere_deformation(n: int = 64, steps: int = 100, reinit_iters: int = 5) -> Case:
    X, Y, Z = _mesh(n, n, n)
    h = 1.0 / (n - 1)
    x, y, z = _fortran(X), _fortran(Y), _fortran(Z)
    phi0 = _fortran(0.15 - np.sqrt((X - 0.35) ** 2 + (Y - 0.35) ** 2 + (Z - 0.35) ** 2))
    sx, sy, sz = np.sin(np.pi * X), np.sin(np.pi * Y), np.sin(np.pi * Z)
    s2x, s2y, s2z = np.sin(2 * np.pi * X), np.sin(2 * np.pi * Y), np.sin(2 * np.pi * Z)
    u0 = 2.0 * sx ** 2 * s2y * s2z
    v0 = -s2x * sy ** 2 * s2z
    w0 = -s2x * s2y * sz ** 2

    def velocity(t: float) -> np.ndarray:
        c = math.cos(math.pi * t / 3.0)
        q = np.zeros((4, n, n, n), order="F")
        q[1], q[2], q[3] = u0 * c, v0 * c, w0 * c
        return q

    p = LsmParams(epslsm=1.5 * h, numiter_lsm=1, delti_lsm=0.5 * h / 2.0, RNitermax=reinit_iters,
                  RNtimestep=0.5 * h, RNfreq=1, btype_lsm=(1,) * 6, isnarrow=1, narrowcoef=4.0, orderAD=1,
                  BigPhi=5.0, M_Sphi0=1)
    return Case("sphere_deformation_%dx%dx%d" % (n, n, n), Grid(n, n, n), x, y, z, phi0, p, steps, 0.5,
                velocity, 0, h)


def solitary_wave(ni: int = 256, nj: int = 128, nk: int = 96, steps: int = 200, reinit_iters: int = 10,
                  Lx: float = 8.0, Ly: float = 2.0, Lz: float = 1.0, x0: float = 2.0,
                  redistance_iters: int = 50) -> Case:
    XI, ET, ZE = _mesh(ni, nj, nk)
    X = Lx * XI + 0.05 * np.sin(2 * np.pi * ET)
    Y = Ly * ET
    Z = Lz * ZE ** 1.3
    A, depth, g = 0.1, 0.5, 9.81
    k = math.sqrt(3.0 * A / (4.0 * depth ** 3))
    sech2 = 1.0 / np.cosh(k * (X - x0)) ** 2
    phi0 = _fortran(Z - (depth + A * sech2))
    c = A * math.sqrt(g * depth)
    u = 1.0 + c * sech2
    w = c * sech2
    q0 = np.zeros((4, ni, nj, nk), order="F")
    q0[1], q0[3] = u, w

    def velocity(t: float) -> np.ndarray:
        return q0

    dx, dy = Lx / (ni - 1), Ly / (nj - 1)
    dz_min = Lz * (1.0 / (nk - 1)) ** 1.3
    h = max(dx, dy)
    p = LsmParams(epslsm=1.5 * h, numiter_lsm=1, delti_lsm=0.0, RNitermax=reinit_iters,
                  RNtimestep=0.5 * min(dx, dy, dz_min), RNfreq=1, btype_lsm=(1,) * 6, isnarrow=1,
                  narrowcoef=4.0, orderAD=1, BigPhi=5.0, M_Sphi0=1)
    return Case("solitary_wave_%dx%dx%d" % (ni, nj, nk), Grid(ni, nj, nk), _fortran(X), _fortran(Y), _fortran(Z),
                phi0, p, steps, 0.4, velocity, redistance_iters, h)


def large_free_surface(ni: int = 512, nj: int = 256, nk: int = 256, steps: int = 200,
                       reinit_iters: int = 10) -> Case:
    Lx, Ly, Lz, x0, A, depth, g = 16.0, 4.0, 2.0, 4.0, 0.08, 1.0, 9.81
    XI, ET, ZE = _mesh(ni, nj, nk)
    X = Lx * XI + 0.05 * np.sin(2 * np.pi * ET)
    Y = Ly * ET
    Z = Lz * ZE ** 1.3
    k = math.sqrt(3.0 * A / (4.0 * depth ** 3))
    sech2 = 1.0 / np.cosh(k * (X - x0)) ** 2
    phi0 = _fortran(Z - depth - A * sech2 * (1.0 + 0.2 * np.cos(2 * np.pi * Y / 4.0)))
    c = A * math.sqrt(g * depth)
    q0 = np.zeros((4, ni, nj, nk), order="F")
    q0[1] = 1.0 + c * sech2
    q0[3] = c * sech2
    del XI, ET, ZE, sech2

    def velocity(t: float) -> np.ndarray:
        return q0

    dx, dy = Lx / (ni - 1), Ly / (nj - 1)
    dz_min = Lz * (1.0 / (nk - 1)) ** 1.3
    h = max(dx, dy)
    p = LsmParams(epslsm=1.5 * h, numiter_lsm=1, delti_lsm=0.0, RNitermax=reinit_iters,
                  RNtimestep=0.5 * min(dx, dy, dz_min), RNfreq=1, btype_lsm=(1,) * 6, isnarrow=1,
                  narrowcoef=4.0, orderAD=1, BigPhi=5.0, M_Sphi0=1)
    return Case("large_free_surface_%dx%dx%d" % (ni, nj, nk), Grid(ni, nj, nk), _fortran(X), _fortran(Y),
                _fortran(Z), phi0, p, steps, 0.4, velocity, 0, h)


@dc.dataclass
class Instance:
    """One instance of a batched workload (single zone, all faces physical)."""
    grid: Grid
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    phi0: np.ndarray
    q: np.ndarray
    eps: float
    dtau: float
    cfl: float

    def time_step(self, csi, eta, zet) -> float:
        u = self.q[1:4]
        s = max(float(np.abs(m[0] * u[0] + m[1] * u[1] + m[2] * u[2]).max()) for m in (csi, eta, zet))
        return self.cfl / s


def batched_instances(n_inst: int = 64, lo: int = 32, hi: int = 96, seed: int = 0, cfl: float = 0.5) -> list:
    """64 independent instances with per-axis sizes drawn from {lo..hi}: unit box
    mapped by identity + random shear (off-diagonal coefficients U(-0.1, 0.1)),
    phi0 = z - 0.5 - (4 Fourier modes, amplitudes U(0, 0.05), wavenumbers 1-4),
    velocity = curl of a vector potential with 8 Fourier modes (Gaussian
    amplitudes, sigma = 0.2), divergence-free."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, size=(n_inst, 3))
    out = []
    for b in range(n_inst):
        ni, nj, nk = (int(v) for v in sizes[b])
        XI, ET, ZE = _mesh(ni, nj, nk)
        S = np.eye(3)
        for r in range(3):
            for c in range(3):
                if r != c:
                    S[r, c] = rng.uniform(-0.1, 0.1)
        X = S[0, 0] * XI + S[0, 1] * ET + S[0, 2] * ZE
        Y = S[1, 0] * XI + S[1, 1] * ET + S[1, 2] * ZE
        Z = S[2, 0] * XI + S[2, 1] * ET + S[2, 2] * ZE
        phi = Z - 0.5
        for _ in range(4):
            a = rng.uniform(0.0, 0.05)
            kx, ky = rng.integers(1, 5, size=2)
            th = rng.uniform(0, 2 * np.pi)
            phi = phi - a * np.cos(2 * np.pi * (kx * X + ky * Y) + th)
        U = np.zeros((3,) + X.shape)
        for _ in range(8):
            amp = rng.normal(0.0, 0.2, size=3)
            kv = rng.integers(1, 5, size=3)
            th = rng.uniform(0, 2 * np.pi)
            c = 2 * np.pi * np.cos(2 * np.pi * (kv[0] * X + kv[1] * Y + kv[2] * Z) + th)
            cr = np.cross(kv, amp)          # curl(a sin(2 pi k.x + th)) = 2 pi cos(...) (k x a)
            for d in range(3):
                U[d] += c * cr[d]
        q = np.zeros((4, ni, nj, nk), order="F")
        q[1], q[2], q[3] = U[0], U[1], U[2]
        h = [1.0 / (ni - 1), 1.0 / (nj - 1), 1.0 / (nk - 1)]
        out.append(Instance(Grid(ni, nj, nk), _fortran(X), _fortran(Y), _fortran(Z), _fortran(phi), q,
                            1.5 * max(h), 0.5 * min(h), cfl))
    return out


CASES = {"sphere_deformation": sphere_deformation, "solitary_wave": solitary_wave,
         "large_free_surface": large_free_surface}
