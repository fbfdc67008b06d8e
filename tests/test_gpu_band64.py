"""The FP64 stage near the interface in the FP32 batch: stage nodes whose
input |phi| is below 2 eps take their contravariant velocity from the FP64
metrics and FP64 velocity (kept per node) and combine the stage in FP64
over the FP32 WENO differences.  LSM_BATCH_BAND64=0 leaves it out.

  * one step without reinitialisation: nodes that were at least 4 eps from
    the interface (so no stage input came within 2 eps) are bit-identical
    with and without it, and band nodes differ (it ran);
  * in the band the FP32 step stays within 1e-6 of the FP64 batch, and its
    error there is printed next to the run without the FP64 terms; after 20
    steps with reinitialisation both band errors are printed.
"""
import os

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _case(ni, nj, nk):
    from nslsm.configs import _mesh
    XI, ET, ZE = _mesh(ni, nj, nk)
    X, Y, Z = XI + 0.05 * ET, ET - 0.03 * ZE, ZE + 0.04 * XI
    phi = Z - 0.5 - 0.04 * np.cos(2 * np.pi * (2 * X + Y))
    q = np.zeros((4, ni, nj, nk), order="F")
    q[1] = 0.6 + 0.3 * np.sin(2 * np.pi * Y)
    q[2] = -0.4 * np.cos(2 * np.pi * X)
    q[3] = 0.2 * np.sin(2 * np.pi * X) * np.sin(np.pi * Z)
    F = lambda a: np.asfortranarray(a, dtype=np.float64)  # noqa: E731
    return F(X), F(Y), F(Z), F(phi), q


def _run(oracle, shape, R, steps, precision, band64):
    from nslsm.batch import LevelSetBatch
    ni, nj, nk = shape
    x, y, z, phi, q = _case(ni, nj, nk)
    g = O.make_grid(ni, nj, nk)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    u = q[1:4]
    smax = max(float(np.abs(m[0] * u[0] + m[1] * u[1] + m[2] * u[2]).max()) for m in (csi, eta, zet))
    h = 1.0 / (min(shape) - 1)
    if not band64:
        os.environ["LSM_BATCH_BAND64"] = "0"
    try:
        b = LevelSetBatch([(ni, nj, nk, 0.4 / smax, 0.5 * h, 1.5 * h)], RNitermax=R, btype=(1,) * 6, BigPhi=5.0,
                          precision=precision, autotune=False)
        b.set_geometry(0, x, y, z, csi, eta, zet)
        b.set_velocity(0, q)
        b.set_phi(0, phi)
        b.step(steps)
        out = b.get_phi(0)
        b.close()
    finally:
        os.environ.pop("LSM_BATCH_BAND64", None)
    return out, phi, 1.5 * h


def test_band_nodes_only_and_closer_to_fp64(oracle, lib_built):
    shape = (48, 40, 36)
    on, phi0, eps = _run(oracle, shape, 0, 1, "fp32", True)
    off, _, _ = _run(oracle, shape, 0, 1, "fp32", False)
    ref, _, _ = _run(oracle, shape, 0, 1, "fp64", True)
    far = np.abs(phi0) > 4 * eps
    band = np.abs(phi0) < eps
    assert np.array_equal(on[far], off[far])
    assert np.any(on[band] != off[band])
    e_on, e_off = float(np.abs(on - ref)[band].max()), float(np.abs(off - ref)[band].max())
    print("one step, band error vs FP64: with the FP64 stage %.2e, without %.2e" % (e_on, e_off))
    assert e_on <= 1e-6


def test_band_error_after_20_steps(oracle, lib_built):
    shape = (48, 40, 36)
    on, _, eps = _run(oracle, shape, 5, 20, "fp32", True)
    off, _, _ = _run(oracle, shape, 5, 20, "fp32", False)
    ref, _, _ = _run(oracle, shape, 5, 20, "fp64", True)
    band = np.abs(ref) < 4 * eps
    e_on, e_off = float(np.abs(on - ref)[band].max()), float(np.abs(off - ref)[band].max())
    print("20 steps, band error vs FP64: with the FP64 stage %.2e, without %.2e" % (e_on, e_off))
    assert e_on <= 1e-5
