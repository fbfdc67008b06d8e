"""The RK stage with its plane tiles staged by TMA copies (k_stage_tma:
cp.async.bulk.tensor into shared memory, completion on an mbarrier) against
the stage staged by the threads (k_stage_z): the same arithmetic on the same
values, so the steps must agree bit for bit.  Grids with partial tiles in
every direction (the copy engine zero-fills the box outside the grid) and
the recorded steps of the adjoint (stage inputs in the adjoint arena, a
second tensor map) are covered.  LSM_BATCH_STAGE forces the kernel."""
import os

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _case(ni, nj, nk):
    """Sheared unit box with a wavy free surface and a smooth velocity."""
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


def _run(oracle, ni, nj, nk, mode, steps=4, record=False):
    from nslsm.batch import LevelSetBatch
    x, y, z, phi, q = _case(ni, nj, nk)
    g = O.make_grid(ni, nj, nk)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    u = q[1:4]
    smax = max(float(np.abs(m[0] * u[0] + m[1] * u[1] + m[2] * u[2]).max()) for m in (csi, eta, zet))
    h = 1.0 / (min(ni, nj, nk) - 1)
    os.environ["LSM_BATCH_STAGE"] = mode
    try:
        b = LevelSetBatch([(ni, nj, nk, 0.4 / smax, 0.5 * h, 1.5 * h)], RNitermax=3, btype=(1,) * 6, BigPhi=5.0,
                          autotune=False)
        b.set_geometry(0, x, y, z, csi, eta, zet)
        b.set_velocity(0, q)
        b.set_phi(0, phi)
        if record:
            b.forward_record(steps, 2)
            w = np.asfortranarray(np.random.default_rng(1).standard_normal((ni, nj, nk)))
            b.set_grad_phi(0, w)
            b.backward()
            out = (b.get_phi(0), b.get_grad_phi0(0), b.get_grad_velocity(0))
        else:
            b.step(steps)
            out = (b.get_phi(0),)
        kernel = b.stage_kernel
        b.close()
    finally:
        del os.environ["LSM_BATCH_STAGE"]
    return out, kernel


@pytest.mark.parametrize("shape", [(64, 24, 20), (96, 37, 45), (36, 9, 70)])
def test_tma_stage_equals_thread_staged_stage(oracle, lib_built, shape):
    (a,), ka = _run(oracle, *shape, "tma")
    (b,), kb = _run(oracle, *shape, "smem")
    assert ka == "tma" and kb == "smem"
    assert np.array_equal(a, b), float(np.abs(a - b).max())


def test_tma_stage_in_recorded_steps_and_adjoint(oracle, lib_built):
    a, ka = _run(oracle, 64, 20, 33, "tma", steps=5, record=True)
    b, kb = _run(oracle, 64, 20, 33, "smem", steps=5, record=True)
    assert ka == "tma" and kb == "smem"
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def test_tma_not_used_where_rows_are_not_16_byte_units(oracle, lib_built):
    (_,), k = _run(oracle, 30, 20, 18, "tma", steps=1)
    assert k == "smem"
