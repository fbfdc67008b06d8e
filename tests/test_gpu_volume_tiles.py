"""The batch's water-volume scan on shapes that exercise its tiling: the scan
marches 32 x 8 cell columns over 32 planes, loads the i + 1 corners of a
tile's last lane itself, and a z tile may hold only the grid's last plane
(no cells).  The FP64 batch's volumes (K tetrahedra, second tetrahedra,
bulk, total) must equal the oracle's TotalWaterVolume of the same field:
every cell counted once (fixed-point rounding of each cell's share to
2^-48 bounds the difference far below the 1e-10 bar).  The FP32 batch
(phi rounded to FP32, the cells' relative vertex coordinates formed once
per geometry) must agree to 1e-6."""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

# (ni, nj, nk): partial tiles in x and z; one cell in a tile's last lane
# column (33); a last z tile holding only the final plane (nk = 33, 65);
# whole tiles (64) where the last lane's i + 1 corner is the grid's edge
SHAPES = [(70, 20, 70), (33, 9, 33), (64, 16, 65), (36, 17, 40)]


def _case(ni, nj, nk):
    from nslsm.configs import _mesh
    XI, ET, ZE = _mesh(ni, nj, nk)
    X, Y, Z = XI + 0.05 * ET, ET - 0.03 * ZE, ZE + 0.04 * XI
    F = lambda a: np.asfortranarray(a, dtype=np.float64)  # noqa: E731
    # a closed surface and a wavy sheet: interface cells in every tile row
    phi = np.minimum(Z - 0.45 - 0.06 * np.cos(2 * np.pi * (3 * X + Y)),
                     0.3 - np.sqrt((X - 0.5) ** 2 + (Y - 0.4) ** 2 + (Z - 0.7) ** 2))
    return F(X), F(Y), F(Z), F(phi)


def _batch_volumes(oracle, shapes, precision="fp64"):
    from nslsm.batch import LevelSetBatch
    cases = []
    for s in shapes:
        x, y, z, phi = _case(*s)
        csi, eta, zet, _ = oracle.mg_metrics(O.make_grid(*s), x, y, z)
        cases.append((s, x, y, z, phi, csi, eta, zet))
    b = LevelSetBatch([(*s, 1e-3, 1e-3, 1e-2) for s, *_ in cases], RNitermax=2, btype=(1,) * 6, BigPhi=5.0,
                      precision=precision, autotune=False)
    q = [np.zeros((4,) + s, order="F") for s, *_ in cases]
    for k, (s, x, y, z, phi, csi, eta, zet) in enumerate(cases):
        b.set_geometry(k, x, y, z, csi, eta, zet)
        b.set_velocity(k, q[k])
        b.set_phi(k, phi)
    v = b.water_volume()
    b.close()
    ref = [np.array(oracle.total_water_volume(O.make_grid(*s), phi, x, y, z)[:4])
           for s, x, y, z, phi, *_ in cases]
    return v, ref


@pytest.mark.parametrize("shape", SHAPES)
def test_scan_volume_equals_oracle_single_instance(oracle, lib_built, shape):
    v, ref = _batch_volumes(oracle, [shape])
    assert ref[0][3] > 0
    assert np.all(np.abs(v[0] - ref[0]) <= 1e-10 * ref[0][3]), (v[0], ref[0])


def test_scan_volume_equals_oracle_uneven_batch(oracle, lib_built):
    v, ref = _batch_volumes(oracle, SHAPES)
    for k in range(len(SHAPES)):
        assert np.all(np.abs(v[k] - ref[k]) <= 1e-10 * ref[k][3]), (k, v[k], ref[k])


def test_scan_volume_fp32_batch_within_fp32_rounding(oracle, lib_built):
    v, ref = _batch_volumes(oracle, SHAPES, "fp32")
    for k in range(len(SHAPES)):
        assert abs(v[k][3] - ref[k][3]) <= 1e-6 * ref[k][3], (k, v[k], ref[k])


def test_cell_coordinate_cache_changes_no_bit(oracle, lib_built):
    """FP32 batches keep each cell's relative vertex coordinates (a cache of
    the values the volume kernels would form per use).  With the cache
    switched off (LSM_BATCH_CELLREL=0, also what a batch that cannot fit it
    does) the mass-corrected steps, their volumes and the gradients through
    the correction's reverse are bit-identical."""
    import os
    from nslsm.batch import LevelSetBatch

    def run():
        cases = []
        for s in SHAPES[:2]:
            x, y, z, phi = _case(*s)
            csi, eta, zet, _ = oracle.mg_metrics(O.make_grid(*s), x, y, z)
            cases.append((s, x, y, z, phi, csi, eta, zet))
        b = LevelSetBatch([(*s, 2e-3, 5e-3, 2e-2) for s, *_ in cases], RNitermax=2, btype=(1,) * 6, BigPhi=5.0,
                          mass_correction=True, autotune=False)
        for k, (s, x, y, z, phi, csi, eta, zet) in enumerate(cases):
            q = np.zeros((4,) + s, order="F")
            q[1], q[3] = 0.3, 0.1 * np.sin(2 * np.pi * x)
            b.set_geometry(k, x, y, z, csi, eta, zet)
            b.set_velocity(k, q)
            b.set_phi(k, phi)
        v0 = b.water_volume()
        for k in range(len(cases)):
            b.set_mass_target(k, 1.001 * v0[k, 3])
        b.forward_record(3, 2)
        out = [b.water_volume()] + [b.get_phi(k) for k in range(len(cases))]
        for k, (s, *_rest) in enumerate(cases):
            b.set_grad_phi(k, np.asfortranarray(np.random.default_rng(k).standard_normal(s)))
        b.backward()
        out += [b.get_grad_phi0(k) for k in range(len(cases))]
        b.close()
        return out

    with_cache = run()
    os.environ["LSM_BATCH_CELLREL"] = "0"
    try:
        without = run()
    finally:
        del os.environ["LSM_BATCH_CELLREL"]
    for a, c in zip(with_cache, without):
        assert np.array_equal(a, c)
