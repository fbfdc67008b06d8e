"""Batched FP32 level-set path (include/lsm_batch.h) against the FP64 oracle.

Each instance of a small uneven batch runs the reference's level-set step
(WENO3-RK3 + bcond + `reinitialization` + water volume) in FP32 inside one
launch per pass; every instance is compared with the CPU FP64 oracle run on
its own.  Bars: L-infinity phi error within the
6-cell narrow band |phi| < 4 eps <= 1e-5, relative volume error <= 1e-6.
Tile shapes, brick or marching pseudo-steps and graph/no-graph must give
bit-identical phi.
"""
import numpy as np
import pytest

import cases
import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
BAND_TOL = 1e-5
VOL_TOL = 1e-6


@pytest.fixture(scope="module")
def small_batch(oracle, lib_built):
    from nslsm import configs
    insts = configs.batched_instances(n_inst=4, lo=12, hi=22, seed=3, cfl=0.5)
    prepared = []
    for it in insts:
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = oracle.mg_metrics(g, it.x, it.y, it.z)
        dt = it.time_step(csi, eta, zet)
        prepared.append(dict(inst=it, g=g, csi=csi, eta=eta, zet=zet, aj=aj, dt=dt))
    return prepared


def _make_batch(prep, R, **kw):
    from nslsm.batch import LevelSetBatch
    b = LevelSetBatch([(*p["inst"].grid.shape, p["dt"], p["inst"].dtau, p["inst"].eps) for p in prep],
                      RNitermax=R, btype=(1,) * 6, BigPhi=5.0, **kw)
    for k, p in enumerate(prep):
        it = p["inst"]
        b.set_geometry(k, it.x, it.y, it.z, p["csi"], p["eta"], p["zet"])
        b.set_velocity(k, it.q)
        b.set_phi(k, it.phi0)
    return b


def _oracle_run(oracle, p, R, nsteps):
    it = p["inst"]
    op = O.make_params(epslsm=it.eps, delti_lsm=p["dt"], RNitermax=R, RNtimestep=it.dtau, BigPhi=5.0)
    phi = it.phi0
    v = None
    for s in range(1, nsteps + 1):
        phi, v = oracle.levelsetmethod(p["g"], op, it.q, p["csi"], p["eta"], p["zet"], p["aj"], phi, phi, it.x,
                                       it.y, it.z, s)
    return phi, v


@pytest.mark.parametrize("R", [5, 0])
def test_batch_matches_fp64_oracle(oracle, small_batch, R):
    nsteps = 4
    b = _make_batch(small_batch, R)
    vols = b.step(nsteps)
    for k, p in enumerate(small_batch):
        ref, rv = _oracle_run(oracle, p, R, nsteps)
        got = b.get_phi(k)
        band = np.abs(ref) < 4.0 * p["inst"].eps
        assert band.any()
        err = float(np.abs(got - ref)[band].max())
        assert err <= BAND_TOL, (k, err)
        assert float(np.abs(got - ref).max()) <= 1e-4
        assert abs(vols[k, 3] - rv[3]) / rv[3] <= VOL_TOL, (k, vols[k], rv)
    b.close()


def test_shapes_and_graph_bit_identical(small_batch):
    outs = []
    # shape 5: the pseudo-steps march in k instead of walking the brick table
    for kw in (dict(autotune=False, shape=0, use_graph=True), dict(autotune=False, shape=3, use_graph=False),
               dict(autotune=False, shape=5, use_graph=True), dict(autotune=False, shape=5, use_graph=False),
               dict(autotune=True, use_graph=True)):
        b = _make_batch(small_batch, 3, **kw)
        b.step(3)
        outs.append([b.get_phi(k) for k in range(len(small_batch))])
        b.close()
    for o in outs[1:]:
        for a, c in zip(outs[0], o):
            assert np.array_equal(a, c)


def test_batch_device_arrays_and_launch_count(small_batch):
    from nslsm import _lib
    b = _make_batch(small_batch, 2)
    lib = _lib.load()
    b.step(0)                   # tunes the tile shape and captures the graph
    n0 = lib.lsm_kernel_launch_count(None)
    b.step(2)
    assert lib.lsm_kernel_launch_count(None) - n0 == 2 * b.launches_per_step
    dev = torch.zeros(small_batch[0]["inst"].grid.shape[::-1], dtype=torch.float64, device="cuda")
    got = b.get_phi(0, like=dev)
    assert np.array_equal(np.asfortranarray(got.cpu().numpy().T), b.get_phi(0))
    assert b.nodes == sum(p["inst"].grid.n for p in small_batch)
    b.close()


def test_tiny_ragged_instances(oracle):
    """Instances of 4..9 nodes per axis (every tile partial in x and z, most
    in y): brick and k-marching pseudo-steps agree bit for bit and match the
    FP64 oracle in the band."""
    from nslsm import configs
    prep = []
    for it in configs.batched_instances(n_inst=5, lo=4, hi=9, seed=5, cfl=0.5):
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = oracle.mg_metrics(g, it.x, it.y, it.z)
        prep.append(dict(inst=it, g=g, csi=csi, eta=eta, zet=zet, aj=aj, dt=it.time_step(csi, eta, zet)))
    R, nsteps = 3, 3
    outs = []
    for shape in (0, 5):
        b = _make_batch(prep, R, autotune=False, shape=shape)
        vols = b.step(nsteps)
        outs.append([b.get_phi(k) for k in range(len(prep))])
        b.close()
    for a, c in zip(*outs):
        assert np.array_equal(a, c)
    for k, p in enumerate(prep):
        ref, rv = _oracle_run(oracle, p, R, nsteps)
        got = outs[1][k]
        band = np.abs(ref) < 4.0 * p["inst"].eps
        if band.any():
            assert float(np.abs(got - ref)[band].max()) <= BAND_TOL
        assert float(np.abs(got - ref).max()) <= 1e-4
        assert abs(vols[k, 3] - rv[3]) / rv[3] <= VOL_TOL


@pytest.mark.parametrize("kind", ["pageable", "pinned", "device"])
def test_batch_wide_transfers_equal_per_instance_calls(small_batch, kind):
    """lsm_batch_set_velocities / lsm_batch_get_phis (every instance in one
    call, one wait) load and return the same bits as the per-instance calls,
    for each kind of caller array."""
    def arr(a):
        a = np.asfortranarray(a)
        if kind == "pageable":
            return a, None
        if kind == "pinned":
            t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
            v = t.numpy().reshape(a.shape, order="F")
            v[...] = a
            return v, t
        return torch.from_numpy(np.ascontiguousarray(a.T)).cuda(), None

    def host(a):
        return a.cpu().numpy().T.copy(order="F") if torch.is_tensor(a) else np.array(a, order="F")

    keep = []
    qs = []
    for p in small_batch:
        q = p["inst"].q.copy(order="F")
        q[1:] *= 0.9                      # a velocity other than the one the batch was built with
        v, t = arr(q)
        qs.append(v)
        keep.append(t)
    outs = []
    for p in small_batch:
        v, t = arr(np.zeros(p["inst"].grid.shape, order="F"))
        outs.append(v)
        keep.append(t)
    a = _make_batch(small_batch, 3)
    for k, q in enumerate(qs):
        a.set_velocity(k, q)
    a.step(2)
    ref = [a.get_phi(k) for k in range(len(small_batch))]
    a.close()
    b = _make_batch(small_batch, 3)
    b.set_velocities(qs)
    b.step(2)
    b.get_phis(outs)
    torch.cuda.synchronize()
    b.close()
    for r, o in zip(ref, outs):
        assert np.array_equal(host(o), r)
    del keep
