"""The plain FP64 path on the two FP64 benchmark configurations, at their
stated sizes and step counts, against the CPU oracle (OpenMP build: the same
per-node arithmetic as the serial checker, the volume sums sequential).

  * sphere in the LeVeque deformation field: 64^3 Cartesian nodes on the
    unit box, velocity cos(pi t / 3)-modulated and re-evaluated every step
    (t = (n - 1) dt, frozen over a step as the reference freezes q over a
    levelsetmethod call), CFL 0.5 (dt = 0.5 h / max|u|), 100 steps, 5
    reinitialisation pseudo-steps per step, eps = 1.5 h, 6-cell band;
  * solitary wave on the stretched curvilinear grid: 256 x 128 x 96 nodes,
    phi0 redistanced by 50 pseudo-steps, CFL 0.4, 200 steps, 10 pseudo-steps
    per step.

Each run goes through lsm_levelsetmethod (src/levelsetmethod.F90:1-372)
from the same inputs as the oracle, the GPU and the oracle each advancing
their own phi.  The bar, normwise relative (max|gpu - ref| / max|ref|):
phi <= 1e-12 after the final step (and at the checkpoints on the way).
Volumes: the per-cell volumes are bit-exact (test_gpu_parity.py), so the
sums differ only by summation order.  The reference adds the cells one after
another (src/TotalWaterVolume.F90:70-84), whose own rounding error grows
with the cell count (up to n u of the total, u = 2^-53: 3.5e-10 for the
3.1 M cells of the solitary-wave grid, where it reaches 5e-12 after one
step); the GPU sums a fixed-order tree.  So at every step the pre-advection
volumes agree within n u, and at the checkpoints the GPU's total is within
1e-12 of the exactly rounded sum (math.fsum) of the oracle's per-cell
volumes of the same phi.  After the final step the narrow band
(src/narrowband.F90:2-19), the AdvectionNodes band
(src/TotalWaterVolume.F90:169-235) and the ghost-fluid list
(src/get_gfm_list.F90:6-141) of the GPU's phi equal the oracle's of its own
phi bit for bit, and so do the GPU's of the oracle's phi.
"""
import math
import os

import numpy as np
import pytest

import cases
import oracle as O
from test_gpu_parity import G, dev, host

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def oracle_omp():
    O.build()
    return O.Oracle(omp=True)


def _oparams(lp, **kw):
    """oracle Params from an nslsm LsmParams (same field names)."""
    d = {}
    for name, _ in O.Params._fields_:
        v = getattr(lp, name)
        d[name] = tuple(v) if name == "btype_lsm" else (int(v) if isinstance(v, bool) else v)
    d.update(kw)
    return O.make_params(**d)


def _cfl_dt(csi, eta, zet, q, cfl):
    u = q[1:4]
    s = max(float(np.abs(m[0] * u[0] + m[1] * u[1] + m[2] * u[2]).max()) for m in (csi, eta, zet))
    return cfl / s


def _run(ls, orc, case, phi_gpu0, phi_ref0, p_lsm, p_orc, velocity, checkpoints):
    g = O.make_grid(*case.grid.shape)
    gg = G(g)
    csi, eta, zet, aj = orc.mg_metrics(g, case.x, case.y, case.z)
    dcsi, deta, dzet, daj = dev(csi), dev(eta), dev(zet), dev(aj)
    dx, dy, dz = dev(case.x), dev(case.y), dev(case.z)
    cur, ref = dev(phi_gpu0), np.asfortranarray(phi_ref0)
    ncell = (case.grid.ni - 1) * (case.grid.nj - 1) * (case.grid.nk - 1)
    vol_seq = ncell * 2.0 ** -53
    hist, vhist = [], []
    for it in range(1, case.steps + 1):
        q = velocity(it)
        before = ref
        ref, rv = orc.levelsetmethod(g, p_orc, q, csi, eta, zet, aj, ref, ref, case.x, case.y, case.z, it)
        v = ls.levelsetmethod(gg, p_lsm, dev(q), dcsi, deta, dzet, daj, cur, cur.clone(), dx, dy, dz, it)
        ev = cases.relerr(v, rv)
        assert ev <= vol_seq, (it, ev, vol_seq)
        if it in checkpoints or it == case.steps:
            exact = math.fsum(orc.cell_water_volumes(g, before, case.x, case.y, case.z).ravel())
            ee = abs(v[3] - exact) / abs(exact)
            vhist.append((it, ee, abs(rv[3] - exact) / abs(exact)))
            assert ee <= TOL, (it, ee)
            e = cases.relerr(host(cur), ref)
            hist.append((it, e))
            assert e <= TOL, (it, e, hist)
    print("%s: phi normwise error by step %s" % (case.name, ", ".join("%d: %.2e" % h for h in hist)))
    print("%s: total volume vs the exact sum of the oracle's cells (gpu, oracle's sequential sum) by step %s"
          % (case.name, ", ".join("%d: %.1e %.1e" % h for h in vhist)))
    return g, gg, host(cur), ref


def _bands_equal(ls, orc, g, gg, p_lsm, p_orc, got, ref, x, y, z):
    # each side on its own final phi, and the GPU on the oracle's phi
    for gpu_phi in (got, ref):
        nb = ls.narrowband(gg, p_lsm, dev(gpu_phi))
        assert np.array_equal(host(nb), orc.narrowband(g, p_orc, ref))
        _, adv = ls.total_water_volume(gg, dev(gpu_phi), dev(x), dev(y), dev(z), with_nodes=True)
        _, adv_ref = orc.total_water_volume(g, ref, x, y, z, with_nodes=True)
        assert np.array_equal(host(adv), adv_ref)
        lst = ls.get_gfm_list(gg, p_lsm, dev(gpu_phi))
        lst_ref = orc.get_gfm_list(g, p_orc, ref)
        assert lst.shape == lst_ref.shape and np.array_equal(lst, lst_ref)
    assert orc.narrowband(g, p_orc, ref).sum() > 0
    assert len(orc.get_gfm_list(g, p_orc, ref)) > 0


def test_sphere_deformation_64_cubed_100_steps(ls, oracle_omp):
    from nslsm import configs
    case = configs.sphere_deformation(64, 100, 5)
    g = O.make_grid(64, 64, 64)
    csi, eta, zet, _ = oracle_omp.mg_metrics(g, case.x, case.y, case.z)
    dt = _cfl_dt(csi, eta, zet, case.q(0.0), case.cfl)
    p_lsm = case.params.replace(delti_lsm=dt)
    p_orc = _oparams(p_lsm)

    def velocity(it):
        return case.q((it - 1) * dt)

    g, gg, got, ref = _run(ls, oracle_omp, case, case.phi0, case.phi0, p_lsm, p_orc, velocity, {1, 25, 50, 75})
    _bands_equal(ls, oracle_omp, g, gg, p_lsm, p_orc, got, ref, case.x, case.y, case.z)


@pytest.mark.skipif(os.environ.get("LSM_SKIP_LARGE") == "1", reason="LSM_SKIP_LARGE=1")
def test_solitary_wave_256x128x96_200_steps(ls, oracle_omp):
    from nslsm import configs
    case = configs.solitary_wave()
    g = O.make_grid(*case.grid.shape)
    csi, eta, zet, _ = oracle_omp.mg_metrics(g, case.x, case.y, case.z)
    q = case.q(0.0)
    dt = _cfl_dt(csi, eta, zet, q, case.cfl)
    p_lsm = case.params.replace(delti_lsm=dt)
    p_orc = _oparams(p_lsm)
    # redistancing before t = 0: 50 pseudo-steps of `reinitialization` and bcond_lsm on both sides
    pr_lsm = p_lsm.replace(RNitermax=case.redistance_iters)
    pr_orc = _oparams(pr_lsm)
    gg = G(g)
    r_gpu = ls.reinitialization(gg, pr_lsm, dev(case.phi0), dev(csi), dev(eta), dev(zet))
    ls.bcond_lsm(gg, pr_lsm, r_gpu)
    r_ref = oracle_omp.bcond_lsm(g, pr_orc, oracle_omp.reinitialization(g, pr_orc, case.phi0, csi, eta, zet))
    e0 = cases.relerr(host(r_gpu), r_ref)
    assert e0 <= TOL, e0
    g, gg, got, ref = _run(ls, oracle_omp, case, host(r_gpu), r_ref, p_lsm, p_orc, lambda it: q,
                           {1, 50, 100, 150})
    _bands_equal(ls, oracle_omp, g, gg, p_lsm, p_orc, got, ref, case.x, case.y, case.z)
