"""The whole level-set step (lsm_levelsetmethod) on the GPU against the CPU
oracle and the committed golden fixtures, plus the error paths of the
C-ABI.  Parity bar: phi after the stated step count within 1e-12 normwise
relative of the oracle (the reference's FP64 arithmetic); volumes 1e-12."""
import json
import os

import numpy as np
import pytest

import cases
import oracle as O
from test_gpu_parity import G, P, dev, host

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
TOL = 1e-12
HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _run(ls, oracle, g, x, y, z, phi, q, p, nsteps, on_device):
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    gg, pp = G(g), P(p)
    ref = phi
    cur = dev(phi) if on_device else phi.copy(order="F")
    args = [dev(a) if on_device else a for a in (q, csi, eta, zet, aj, x, y, z)]
    for it in range(1, nsteps + 1):
        ref, rv = oracle.levelsetmethod(g, p, q, csi, eta, zet, aj, ref, ref, x, y, z, it)
        phin = cur.clone() if on_device else cur.copy(order="F")
        v = ls.levelsetmethod(gg, pp, args[0], args[1], args[2], args[3], args[4], cur, phin, args[5], args[6],
                              args[7], it)
        got = host(cur) if on_device else cur
        assert cases.relerr(got, ref) <= TOL, (it, cases.relerr(got, ref))
        assert cases.relerr(v, rv) <= TOL
    return ref


@pytest.mark.parametrize("on_device", [True, False])
def test_sphere_deformation_steps(ls, oracle, on_device):
    n = 24
    g, x, y, z, phi, q = cases.sphere(n)
    h = 1.0 / (n - 1)
    p = O.make_params(epslsm=1.5 * h, RNtimestep=0.5 * h, RNitermax=5, delti_lsm=0.25 * h, narrowcoef=4.0,
                      isnarrow=1)
    _run(ls, oracle, g, x, y, z, phi, q, p, 6, on_device)


def test_curvilinear_steps_upwind_and_numiter(ls, oracle):
    g, x, y, z, phi, q = cases.curvilinear(26, 15, 12, seed=2)
    h = 1.0 / 25
    p = O.make_params(epslsm=1.5 * h, RNtimestep=0.3 * h, RNitermax=10, delti_lsm=0.01, narrowcoef=4.0,
                      isnarrow=1, numiter_lsm=2, btype_lsm=(1, 2, 1, 0, 1, 1))
    _run(ls, oracle, g, x, y, z, phi, q, p, 3, True)
    pu = O.make_params(epslsm=1.5 * h, RNtimestep=0.3 * h, RNitermax=4, delti_lsm=0.01, orderAD=0, RNfreq=2)
    _run(ls, oracle, g, x, y, z, phi, q, pu, 3, True)


@pytest.mark.parametrize("kind", ["sphere", "curvilinear"])
def test_golden_steps(ls, kind):
    with open(os.path.join(HERE, "golden.json")) as f:
        meta = json.load(f)["steps_" + kind]
    fx = np.load(os.path.join(HERE, "steps_%s.npz" % kind))
    ni, nj, nk = meta["grid"]
    from nslsm import Grid, LsmParams
    gg = Grid(ni, nj, nk)
    p = LsmParams(**{k: (tuple(v) if k == "btype_lsm" else v) for k, v in meta["params"].items()})
    x, y, z, phi, q = (np.asfortranarray(fx[k]) for k in ("x", "y", "z", "phi0", "q"))
    csi, eta, zet, aj = ls.mg_metrics(gg, x, y, z)
    cur = dev(phi)
    for it in range(1, meta["steps"] + 1):
        v = ls.levelsetmethod(gg, p, dev(q), dev(csi), dev(eta), dev(zet), dev(aj), cur, cur.clone(), dev(x),
                              dev(y), dev(z), it)
        assert cases.relerr(host(cur), fx["phi_%d" % it]) <= TOL
        assert cases.relerr(v, fx["volumes_%d" % it]) <= TOL


def test_error_codes(ls):
    from nslsm import Grid, LsmError, LsmParams
    from nslsm import _lib
    n = 8
    g, x, y, z, phi, q = cases.sphere(n)
    gg = Grid(n, n, n)
    m3 = np.zeros((3, n, n, n), order="F")
    with pytest.raises(LsmError) as e:
        ls.levelsetmethod(gg, LsmParams(sussman_correction_method=1), q, m3, m3, m3, x, phi, phi, x, y, z, 1)
    assert e.value.status == _lib.LSM_ERR_UNSUPPORTED
    # the hybrid (geometric) branch runs on one subdomain without ghost planes
    with pytest.raises(LsmError) as e:
        ls.levelsetmethod(Grid(n, n, n, igp=2, physical=(0, 0, 1, 1, 1, 1)), LsmParams(hybrid_reinitialisation=True),
                          q, m3, m3, m3, x, phi, phi, x, y, z, 1)
    assert e.value.status == _lib.LSM_ERR_UNSUPPORTED
    with pytest.raises(LsmError) as e:
        ls.bcond_lsm(Grid(3, n, n), LsmParams(), np.zeros((3, n, n), order="F"))
    assert e.value.status == _lib.LSM_ERR_BAD_SHAPE
    with pytest.raises(LsmError) as e:
        ls.bcond_lsm(Grid(n, n, n, igp=1, physical=(0, 1, 1, 1, 1, 1)), LsmParams(), phi.copy(order="F"))
    assert e.value.status == _lib.LSM_ERR_BAD_SHAPE
    with pytest.raises(LsmError) as e:
        ls.calc_rh_ad_weno3(gg, dev(phi), np.zeros((3, n, n, n), order="F"))     # host + device mixed
    assert e.value.status == _lib.LSM_ERR_MIXED_MEMORY
    with pytest.raises(LsmError) as e:
        ls.bcond_lsm(gg, LsmParams(btype_lsm=(3, 1, 1, 1, 1, 1)), phi.copy(order="F"))
    assert e.value.status == _lib.LSM_ERR_BAD_PARAM
    # capacity: ask for the list with too small a buffer through the raw ABI
    import ctypes as C
    lib = _lib.load()
    cnt = C.c_int(0)
    small = np.zeros((1, 3), dtype=np.int32, order="F")
    gc, pc = gg.to_c(), LsmParams().to_c()
    st = lib.lsm_get_gfm_list(ls.h, C.byref(gc), C.byref(pc), phi.ctypes.data, C.byref(cnt), small.ctypes.data, 1)
    assert st == _lib.LSM_ERR_CAPACITY and cnt.value > 1
    # a NaN in phi propagates and is reported after the step
    bad = phi.copy(order="F")
    bad[4, 4, 4] = np.nan
    csi, eta, zet, aj = ls.mg_metrics(gg, x, y, z)
    with pytest.raises(LsmError) as e:
        ls.levelsetmethod(gg, LsmParams(epslsm=0.2, RNtimestep=0.05, RNitermax=2, delti_lsm=0.01), q, csi, eta,
                          zet, aj, bad, bad.copy(order="F"), x, y, z, 1)
    assert e.value.status == _lib.LSM_ERR_NONFINITE


def test_kernels_were_launched(ls):
    assert ls.launches > 0


def test_global_mass_correction_convergence_volume(ls, oracle):
    """GlobalMassCorrection (src/levelsetmethod.F90:245-264): the advected
    phi's K- and second-tetrahedra volumes, subtracted from the
    pre-advection total, against the oracle's volume of its advected phi;
    without the flag the convergence volume is the pre-advection total."""
    n = 20
    g, x, y, z, phi, q = cases.sphere(n)
    h = 1.0 / (n - 1)
    kw = dict(epslsm=1.5 * h, RNtimestep=0.5 * h, RNitermax=3, delti_lsm=0.25 * h, narrowcoef=4.0, isnarrow=1)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    # the oracle's advected phi: the same step without reinitialisation
    padv = O.make_params(call_reinitialisation=0, **kw)
    adv, rv = oracle.levelsetmethod(g, padv, q, csi, eta, zet, aj, phi, phi, x, y, z, 1)
    post = oracle.total_water_volume(g, adv, x, y, z)
    want = rv[3] - (post[0] + post[1])
    for gmc, expect in ((1, want), (0, rv[3])):
        p = O.make_params(GlobalMassCorrection=gmc, **kw)
        cur = dev(phi)
        v = ls.levelsetmethod(G(g), P(p), dev(q), dev(csi), dev(eta), dev(zet), dev(aj), cur, cur.clone(), dev(x),
                              dev(y), dev(z), 1)
        assert abs(v[3] - rv[3]) <= 1e-12 * abs(rv[3])
        assert abs(ls.convergence_volume() - expect) <= 1e-12 * abs(rv[3]), (gmc, ls.convergence_volume(), expect)
