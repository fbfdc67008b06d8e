"""The oracle reproduces the committed golden fixtures (tests/golden, made by
tests/golden/make_golden.py).  Integer outputs must match exactly; FP64
outputs within 1e-13 relative (the fixtures may have been made on another
CPU, whose libm sin/cos can differ in the last bit)."""
import json
import os

import numpy as np
import pytest

import cases
import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-13


def _meta():
    with open(os.path.join(HERE, "golden.json")) as f:
        return json.load(f)


def _params(d):
    return O.make_params(**{k: (tuple(v) if k == "btype_lsm" else v) for k, v in d.items()})


def test_routines_fixture(oracle):
    meta = _meta()["routines"]
    f = np.load(os.path.join(HERE, "routines.npz"))
    ni, nj, nk = meta["grid"]
    g = O.make_grid(ni, nj, nk)
    p = _params(meta["params"])
    pu = _params(meta["params_upwind"])
    x, y, z, phi, q = (np.asfortranarray(f[k]) for k in ("x", "y", "z", "phi", "q"))
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    for k, v in (("csi", csi), ("eta", eta), ("zet", zet), ("aj", aj)):
        assert np.array_equal(v, f[k]), k
    ucn = oracle.rhs_contra_j(g, q, csi, eta, zet, aj)
    assert np.array_equal(ucn, f["ucn"])
    assert cases.relerr(oracle.calc_rh_ad_weno3(g, phi, ucn), f["rh_weno3"]) <= TOL
    assert cases.relerr(oracle.calc_rh_ad(g, phi, ucn), f["rh_upwind"]) <= TOL
    assert cases.relerr(oracle.ad_rktvd3(g, p, phi, ucn, aj), f["rk3"]) <= TOL
    assert cases.relerr(oracle.ad_rktvd3(g, pu, phi, ucn, aj), f["rk3_upwind_mixedbc"]) <= TOL
    assert cases.relerr(oracle.bcond_lsm(g, p, phi), f["bcond"]) <= TOL
    s, ng = oracle.calc_sign_ini(g, phi, csi, eta, zet, p.epslsm, 1)
    assert cases.relerr(s, f["sign"]) <= TOL and cases.relerr(ng, f["ngrad"]) <= TOL
    s0, ng0 = oracle.calc_sign_ini(g, phi, csi, eta, zet, p.epslsm, 0)
    assert cases.relerr(s0, f["sign0"]) <= TOL and cases.relerr(ng0, f["ngrad0"]) <= TOL
    assert cases.relerr(oracle.calc_rh_rn(g, phi * 1.3, f["sign"], csi, eta, zet), f["rh_rn"]) <= TOL
    assert cases.relerr(oracle.calc_lambda_rn(g, p, phi, f["ngrad"], phi * 1.01, p.RNtimestep), f["lambda"]) <= TOL
    assert cases.relerr(oracle.reinitialization(g, p, phi, csi, eta, zet), f["reinit"]) <= TOL
    assert np.array_equal(oracle.narrowband(g, p, phi), f["narrowband"])
    assert np.array_equal(oracle.get_gfm_list(g, p, phi), f["gfm_list"])
    v, adv = oracle.total_water_volume(g, phi, x, y, z, with_nodes=True)
    assert np.array_equal(adv, f["adv_nodes"])
    assert cases.relerr(v, f["volumes"]) <= TOL
    assert cases.relerr(oracle.cell_water_volumes(g, phi, x, y, z), f["cellvol"]) <= TOL


@pytest.mark.parametrize("kind", ["sphere", "curvilinear"])
def test_steps_fixture(oracle, kind):
    meta = _meta()["steps_" + kind]
    f = np.load(os.path.join(HERE, "steps_%s.npz" % kind))
    ni, nj, nk = meta["grid"]
    g = O.make_grid(ni, nj, nk)
    p = _params(meta["params"])
    x, y, z, phi, q = (np.asfortranarray(f[k]) for k in ("x", "y", "z", "phi0", "q"))
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    cur = phi
    for it in range(1, meta["steps"] + 1):
        cur, v = oracle.levelsetmethod(g, p, q, csi, eta, zet, aj, cur, cur, x, y, z, it)
        assert cases.relerr(cur, f["phi_%d" % it]) <= 1e-12
        assert cases.relerr(v, f["volumes_%d" % it]) <= 1e-12
