"""Generate the committed golden fixtures of the level-set routines.

The reference (Fortran 90 + MPI) cannot be built in this image and ships no
tests or recorded outputs, so these fixtures come from the CPU FP64 oracle
(oracle/lsm_oracle.cpp) on seeded inputs.  They pin the oracle against
regressions and give the GPU tests a second, platform-independent
comparison point.  Inputs are stored in the fixture (not regenerated) so
that libm differences between machines cannot change them.

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "tests"))

import oracle as O  # noqa: E402
import cases  # noqa: E402


def params_dict(p):
    d = {}
    for name, _ in O.Params._fields_:
        v = getattr(p, name)
        d[name] = list(v) if name == "btype_lsm" else v
    return d


def routines(orc):
    g, x, y, z, phi, q = cases.curvilinear(14, 10, 8, seed=3)
    csi, eta, zet, aj = orc.mg_metrics(g, x, y, z)
    h = 1.0 / 13
    p = O.make_params(epslsm=1.5 * h, RNtimestep=0.3 * h, RNitermax=4, delti_lsm=0.02, narrowcoef=4.0,
                      isnarrow=1, BigPhi=0.3)
    ucn = orc.rhs_contra_j(g, q, csi, eta, zet, aj)
    out = dict(x=x, y=y, z=z, phi=phi, q=q)
    out["csi"], out["eta"], out["zet"], out["aj"] = csi, eta, zet, aj
    out["ucn"] = ucn
    out["rh_weno3"] = orc.calc_rh_ad_weno3(g, phi, ucn)
    out["rh_upwind"] = orc.calc_rh_ad(g, phi, ucn)
    out["rk3"] = orc.ad_rktvd3(g, p, phi, ucn, aj)
    pu = O.make_params(**{**params_dict(p), "orderAD": 0, "btype_lsm": (1, 2, 0, 1, 1, 0)})
    out["rk3_upwind_mixedbc"] = orc.ad_rktvd3(g, pu, phi, ucn, aj)
    out["bcond"] = orc.bcond_lsm(g, p, phi)
    out["sign"], out["ngrad"] = orc.calc_sign_ini(g, phi, csi, eta, zet, p.epslsm, 1)
    out["sign0"], out["ngrad0"] = orc.calc_sign_ini(g, phi, csi, eta, zet, p.epslsm, 0)
    out["rh_rn"] = orc.calc_rh_rn(g, phi * 1.3, out["sign"], csi, eta, zet)
    out["lambda"] = orc.calc_lambda_rn(g, p, phi, out["ngrad"], phi * 1.01, p.RNtimestep)
    out["reinit"] = orc.reinitialization(g, p, phi, csi, eta, zet)
    out["narrowband"] = orc.narrowband(g, p, phi)
    out["gfm_list"] = orc.get_gfm_list(g, p, phi)
    v, adv = orc.total_water_volume(g, phi, x, y, z, with_nodes=True)
    out["volumes"], out["adv_nodes"] = v, adv
    out["cellvol"] = orc.cell_water_volumes(g, phi, x, y, z)
    return out, {"grid": [14, 10, 8], "params": params_dict(p), "params_upwind": params_dict(pu)}


def steps(orc, kind):
    if kind == "sphere":
        n = 12
        g, x, y, z, phi, q = cases.sphere(n)
        h = 1.0 / (n - 1)
        p = O.make_params(epslsm=1.5 * h, RNtimestep=0.5 * h, RNitermax=5, delti_lsm=0.25 * h, narrowcoef=4.0,
                          isnarrow=1)
        nsteps = 3
    else:
        g, x, y, z, phi, q = cases.curvilinear(16, 10, 9, seed=7)
        h = 1.0 / 15
        p = O.make_params(epslsm=1.5 * h, RNtimestep=0.3 * h, RNitermax=10, delti_lsm=0.03, narrowcoef=4.0,
                          isnarrow=1)
        nsteps = 2
    csi, eta, zet, aj = orc.mg_metrics(g, x, y, z)
    out = dict(x=x, y=y, z=z, phi0=phi, q=q)
    cur = phi
    for it in range(1, nsteps + 1):
        cur, v = orc.levelsetmethod(g, p, q, csi, eta, zet, aj, cur, cur, x, y, z, it)
        out["phi_%d" % it] = cur
        out["volumes_%d" % it] = v
    return out, {"grid": [g.iu, g.ju, g.ku], "params": params_dict(p), "steps": nsteps}


def main():
    O.build()
    orc = O.Oracle()
    meta = {}
    arrs, meta["routines"] = routines(orc)
    np.savez_compressed(os.path.join(HERE, "routines.npz"), **arrs)
    for kind in ("sphere", "curvilinear"):
        arrs, meta["steps_" + kind] = steps(orc, kind)
        np.savez_compressed(os.path.join(HERE, "steps_%s.npz" % kind), **arrs)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("written", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
