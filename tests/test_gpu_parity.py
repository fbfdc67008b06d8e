"""GPU parity of every level-set routine against the CPU FP64 oracle, called
through the C-ABI (liblsm_gb300.so).

Tolerances (FP64 path, built with --fmad=false in the reference's operation
order):
  * bit-exact: contravariant velocity, WENO3 / upwind RHS, RK3 stages, bcond,
    Godunov RHS, narrow band, AdvectionNodes, ghost-fluid list, per-cell
    volumes, metrics;
  * 1e-13 normwise relative where CUDA's sin/cos enter (smoothed sign,
    delta function, lambda, reinitialisation);
  * 1e-12 normwise relative for the volume sums (fixed-order tree vs the
    reference's sequential sum) and for phi after the full level-set step.
Normwise relative = max|gpu - ref| / max|ref|.
"""
import numpy as np
import pytest

import cases
import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TRIG = 1e-13
SUM = 1e-12


def dev(a):
    """numpy Fortran array -> CUDA tensor with the same bytes (reversed shape)."""
    a = np.asfortranarray(a)
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def host(t):
    return np.asfortranarray(t.cpu().numpy().T)


def G(g):
    from nslsm import Grid
    return Grid(g.iu - g.il + 1, g.ju - g.jl + 1, g.ku - g.kl + 1, g.igp, g.jgp, g.kgp,
                tuple(g.physical_face), g.dc, g.de, g.dz, g.il, g.jl, g.kl)


def P(op, **kw):
    from nslsm import LsmParams
    d = {}
    for name, _ in O.Params._fields_:
        v = getattr(op, name)
        d[name] = tuple(v) if name == "btype_lsm" else v
    d.update(kw)
    return LsmParams(**d)


@pytest.fixture(scope="module")
def setup(oracle):
    g, x, y, z, phi, q = cases.curvilinear(21, 13, 11, seed=11)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    h = 1.0 / 20
    p = O.make_params(epslsm=1.5 * h, RNtimestep=0.3 * h, RNitermax=6, delti_lsm=0.02, narrowcoef=4.0,
                      isnarrow=1, BigPhi=0.35)
    return dict(g=g, x=x, y=y, z=z, phi=phi, q=q, csi=csi, eta=eta, zet=zet, aj=aj, p=p)


@pytest.mark.parametrize("where", ["device", "host"])
def test_metrics_and_contra(ls, oracle, setup, where):
    s = setup
    gg = G(s["g"])
    conv = dev if where == "device" else (lambda a: a)
    back = host if where == "device" else (lambda a: a)
    csi, eta, zet, aj = (back(t) for t in ls.mg_metrics(gg, conv(s["x"]), conv(s["y"]), conv(s["z"])))
    for a, b in ((csi, s["csi"]), (eta, s["eta"]), (zet, s["zet"]), (aj, s["aj"])):
        assert np.array_equal(a, b)
    u = back(ls.rhs_contra_j(gg, conv(s["q"]), conv(s["csi"]), conv(s["eta"]), conv(s["zet"]), conv(s["aj"])))
    assert np.array_equal(u, oracle.rhs_contra_j(s["g"], s["q"], s["csi"], s["eta"], s["zet"], s["aj"]))


def test_rhs_weno3_upwind_bit_exact(ls, oracle, setup):
    s = setup
    gg = G(s["g"])
    ucn = oracle.rhs_contra_j(s["g"], s["q"], s["csi"], s["eta"], s["zet"], s["aj"])
    mask = np.ones(s["phi"].shape, dtype=np.int32, order="F")
    mask[5:9, 3:7, 2:5] = 0
    for m in (None, mask):
        r = host(ls.calc_rh_ad_weno3(gg, dev(s["phi"]), dev(ucn), None if m is None else dev(m)))
        assert np.array_equal(r, oracle.calc_rh_ad_weno3(s["g"], s["phi"], ucn, m))
        r = host(ls.calc_rh_ad(gg, dev(s["phi"]), dev(ucn), None if m is None else dev(m)))
        assert np.array_equal(r, oracle.calc_rh_ad(s["g"], s["phi"], ucn, m))


@pytest.mark.parametrize("orderAD,btype", [(1, (1, 1, 1, 1, 1, 1)), (1, (0, 2, 1, 0, 1, 1)),
                                           (0, (1, 2, 0, 1, 1, 0)), (0, (2, 2, 2, 2, 2, 2))])
def test_rk3_bit_exact(ls, oracle, setup, orderAD, btype):
    s = setup
    gg = G(s["g"])
    p = O.make_params(delti_lsm=0.02, orderAD=orderAD, btype_lsm=btype, BigPhi=0.35)
    ucn = oracle.rhs_contra_j(s["g"], s["q"], s["csi"], s["eta"], s["zet"], s["aj"])
    ref = oracle.ad_rktvd3(s["g"], p, s["phi"], ucn, s["aj"])
    out = host(ls.ad_rktvd3(gg, P(p), dev(s["phi"]), dev(ucn), dev(s["aj"])))
    assert np.array_equal(out, ref)
    mask = np.ones(s["phi"].shape, dtype=np.int32, order="F")
    mask[::3, 2:9, :] = 0
    ref = oracle.ad_rktvd3(s["g"], p, s["phi"], ucn, s["aj"], mask)
    out = host(ls.ad_rktvd3(gg, P(p), dev(s["phi"]), dev(ucn), dev(s["aj"]), dev(mask)))
    assert np.array_equal(out, ref)


@pytest.mark.parametrize("btype", [(1,) * 6, (0, 2, 1, 0, 0, 1), (2, 1, 2, 1, 2, 1)])
def test_bcond_bit_exact(ls, oracle, setup, btype):
    s = setup
    gg = G(s["g"])
    p = O.make_params(btype_lsm=btype, BigPhi=0.35)
    t = dev(s["phi"])
    ls.bcond_lsm(gg, P(p), t)
    assert np.array_equal(host(t), oracle.bcond_lsm(s["g"], p, s["phi"]))
    h = s["phi"].copy(order="F")
    ls.bcond_lsm(gg, P(p), h)                  # host arrays in place
    assert np.array_equal(h, oracle.bcond_lsm(s["g"], p, s["phi"]))


@pytest.mark.parametrize("M", [1, 0])
def test_sign_and_godunov(ls, oracle, setup, M):
    s = setup
    gg = G(s["g"])
    eps = s["p"].epslsm
    sg, ng = (host(t) for t in ls.calc_sign_ini(gg, dev(s["phi"]), dev(s["csi"]), dev(s["eta"]), dev(s["zet"]),
                                                 eps, M))
    rs, rn = oracle.calc_sign_ini(s["g"], s["phi"], s["csi"], s["eta"], s["zet"], eps, M)
    assert np.array_equal(ng, rn)
    assert cases.relerr(sg, rs) <= TRIG
    d = cases.F(s["phi"] * 1.2 + 0.01)
    r = host(ls.calc_rh_rn(gg, dev(d), dev(rs), dev(s["csi"]), dev(s["eta"]), dev(s["zet"])))
    assert np.array_equal(r, oracle.calc_rh_rn(s["g"], d, rs, s["csi"], s["eta"], s["zet"]))


def test_lambda_and_reinitialization(ls, oracle, setup):
    s = setup
    gg = G(s["g"])
    p = s["p"]
    rs, rn = oracle.calc_sign_ini(s["g"], s["phi"], s["csi"], s["eta"], s["zet"], p.epslsm, 1)
    d = cases.F(s["phi"] * 1.01)
    lam = host(ls.calc_lambda_rn(gg, P(p), dev(s["phi"]), dev(rn), dev(d), p.RNtimestep))
    assert cases.relerr(lam, oracle.calc_lambda_rn(s["g"], p, s["phi"], rn, d, p.RNtimestep)) <= TRIG
    out = host(ls.reinitialization(gg, P(p), dev(s["phi"]), dev(s["csi"]), dev(s["eta"]), dev(s["zet"])))
    assert cases.relerr(out, oracle.reinitialization(s["g"], p, s["phi"], s["csi"], s["eta"], s["zet"])) <= TRIG


def test_narrowband_gfm_band_bit_exact(ls, oracle, setup):
    s = setup
    gg = G(s["g"])
    p = s["p"]
    assert np.array_equal(host(ls.narrowband(gg, P(p), dev(s["phi"]))), oracle.narrowband(s["g"], p, s["phi"]))
    for bp in (0.35, 5.0):
        q = O.make_params(BigPhi=bp)
        lst = ls.get_gfm_list(gg, P(q), dev(s["phi"]))
        ref = oracle.get_gfm_list(s["g"], q, s["phi"])
        assert len(ref) > 0 and np.array_equal(lst, ref)
    v, adv = ls.total_water_volume(gg, dev(s["phi"]), dev(s["x"]), dev(s["y"]), dev(s["z"]), with_nodes=True)
    rv, radv = oracle.total_water_volume(s["g"], s["phi"], s["x"], s["y"], s["z"], with_nodes=True)
    assert np.array_equal(host(adv), radv)
    assert cases.relerr(v, rv) <= SUM
    cv = host(ls.cell_water_volumes(gg, dev(s["phi"]), dev(s["x"]), dev(s["y"]), dev(s["z"])))
    assert np.array_equal(cv, oracle.cell_water_volumes(s["g"], s["phi"], s["x"], s["y"], s["z"]))


def test_volume_edge_cases(ls, oracle):
    n = 9
    g, x, y, z, _, _ = cases.sphere(n)
    gg = G(g)
    for phi in (cases.F(z - 0.5), np.zeros((n, n, n), order="F"), np.full((n, n, n), -1.0, order="F"),
                np.ones((n, n, n), order="F")):
        cv = ls.cell_water_volumes(gg, phi, x, y, z)            # host arrays
        assert np.array_equal(cv, oracle.cell_water_volumes(g, phi, x, y, z))
        v = ls.total_water_volume(gg, phi, x, y, z)
        assert cases.relerr(v, oracle.total_water_volume(g, phi, x, y, z)) <= SUM or np.all(v == 0)


def test_ghosted_subdomain(ls, oracle):
    """A subdomain with two ghost planes on its non-physical faces (as one
    MPI rank of a decomposition sees it); ghosts hold the caller's values."""
    g, x, y, z, phi, q = cases.curvilinear(16, 14, 12, seed=5)
    og = O.make_grid(16, 14, 12, igp=2, jgp=2, kgp=0, physical=(1, 0, 0, 1, 1, 1))
    full = O.make_grid(16, 14, 12)
    csi, eta, zet, aj = oracle.mg_metrics(full, x, y, z)
    ucn = oracle.rhs_contra_j(og, q, csi, eta, zet, aj)
    gg = G(og)
    assert np.array_equal(host(ls.rhs_contra_j(gg, dev(q), dev(csi), dev(eta), dev(zet), dev(aj))), ucn)
    p = O.make_params(delti_lsm=0.01, BigPhi=5.0, epslsm=0.1, RNtimestep=0.02, RNitermax=3)
    assert np.array_equal(host(ls.calc_rh_ad_weno3(gg, dev(phi), dev(ucn))), oracle.calc_rh_ad_weno3(og, phi, ucn))
    assert np.array_equal(host(ls.ad_rktvd3(gg, P(p), dev(phi), dev(ucn), dev(aj))),
                          oracle.ad_rktvd3(og, p, phi, ucn, aj))
    out = host(ls.reinitialization(gg, P(p), dev(phi), dev(csi), dev(eta), dev(zet)))
    assert cases.relerr(out, oracle.reinitialization(og, p, phi, csi, eta, zet)) <= TRIG
    assert np.array_equal(ls.get_gfm_list(gg, P(p), dev(phi)), oracle.get_gfm_list(og, p, phi))
    v, adv = ls.total_water_volume(gg, dev(phi), dev(x), dev(y), dev(z), with_nodes=True)
    rv, radv = oracle.total_water_volume(og, phi, x, y, z, with_nodes=True)
    assert np.array_equal(host(adv), radv) and cases.relerr(v, rv) <= SUM


def test_exchange_callback_called_per_stage(ls, oracle, setup):
    s = setup
    gg = G(s["g"])
    calls = []
    ls.set_exchange_callback(lambda field, g: calls.append(field) or 0)
    try:
        ucn = oracle.rhs_contra_j(s["g"], s["q"], s["csi"], s["eta"], s["zet"], s["aj"])
        ls.ad_rktvd3(gg, P(s["p"]), dev(s["phi"]), dev(ucn), dev(s["aj"]))
        assert len(calls) == 3                       # after every RK stage (ad_RKTVD3.F90:84)
        calls.clear()
        ls.reinitialization(gg, P(s["p"]), dev(s["phi"]), dev(s["csi"]), dev(s["eta"]), dev(s["zet"]))
        assert len(calls) == 2 + s["p"].RNitermax    # sign, |grad phi0|, one per pseudo-step
    finally:
        ls.set_exchange_callback(None)
