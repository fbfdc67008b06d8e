"""GPU parity of the reference's live reinitialisation (reinitialisation_test2
with calc_NormGrad_d) against the CPU FP64 oracle, through the C-ABI.

  * calc_NormGrad_d: bit-exact (FP64, the reference's operation order), for
    boundary orders 1, 2, 3 and ENO2Boundary, on a full single-zone grid and
    on a ghosted subdomain; the i-face blocks' stale phi0 is reproduced;
  * reinitialisation_test2: same iteration count, phi within 1e-13 normwise
    relative (CUDA's sin/cos in the smoothed sign and the delta function);
  * levelsetmethod with reinit_scheme = 1 over three steps: 1e-12.
"""
import numpy as np
import pytest

import cases
import oracle as O
from test_gpu_parity import G, P, dev, host

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TRIG = 1e-13


@pytest.fixture(scope="module")
def sus(oracle):
    g, x, y, z, phi, q = cases.curvilinear(17, 12, 10, seed=21)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    return dict(g=g, x=x, y=y, z=z, phi=phi, q=q, csi=csi, eta=eta, zet=zet, aj=aj)


@pytest.mark.parametrize("order,enobc", [(1, 0), (2, 0), (2, 1), (3, 0)])
def test_normgrad_d_bit_exact(ls, oracle, sus, order, enobc):
    s = sus
    p = O.make_params(epslsm=0.08, OrderReinitialisationBoundaries=order, ENOBCReinitialisation=enobc)
    d = cases.F(s["phi"] + 0.02 * np.sin(7.0 * s["x"]))
    ref = oracle.calc_normgrad_d(s["g"], p, d, s["phi"], s["csi"], s["eta"], s["zet"])
    got = host(ls.calc_normgrad_d(G(s["g"]), P(p), dev(d), dev(s["phi"]), dev(s["csi"]), dev(s["eta"]),
                                  dev(s["zet"])))
    assert np.array_equal(got, ref)


def test_normgrad_d_ghosted_subdomain(ls, oracle):
    g, x, y, z, phi, q = cases.curvilinear(16, 14, 12, seed=5)
    og = O.make_grid(16, 14, 12, igp=2, jgp=2, kgp=0, physical=(1, 0, 0, 1, 1, 1))
    csi, eta, zet, aj = oracle.mg_metrics(O.make_grid(16, 14, 12), x, y, z)
    p = O.make_params(epslsm=0.1, OrderReinitialisationBoundaries=2)
    ref = oracle.calc_normgrad_d(og, p, phi, phi, csi, eta, zet)
    got = host(ls.calc_normgrad_d(G(og), P(p), dev(phi), dev(phi), dev(csi), dev(eta), dev(zet)))
    assert np.array_equal(got, ref)
    ref2, it2 = oracle.reinitialisation_test2(og, O.make_params(epslsm=0.1, RNitermax=4, RNtimestep=0.01,
                                                                epsReinitialisation=1e-5), phi, csi, eta, zet)
    got2, git2 = ls.reinitialisation_test2(G(og), P(O.make_params(epslsm=0.1, RNitermax=4, RNtimestep=0.01,
                                                                  epsReinitialisation=1e-5)),
                                           dev(phi), dev(csi), dev(eta), dev(zet))
    assert git2 == it2 and cases.relerr(host(got2), ref2) <= TRIG


def test_normgrad_d_stale_phi0_on_i_faces(ls, oracle):
    """Changing phizero at the last interior node changes the i-face values
    on the GPU exactly as in the oracle."""
    n = 9
    g, x, y, z, _, _ = cases.sphere(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    d = cases.F(np.abs(y - 0.5) + 0.3 * (z - 0.5) ** 2)
    pz = cases.F(np.ones_like(d))
    pz[n - 2, n - 2, n - 2] = -1.0
    p = O.make_params(epslsm=0.2)
    ref = oracle.calc_normgrad_d(g, p, d, pz, csi, eta, zet)
    got = host(ls.calc_normgrad_d(G(g), P(p), dev(d), dev(pz), dev(csi), dev(eta), dev(zet)))
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("order,enobc,epsr", [(1, 0, 1e-5), (2, 1, 1e-5), (3, 0, 0.3)])
def test_reinitialisation_test2(ls, oracle, sus, order, enobc, epsr):
    s = sus
    p = O.make_params(epslsm=0.08, RNitermax=8, RNtimestep=0.01, epsReinitialisation=epsr,
                      OrderReinitialisationBoundaries=order, ENOBCReinitialisation=enobc)
    ref, it = oracle.reinitialisation_test2(s["g"], p, s["phi"], s["csi"], s["eta"], s["zet"])
    got, git = ls.reinitialisation_test2(G(s["g"]), P(p), dev(s["phi"]), dev(s["csi"]), dev(s["eta"]),
                                         dev(s["zet"]))
    assert git == it
    assert cases.relerr(host(got), ref) <= TRIG


def test_levelsetmethod_with_live_reinitialisation(ls, oracle, sus):
    s = sus
    p = O.make_params(epslsm=0.08, RNitermax=5, RNtimestep=0.01, delti_lsm=0.01, epsReinitialisation=1e-5,
                      reinit_scheme=1, BigPhi=5.0)
    phi_ref = s["phi"].copy(order="F")
    phi_gpu = dev(s["phi"])
    for it in range(1, 4):
        phi_ref, vr = oracle.levelsetmethod(s["g"], p, s["q"], s["csi"], s["eta"], s["zet"], s["aj"], phi_ref,
                                            phi_ref, s["x"], s["y"], s["z"], it)
        phin = phi_gpu.clone()
        vg = ls.levelsetmethod(G(s["g"]), P(p), dev(s["q"]), dev(s["csi"]), dev(s["eta"]), dev(s["zet"]),
                               dev(s["aj"]), phi_gpu, phin, dev(s["x"]), dev(s["y"]), dev(s["z"]), it)
    assert cases.relerr(host(phi_gpu), phi_ref) <= 1e-12
