"""Known-answer tests of the CPU oracle (no GPU).

The reference has no tests or recorded outputs, so the oracle is pinned by
analytic answers the reference's formulas must give: WENO3 and upwind are
exact on linear data, marching tetrahedra are exact for planar interfaces,
the sphere volume converges at second order, bcond_lsm's extrapolation
weights, Cartesian metrics, the narrow-band literal, hand-built ghost-fluid
and band patterns, and |grad phi| -> 1 under reinitialisation.
"""
import math

import numpy as np
import pytest

import cases
import oracle as O


def _cart(n):
    g, x, y, z, phi, q = cases.sphere(n)
    return g, x, y, z, phi, q


def test_cartesian_metrics(oracle):
    n = 9
    g, x, y, z, _, _ = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    h = 1.0 / (n - 1)
    assert np.allclose(csi[0], 1 / h) and np.allclose(csi[1:], 0)
    assert np.allclose(eta[1], 1 / h) and np.allclose(zet[2], 1 / h)
    assert np.allclose(aj, 1 / h ** 3)


def test_weno3_and_upwind_exact_on_linear_data(oracle):
    n = 11
    g, x, y, z, _, _ = _cart(n)
    h = 1.0 / (n - 1)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    phi = cases.F(0.3 * x + 0.1 * y - 0.2 * z)
    q = np.zeros((4, n, n, n), order="F")
    q[1], q[2], q[3] = 1.0, -0.5, 0.25
    u = oracle.rhs_contra_j(g, q, csi, eta, zet, aj)
    assert np.allclose(u[0], h * h * 1.0) and np.allclose(u[1], -0.5 * h * h)
    expect = h * h * h * (0.3 * 1.0 - 0.1 * 0.5 - 0.2 * 0.25)
    rh = oracle.calc_rh_ad_weno3(g, phi, u)
    inner = rh[1:-1, 1:-1, 1:-1]
    assert np.allclose(inner, expect, rtol=1e-12, atol=0)
    assert np.all(rh[0] == 0) and np.all(rh[:, -1] == 0)     # boundary nodes untouched
    rhu = oracle.calc_rh_ad(g, phi, u)
    assert np.allclose(rhu, expect, rtol=1e-12, atol=0)      # one-sided faces are exact too


def test_weno3_mask_skips_nodes(oracle):
    n = 9
    g, x, y, z, phi, q = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    u = oracle.rhs_contra_j(g, q, csi, eta, zet, aj)
    mask = np.ones((n, n, n), dtype=np.int32, order="F")
    mask[3:6, 2:5, 4] = 0
    rh = oracle.calc_rh_ad_weno3(g, phi, u, mask)
    full = oracle.calc_rh_ad_weno3(g, phi, u)
    assert np.all(rh[mask == 0] == 0)
    assert np.array_equal(rh[mask == 1], full[mask == 1])


@pytest.mark.parametrize("surface,expect", [(lambda x, y: 0.4 + 0.2 * x, 0.5),
                                            (lambda x, y: 0.5 + 0 * x, 0.5),
                                            (lambda x, y: 0.3 + 0.1 * x + 0.2 * y, 0.55)])
def test_planar_interface_volume_exact(oracle, surface, expect):
    n = 13
    g, x, y, z, _, _ = _cart(n)
    phi = cases.F(z - surface(x, y))   # water (phi > 0) above the plane
    v = oracle.total_water_volume(g, phi, x, y, z)
    assert v[3] == pytest.approx(expect, rel=1e-13)
    assert v[3] == v[0] + v[1] + v[2]


def test_all_water_box_and_curvilinear_bulk(oracle):
    g, x, y, z, _, _ = cases.curvilinear(12, 9, 7, seed=1)
    one = np.ones(x.shape, order="F")
    v = oracle.total_water_volume(g, one, x, y, z)
    assert v[0] == 0 and v[1] == 0 and v[2] > 0
    # all-water: the cell volumes sum to the volume bounded by the grid (shoelace check on a slab)
    cv = oracle.cell_water_volumes(g, one, x, y, z)
    assert cv.sum() == pytest.approx(v[3], rel=1e-13)


def test_sphere_volume_second_order(oracle):
    exact = 4.0 / 3.0 * math.pi * 0.15 ** 3
    errs = []
    for n in (17, 33, 65):
        g, x, y, z, phi, _ = _cart(n)
        errs.append(abs(oracle.total_water_volume(g, phi, x, y, z)[3] - exact) / exact)
    assert errs[2] < 0.01
    assert errs[0] / errs[1] > 3.0 and errs[1] / errs[2] > 3.0


def test_zero_vertex_cases(oracle):
    # phi exactly zero on nodes exercises the MarchingTetrahedron special cases
    n = 9
    g, x, y, z, _, _ = _cart(n)
    phi = cases.F(z - 0.5)          # nodes at z = 0.5 are exactly zero
    v = oracle.total_water_volume(g, phi, x, y, z)
    assert v[3] == pytest.approx(0.5, rel=1e-13)
    zero = np.zeros(x.shape, order="F")   # four zero vertices: full tetrahedra
    v0 = oracle.total_water_volume(g, zero, x, y, z)
    assert v0[0] == pytest.approx(1.0, rel=1e-13)


def test_bcond_weights_and_bigphi(oracle):
    n = 8
    g, _, _, _, _, _ = _cart(n)
    rng = np.random.default_rng(0)
    f = cases.F(rng.uniform(-1, 1, (n, n, n)))
    p = O.make_params(BigPhi=5.0)
    b = oracle.bcond_lsm(g, p, f)
    assert b[0, 3, 4] == 4.0 / 3.0 * f[1, 3, 4] + (-1.0 / 3.0) * f[2, 3, 4]
    f2 = f.copy(order="F")
    f2[2, 3, 4] = 7.0                     # |phi(3)| >= BigPhi -> first order
    b2 = oracle.bcond_lsm(g, p, f2)
    assert b2[0, 3, 4] == f2[1, 3, 4]
    p0 = O.make_params(btype_lsm=(0, 2, 1, 1, 1, 1))
    b3 = oracle.bcond_lsm(g, p0, f)
    assert b3[0, 3, 4] == f[1, 3, 4]                       # absorption copies
    assert b3[-1, 3, 4] == 2.0 * f[-2, 3, 4] - 1.0 * f[-3, 3, 4]   # type 2 on the im face
    # corner: k faces come last and read the j-face values
    jface = 4.0 / 3.0 * b[0, 1, 0 + 1] - 1.0 / 3.0 * b[0, 2, 1]
    assert np.isfinite(jface)


def test_narrowband_single_precision_literal(oracle):
    n = 6
    g, _, _, _, _, _ = _cart(n)
    tol = float(np.float32(1.0e-5))
    assert tol == 9.999999747378752e-06
    thr = 4.0 * 0.1 + tol
    phi = np.full((n, n, n), 1.0, order="F")
    phi[1, 1, 1] = np.nextafter(thr, 0.0)
    phi[2, 2, 2] = np.nextafter(thr, 1.0)
    phi[3, 3, 3] = -np.nextafter(thr, 0.0)
    nb = oracle.narrowband(g, O.make_params(epslsm=0.1, narrowcoef=4.0, isnarrow=1), phi)
    assert nb[1, 1, 1] == 1 and nb[2, 2, 2] == 0 and nb[3, 3, 3] == 1 and nb.sum() == 2
    assert oracle.narrowband(g, O.make_params(isnarrow=0), phi).sum() == n ** 3


def test_gfm_list_single_water_node(oracle):
    n = 8
    g, _, _, _, _, _ = _cart(n)
    phi = np.full((n, n, n), -0.5, order="F")
    phi[3, 4, 2] = 0.5                    # Fortran node (4, 5, 3)
    lst = oracle.get_gfm_list(g, O.make_params(BigPhi=5.0), phi)
    expect = [(i, j, k) for k in (2, 3, 4) for j in (4, 5, 6) for i in (3, 4, 5) if (i, j, k) != (4, 5, 3)]
    assert [tuple(r) for r in lst] == expect
    assert len(oracle.get_gfm_list(g, O.make_params(BigPhi=0.4), phi)) == 0   # |phi| > BigPhi


def test_advection_nodes_dilation(oracle):
    n = 9
    g, x, y, z, _, _ = _cart(n)
    phi = np.full((n, n, n), 1.0, order="F")
    phi[4, 4, 4] = -1.0
    _, adv = oracle.total_water_volume(g, phi, x, y, z, with_nodes=True)
    # every base node within 1 of the negative node changes sign -> its 3x3x3 box
    expect = np.zeros_like(adv)
    expect[2:7, 2:7, 2:7] = 1
    assert np.array_equal(adv, expect)


def test_reinit_drives_gradient_to_one(oracle):
    n = 33
    g, x, y, z, phi, _ = _cart(n)
    h = 1.0 / (n - 1)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    p = O.make_params(epslsm=1.5 * h, RNtimestep=0.5 * h, RNitermax=60)
    out = oracle.reinitialization(g, p, cases.F(2.0 * phi), csi, eta, zet)
    gn = np.sqrt(sum(a ** 2 for a in np.gradient(out, h)))
    band = np.abs(out) < 3 * h
    assert abs(np.median(gn[band]) - 1.0) < 0.15
    s, ng = oracle.calc_sign_ini(g, phi, csi, eta, zet, 1.5 * h, 1)
    assert np.all(np.abs(s) <= 1.0) and np.all(s[phi >= 1.5 * h] == 1.0)


def test_rk3_zero_velocity_keeps_interior(oracle):
    n = 9
    g, x, y, z, phi, _ = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    u = np.zeros((3, n, n, n), order="F")
    p = O.make_params(delti_lsm=0.01)
    out = oracle.ad_rktvd3(g, p, phi, u, aj)
    # (1/3) phi + (2/3) phi rounds within an ulp of phi
    assert np.allclose(out[1:-1, 1:-1, 1:-1], phi[1:-1, 1:-1, 1:-1], rtol=1e-15, atol=0)
    assert np.allclose(out, oracle.bcond_lsm(g, p, phi), rtol=1e-14, atol=1e-16)


def test_rk3_translation_accuracy(oracle):
    # a smooth profile advected by a uniform velocity matches the translated profile
    n = 33
    g, x, y, z, _, _ = _cart(n)
    h = 1.0 / (n - 1)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    phi = cases.F(np.sin(2 * np.pi * x) * 0.1)
    q = np.zeros((4, n, n, n), order="F")
    q[1] = 1.0
    u = oracle.rhs_contra_j(g, q, csi, eta, zet, aj)
    dt = 0.2 * h
    p = O.make_params(delti_lsm=dt)
    cur = phi
    for _ in range(10):
        cur = oracle.ad_rktvd3(g, p, cur, u, aj)
    exact = 0.1 * np.sin(2 * np.pi * (x - 10 * dt))
    assert np.abs(cur - exact)[4:-4].max() < 5e-3   # WENO3 clips the extrema slightly


# ---------------------------------------------------------------- live Sussman reinit
@pytest.mark.parametrize("order,enobc", [(1, 0), (2, 0), (2, 1), (3, 0)])
def test_normgrad_d_exact_on_linear_data(oracle, order, enobc):
    """ENO2 (interior), BiasedDerivative orders 1-3 and ENO2Boundary
    (physical faces, edges, corners) are exact on linear data."""
    n = 9
    g, x, y, z, _, _ = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    phi = cases.F(0.3 * x + 0.4 * y - 1.2 * z + 0.1)
    p = O.make_params(epslsm=0.2, OrderReinitialisationBoundaries=order, ENOBCReinitialisation=enobc)
    ng = oracle.calc_normgrad_d(g, p, phi, phi, csi, eta, zet)
    assert np.allclose(ng, math.sqrt(0.3 ** 2 + 0.4 ** 2 + 1.2 ** 2), rtol=1e-12, atol=0)


def test_normgrad_d_second_order_on_quadratic(oracle):
    """Interior ENO2 = central difference on a quadratic (exact); second- and
    third-order one-sided derivatives are exact on the faces too."""
    n = 9
    g, x, y, z, _, _ = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    phi = cases.F(x * x + 0.5)
    for order in (2, 3):
        p = O.make_params(epslsm=0.2, OrderReinitialisationBoundaries=order)
        ng = oracle.calc_normgrad_d(g, p, phi, phi, csi, eta, zet)
        assert np.allclose(ng, 2 * x, rtol=1e-11, atol=1e-12)


def test_reinitialisation_test2_exits_on_signed_distance(oracle):
    """A planar signed distance has |grad phi| = 1 at every node: the first
    convergence test exits before any pseudo-step and phi is unchanged."""
    n = 9
    g, x, y, z, _, _ = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    phi = cases.F(0.6 * x + 0.8 * z - 0.5)
    p = O.make_params(epslsm=0.2, RNitermax=10, RNtimestep=0.01, epsReinitialisation=1e-8)
    out, iters = oracle.reinitialisation_test2(g, p, phi, csi, eta, zet)
    assert iters == 0 and np.array_equal(out, phi)


def test_reinitialisation_test2_masks_nodes_below_one(oracle):
    """Only nodes whose |grad d| exceeds 1 + epsReinitialisation move
    (src/reinitialisation_test2.F90:146): a field with |grad phi| = 0.5
    everywhere is never updated, whatever the iteration count."""
    n = 9
    g, x, y, z, _, _ = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    phi = cases.F(0.5 * (y - 0.45))
    p = O.make_params(epslsm=0.2, RNitermax=5, RNtimestep=0.01, epsReinitialisation=1e-5)
    out, iters = oracle.reinitialisation_test2(g, p, phi, csi, eta, zet)
    assert iters == 5 and np.array_equal(out, phi)


def test_normgrad_d_i_faces_use_the_last_interior_phi0(oracle):
    """The two i-face blocks of calc_NormGrad_d never assign phi0, so their
    ENO2 stencil choice takes phizero of the last interior node: flipping
    phizero there (and only there) changes the i-face gradients of a field
    whose ENO2 choices differ by sign, and nothing else."""
    n = 9
    g, x, y, z, _, _ = _cart(n)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    d = cases.F(np.abs(y - 0.5) + 0.3 * (z - 0.5) ** 2)   # kink: ENO2 sides differ
    p = O.make_params(epslsm=0.2)
    pz = cases.F(np.ones_like(d))
    a = oracle.calc_normgrad_d(g, p, d, pz, csi, eta, zet)
    pz2 = cases.F(pz.copy())
    pz2[n - 2, n - 2, n - 2] = -1.0          # last node of the interior loop
    b = oracle.calc_normgrad_d(g, p, d, pz2, csi, eta, zet)
    diff = a != b
    iface = np.zeros_like(diff)
    iface[[0, n - 1], 1:n - 1, 1:n - 1] = True
    assert diff.any() and not (diff & ~iface & ~(np.indices(diff.shape) == n - 2).all(0)).any()
