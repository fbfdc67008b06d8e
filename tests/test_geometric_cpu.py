"""The oracle's geometric reinitialisation (the hybrid path,
src/geometric_reinitialisation.F90), pinned on CPU by known answers:

1. an axis-aligned plane phi = 2 (z0 - z) comes back as the signed distance
   z0 - z on the pnodes and on the nodes tagged -1 (to rounding);
2. for a tilted plane the distances never fall below the exact ones and keep
   their sign (the reference's projection step weights the triangle's first
   and third vertices the other way round, so its in-triangle distance can
   only over-estimate; vertex and edge distances are exact);
3. the tags: pnodes are numbered 1.. in Fortran order, -1 marks exactly the
   other nodes within 4 nodes (per axis) of a pnode, every other node keeps
   the caller's value;
4. with GlobalMassCorrection and a reachable target (the K-tetrahedra water
   volume of the input), Newton converges and the corrected phi holds that
   volume;
5. the hybrid levelsetmethod runs, advects only the AdvectionNodes band and
   leaves nodes far from the interface at +-9.9.
"""
import numpy as np
import pytest

import cases
import oracle as O

EPS = np.finfo(np.float64).eps


def _box(n, z0=0.4371, tilt=None, scale=2.0):
    X, Y, Z = np.meshgrid(*(np.linspace(0, 1, n),) * 3, indexing="ij")
    if tilt is None:
        sd = z0 - Z
    else:
        nv = np.array(tilt, dtype=np.float64)
        nv /= np.linalg.norm(nv)
        sd = z0 - (nv[0] * (X - 0.5) + nv[1] * (Y - 0.5) + nv[2] * Z)
    phi = cases.F(scale * sd)
    return O.make_grid(n, n, n), cases.F(X), cases.F(Y), cases.F(Z), phi, sd


def seed(phi):
    """levelsetmethod's phicorrected before the geometric step (:303-304)"""
    return cases.F(np.where(phi < -EPS, -9.9, np.where(phi > EPS, 9.9, phi)))


def test_axis_plane_is_exact(oracle):
    g, x, y, z, phi, sd = _box(14)
    out, ids, info = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    assert info["nnodes"] > 0 and info["nsecond"] > 0
    m = ids != 0
    assert np.abs(out[m] - sd[m]).max() <= 1e-13
    assert np.all(out[ids == 0] == np.where(phi[ids == 0] > 0, 9.9, -9.9))


def test_tilted_plane_never_underestimates(oracle):
    g, x, y, z, phi, sd = _box(14, tilt=(0.3, -0.2, 1.0), scale=3.0)
    out, ids, _ = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    m = ids != 0
    assert np.all(np.sign(out[m]) == np.sign(sd[m]))
    assert (np.abs(out[m]) - np.abs(sd[m])).min() >= -1e-12
    # pnodes sit next to the surface: their error is O(h^2)
    assert (np.abs(out[ids > 0]) - np.abs(sd[ids > 0])).max() <= 0.01


def test_tags(oracle):
    g, x, y, z, phi, q = cases.curvilinear(16, 12, 10, seed=4)
    out, ids, info = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    pn = ids > 0
    flat = ids.ravel(order="F")
    # ids 1..nnodes in the array's own order
    assert np.array_equal(flat[flat > 0], np.arange(1, info["nnodes"] + 1))
    # -1 = non-pnode within +-4 of a pnode (dilation of the pnode mask)
    d = pn.copy()
    for ax in range(3):
        e = d.copy()
        for s in range(1, 5):
            sl_a = [slice(None)] * 3
            sl_b = [slice(None)] * 3
            sl_a[ax], sl_b[ax] = slice(s, None), slice(None, -s)
            e[tuple(sl_a)] |= d[tuple(sl_b)]
            e[tuple(sl_b)] |= d[tuple(sl_a)]
        d = e
    assert np.array_equal(ids == -1, d & ~pn)
    assert info["nsecond"] == int((ids == -1).sum())
    # both ends of every grid edge that crosses zero are pnodes (each grid
    # edge is an edge of a tetrahedron of the split, which is then a K one)
    s = np.sign(phi)
    for ax in range(3):
        a = [slice(None)] * 3
        b = [slice(None)] * 3
        a[ax], b[ax] = slice(1, None), slice(None, -1)
        cross = s[tuple(a)] * s[tuple(b)] < 0
        assert cross.any()
        assert np.all(pn[tuple(a)][cross]) and np.all(pn[tuple(b)][cross])
    assert np.all(np.abs(out[ids == 0]) == 9.9)


def test_global_mass_correction_restores_the_k_volume(oracle):
    g, x, y, z, phi, _ = cases.curvilinear(16, 12, 10, seed=5)
    phi = cases.F(1.7 * phi)
    v = oracle.total_water_volume(g, phi, x, y, z)
    p = O.make_params(GlobalMassCorrection=1)
    out, ids, info = oracle.geometric_reinitialisation(g, p, phi, x, y, z, v[0], seed(phi))
    assert info["newton_converged"] == 1 and info["C"] != 0.0
    w = oracle.total_water_volume(g, out, x, y, z)
    assert abs(w[0] - v[0]) <= 1e-9 * v[0]
    # without the correction the K volume moves
    out0, _, _ = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, v[0], seed(phi))
    w0 = oracle.total_water_volume(g, out0, x, y, z)
    assert abs(w0[0] - v[0]) > 100 * abs(w[0] - v[0])


def test_unreachable_target_drops_the_correction(oracle):
    """The reference's own ConvergenceVolume (total before minus K and second
    volumes after) aims the K tetrahedra at the bulk volume; Newton does not
    converge in 20 iterations and C is dropped (NewtonRaphsonSolver.F90)."""
    g, x, y, z, phi, _ = cases.curvilinear(14, 10, 9, seed=6)
    v = oracle.total_water_volume(g, phi, x, y, z)
    p = O.make_params(GlobalMassCorrection=1)
    out, _, info = oracle.geometric_reinitialisation(g, p, phi, x, y, z, v[3] - (v[0] + v[1]), seed(phi))
    out0, _, _ = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    if not info["newton_converged"]:
        assert info["C"] == 0.0
        assert np.array_equal(out, out0)


def test_hybrid_levelsetmethod_band(oracle):
    g, x, y, z, phi, q = cases.curvilinear(18, 12, 24, seed=7)
    csi, eta, zet, aj = oracle.mg_metrics(g, x, y, z)
    h = 1.0 / 17
    p = O.make_params(epslsm=1.5 * h, delti_lsm=0.01, hybrid_reinitialisation=1)
    out, vols = oracle.levelsetmethod(g, p, q, csi, eta, zet, aj, phi, phi, x, y, z, 1)
    assert np.isfinite(out).all()
    assert np.any(np.abs(out) == 9.9)
    # RNfreq = 2 at iteration 1: no reinitialisation, but the band mask still
    # applies (it depends on call_reinitialisation and the hybrid switch only)
    p2 = O.make_params(epslsm=1.5 * h, delti_lsm=0.01, hybrid_reinitialisation=1, RNfreq=2)
    adv_only, _ = oracle.levelsetmethod(g, p2, q, csi, eta, zet, aj, phi, phi, x, y, z, 1)
    p3 = O.make_params(epslsm=1.5 * h, delti_lsm=0.01, hybrid_reinitialisation=0, RNfreq=2)
    full, _ = oracle.levelsetmethod(g, p3, q, csi, eta, zet, aj, phi, phi, x, y, z, 1)
    _, band = oracle.total_water_volume(g, phi, x, y, z, with_nodes=True)
    inner = np.zeros(phi.shape, dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    off = inner & (band == 0)
    assert off.any() and np.array_equal(adv_only[off], phi[off])
    assert np.abs(full[off] - phi[off]).max() > 0.0


@pytest.mark.parametrize("bad", ["ghost", "open_face"])
def test_geometric_rejects_subdomains(oracle, bad):
    g, x, y, z, phi, _ = cases.curvilinear(12, 10, 9, seed=1)
    if bad == "ghost":
        g.igp = 2
        g.physical_face[0] = 0
    else:
        g.physical_face[3] = 0
        g.jgp = 2
    with pytest.raises(RuntimeError):
        oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))


def _zero_plane(n=13):
    """phi exactly 0 on the node plane z = 0.5 (n odd): tetrahedra with three
    zero vertices (a face on the surface) and with one or two"""
    X, Y, Z = np.meshgrid(*(np.linspace(0, 1, n),) * 3, indexing="ij")
    k = np.arange(n)[None, None, :] - (n - 1) // 2
    phi = cases.F(-2.0 * k / (n - 1) + 0.0 * X)
    return O.make_grid(n, n, n), cases.F(X), cases.F(Y), cases.F(Z), phi


def _zero_slab(n=13):
    """phi exactly 0 on three node planes: tetrahedra with four zero vertices"""
    g, x, y, z, phi = _zero_plane(n)
    k = np.arange(n)[None, None, :] - (n - 1) // 2
    phi = cases.F(np.where(np.abs(k) <= 1, 0.0, phi) + 0.0 * x)
    return g, x, y, z, phi


def test_zero_plane_is_exact(oracle):
    g, x, y, z, phi = _zero_plane()
    out, ids, info = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    sd = 0.5 - z
    m = ids != 0
    # the surface is the node plane itself: its faces are the triangles
    assert info["ntetrahedra"] > 0
    assert np.abs(np.abs(out[m]) - np.abs(sd[m])).max() <= 1e-13
    assert np.all(out[(ids > 0) & (phi == 0.0)] == 0.0)


def test_zero_slab_runs(oracle):
    g, x, y, z, phi = _zero_slab()
    out, ids, info = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    assert np.isfinite(out).all() and info["nnodes"] > 0
    # nodes of the slab are pnodes; the nearest triangles are the faces of
    # the tetrahedra that touch the slab's outer planes
    assert np.all(ids[phi == 0.0] > 0)


def _near_zero(n=13):
    """the zero plane with its nodes perturbed to +-1e-17 (below epsilon),
    +-1e-310 (below tiny), +0.0 and -0.0, in a seeded pattern"""
    g, x, y, z, phi = _zero_plane(n)
    rng = np.random.default_rng(12)
    vals = np.array([1e-17, -1e-17, 1e-310, -1e-310, 0.0, -0.0])
    kz = (n - 1) // 2
    phi[:, :, kz] = vals[rng.integers(0, len(vals), size=(n, n))]
    return g, x, y, z, phi


def test_near_zero_values_run(oracle):
    g, x, y, z, phi = _near_zero()
    out, ids, info = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    assert np.isfinite(out).all() and info["ntetrahedra"] > 0
    kz = (phi.shape[2] - 1) // 2
    assert np.all(ids[:, :, kz] > 0)
    # every triangle lies on the plane to ~1e-17: no distance falls below the
    # plane's (vertices and edges on the zero level give no triangle in the
    # reference, so some distances come from farther triangles)
    m = ids != 0
    assert (np.abs(out[m]) - np.abs(0.5 - z[m])).min() >= -1e-12


def test_openmp_oracle_is_bit_identical(oracle):
    """the timing build (OpenMP) gives the checker's bits (no mass correction:
    its Newton sums are serial in both)"""
    omp = O.Oracle(omp=True)
    g, x, y, z, phi, _ = cases.curvilinear(20, 14, 16, seed=3)
    a = oracle.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    b = omp.geometric_reinitialisation(g, O.make_params(), phi, x, y, z, 0.0, seed(phi))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[2] == b[2]


def test_no_interface_changes_nothing(oracle):
    g, x, y, z, phi, _ = cases.curvilinear(12, 10, 9, seed=2)
    phi = cases.F(np.abs(phi) + 0.5)          # all water: no phase-change cell
    pc0 = seed(phi)
    out, ids, info = oracle.geometric_reinitialisation(g, O.make_params(GlobalMassCorrection=1), phi, x, y, z,
                                                       1.0, pc0)
    assert info["nnodes"] == 0 and info["ntetrahedra"] == 0 and info["nsecond"] == 0
    assert np.array_equal(out, pc0) and not ids.any()
