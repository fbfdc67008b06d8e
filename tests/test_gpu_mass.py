"""FP64 mass correction of the batched path (lsm_batch_config.mass_correction,
lsm_batch_set_mass_target) on the GPU.

After each step's final bcond_lsm the batch measures the water volume V of
the result (the reference's TotalWaterVolume cases, exact fixed-point sum)
and A = dV/dC, its derivative under a uniform shift phi + C, and applies
phi += C with C = (target - V) / A.  Checked here:

  * one FP64 step: V equals the oracle's volume of the oracle's
    uncorrected step; A equals a central difference of the oracle's volume
    under a shift (1e-6); C = (target - V) / A; phi - C equals the oracle's
    uncorrected phi (1e-12); the corrected field's volume is much closer to
    the target (one Newton step: the error falls by > 100x);
  * 20 FP32 steps on instances of 40..56 nodes per axis: the relative
    volume drift against the target stays below 1e-6 (spec bar), well
    below the uncorrected run's (on coarser grids the per-step volume loss
    is larger and the one Newton step per step leaves a residual of order
    its square);
  * the FP64 adjoint with the correction equals central differences of the
    corrected forward along 24 seeded directions (the shift's derivative
    includes dA/dphi through second-order dual numbers), each at step 1e-5
    where its quotients at h and h/2 agree, else at 1e-6: within BAR_MC =
    1e-3 (measured worst 2.5e-4, median ~5e-6), the quotients' own limit (the
    fixed-point volume makes the corrected forward noisy at ~1e-11 in the
    loss), while dropping the correction's adjoint moves the gradient by
    more than 1e-2;
  * the checkpoint interval does not change that gradient (bit-identical);
  * the FP32 adjoint follows the FP64 one.
"""
import math

import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

NSTEPS = 3
# the corrected step's fixed-point volume (2^-48 per cell) moves C by ~1e-13
# between nearby inputs (~1e-11 in these losses), and the correction adds
# kinks (tetrahedron cases switching): difference quotients reach ~3e-4
BAR_MC = 1e-3


@pytest.fixture(scope="module")
def mcases(oracle, lib_built):
    from nslsm import configs
    out = []
    for it in configs.batched_instances(n_inst=3, lo=12, hi=20, seed=7, cfl=0.5):
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = oracle.mg_metrics(g, it.x, it.y, it.z)
        out.append(dict(it=it, g=g, csi=csi, eta=eta, zet=zet, aj=aj, dt=it.time_step(csi, eta, zet)))
    return out


def _batch(cases, R, precision="fp64", **kw):
    from nslsm.batch import LevelSetBatch
    b = LevelSetBatch([(*c["it"].grid.shape, c["dt"], c["it"].dtau, c["it"].eps) for c in cases], RNitermax=R,
                      btype=(1,) * 6, BigPhi=5.0, precision=precision, mass_correction=True, **kw)
    for k, c in enumerate(cases):
        it = c["it"]
        b.set_geometry(k, it.x, it.y, it.z, c["csi"], c["eta"], c["zet"])
        b.set_velocity(k, it.q)
        b.set_phi(k, it.phi0)
    return b


def _targets(oracle, cases, scale):
    return [scale * oracle.total_water_volume(c["g"], c["it"].phi0, c["it"].x, c["it"].y, c["it"].z)[3]
            for c in cases]


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def test_one_fp64_step_matches_oracle_plus_shift(oracle, mcases):
    R = 3
    b = _batch(mcases, R)
    tg = _targets(oracle, mcases, 1.002)
    for k, t in enumerate(tg):
        b.set_mass_target(k, t)
    b.step(1)
    st = b.mass_state()
    for k, c in enumerate(mcases):
        it = c["it"]
        op = O.make_params(epslsm=it.eps, delti_lsm=c["dt"], RNitermax=R, RNtimestep=it.dtau, BigPhi=5.0)
        pu, _ = oracle.levelsetmethod(c["g"], op, it.q, c["csi"], c["eta"], c["zet"], c["aj"], it.phi0, it.phi0, it.x,
                                      it.y, it.z, 1)
        vol = lambda f: oracle.total_water_volume(c["g"], np.asfortranarray(f), it.x, it.y, it.z)[3]  # noqa: E731
        V, A, C, T = st[k]
        assert T == tg[k]
        assert abs(V - vol(pu)) <= 1e-10 * abs(V), (V, vol(pu))
        d = 1e-7
        a_fd = (vol(pu + d) - vol(pu - d)) / (2 * d)
        assert abs(A - a_fd) <= 1e-6 * abs(a_fd), (A, a_fd)
        assert abs(C - (T - V) / A) <= 1e-15 * abs(C)
        got = b.get_phi(k)
        assert float(np.abs((got - C) - pu).max()) <= 1e-12
        before, after = abs(V - T), abs(vol(got) - T)
        assert after <= 1e-2 * before, (before, after)
    b.close()


def test_fp32_volume_drift_below_bar(oracle, lib_built):
    from nslsm import configs
    from nslsm.batch import LevelSetBatch
    mcases = []
    for it in configs.batched_instances(n_inst=3, lo=40, hi=56, seed=9, cfl=0.5):
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = oracle.mg_metrics(g, it.x, it.y, it.z)
        mcases.append(dict(it=it, g=g, csi=csi, eta=eta, zet=zet, aj=aj, dt=it.time_step(csi, eta, zet)))
    R, n = 5, 20
    tg = _targets(oracle, mcases, 1.0)
    drift = {}
    for mc in (True, False):
        b = LevelSetBatch([(*c["it"].grid.shape, c["dt"], c["it"].dtau, c["it"].eps) for c in mcases], RNitermax=R,
                          btype=(1,) * 6, BigPhi=5.0, mass_correction=mc)
        for k, c in enumerate(mcases):
            it = c["it"]
            b.set_geometry(k, it.x, it.y, it.z, c["csi"], c["eta"], c["zet"])
            b.set_velocity(k, it.q)
            b.set_phi(k, it.phi0)
            if mc:
                b.set_mass_target(k, tg[k])
        b.step(n)
        v = b.water_volume()[:, 3]
        drift[mc] = max(abs(v[k] - tg[k]) / tg[k] for k in range(len(mcases)))
        b.close()
    print("relative volume drift after %d FP32 steps: corrected %.2e, uncorrected %.2e" % (n, drift[True],
                                                                                          drift[False]))
    assert drift[True] <= 1e-6
    assert drift[True] < drift[False]


def _adjoint(b, cases, wts, nsteps=NSTEPS, ck=2):
    for k, c in enumerate(cases):
        b.set_phi(k, c["it"].phi0)
    b.forward_record(nsteps, ck)
    for k, w in enumerate(wts):
        b.set_grad_phi(k, w)
    b.backward()
    return [b.get_grad_phi0(k) for k in range(len(cases))], [b.get_grad_velocity(k) for k in range(len(cases))]


def _weights(cases, seed=13):
    rng = np.random.default_rng(seed)
    return [np.asfortranarray(rng.standard_normal(c["it"].grid.shape)) for c in cases]


def test_fp64_adjoint_with_mass_correction_matches_central_differences(oracle, mcases):
    R = 3
    b = _batch(mcases, R)
    for k, t in enumerate(_targets(oracle, mcases, 1.002)):
        b.set_mass_target(k, t)
    wts = _weights(mcases)
    gphi, gq = _adjoint(b, mcases, wts)

    def loss(phis=None, qs=None):
        for k, c in enumerate(mcases):
            b.set_phi(k, c["it"].phi0 if phis is None else phis[k])
            b.set_velocity(k, c["it"].q if qs is None else qs[k])
        b.step(NSTEPS, volumes=False)
        return sum(float((b.get_phi(k) * wts[k]).sum()) for k in range(len(mcases)))

    rng = np.random.default_rng(5)
    worst, rows = 0.0, []
    for d in range(24):
        if d % 2 == 0:
            v = [np.asfortranarray(rng.standard_normal(c["it"].grid.shape)) for c in mcases]
            x0 = [c["it"].phi0 for c in mcases]
            f = lambda t: loss(phis=[x + t * vv for x, vv in zip(x0, v)])  # noqa: E731
            an = sum(float((g * vv).sum()) for g, vv in zip(gphi, v))
        else:
            v = []
            for c in mcases:
                vv = np.zeros_like(c["it"].q)
                vv[1:] = rng.standard_normal(vv[1:].shape)
                v.append(vv)
            x0 = [c["it"].q for c in mcases]
            f = lambda t: loss(qs=[x + t * vv for x, vv in zip(x0, v)])  # noqa: E731
            an = sum(float((g * vv).sum()) for g, vv in zip(gq, v))
        # the corrected forward is piecewise smooth, and its fixed-point
        # volume (2^-48 per cell) moves C by ~1e-13 between nearby inputs, a
        # noise of ~1e-11 in the loss: steps of 1e-5 (else 1e-6 when a
        # branch point was crossed), errors relative to the larger of the
        # directional derivative and its typical size |g| |v| / sqrt(n)
        gn = math.sqrt(sum(float((g * g).sum()) for g in (gphi if d % 2 == 0 else gq)))
        vn = math.sqrt(sum(float((vv * vv).sum()) for vv in v))
        scale = max(abs(an), gn * vn / math.sqrt(sum(vv.size for vv in v)))
        used = None
        for h in (1e-5, 1e-6):
            fd1 = (f(h) - f(-h)) / (2 * h)
            fd2 = (f(0.5 * h) - f(-0.5 * h)) / h
            if abs(fd1 - fd2) <= 1e-4 * scale:
                used = h
                break
        assert used is not None, (d, fd1, fd2, scale)
        err = abs(an - fd1) / scale
        rows.append("h=%g err=%.1e" % (used, err))
        worst = max(worst, err)
    b.close()
    # the check must be able to see the correction's adjoint: the gradient
    # without it differs by far more than the bar
    from nslsm.batch import LevelSetBatch
    b0 = LevelSetBatch([(*c["it"].grid.shape, c["dt"], c["it"].dtau, c["it"].eps) for c in mcases], RNitermax=R,
                       btype=(1,) * 6, BigPhi=5.0, precision="fp64")
    for k, c in enumerate(mcases):
        it = c["it"]
        b0.set_geometry(k, it.x, it.y, it.z, c["csi"], c["eta"], c["zet"])
        b0.set_velocity(k, it.q)
    g0phi, _ = _adjoint(b0, mcases, wts)
    b0.close()
    moved = max(_rel(g0phi[k], gphi[k]) for k in range(len(mcases)))
    print("mass-corrected adjoint vs central differences: " + "; ".join(rows))
    print("the correction moves the phi0 gradient by %.2e (relative)" % moved)
    assert worst <= BAR_MC, worst
    assert moved >= 10 * BAR_MC, moved


def test_checkpoint_interval_does_not_change_corrected_gradient(oracle, mcases):
    wts = _weights(mcases)
    tg = _targets(oracle, mcases, 1.002)
    outs = []
    for ck in (1, 2, 5):
        b = _batch(mcases, 2)
        for k, t in enumerate(tg):
            b.set_mass_target(k, t)
        outs.append(_adjoint(b, mcases, wts, nsteps=5, ck=ck))
        b.close()
    for o in outs[1:]:
        for a, c in zip(outs[0][0] + outs[0][1], o[0] + o[1]):
            assert np.array_equal(a, c)


def test_fp32_corrected_adjoint_follows_fp64(oracle, mcases):
    wts = _weights(mcases)
    tg = _targets(oracle, mcases, 1.002)
    res = {}
    for prec in ("fp64", "fp32"):
        b = _batch(mcases, 3, precision=prec, autotune=False)
        for k, t in enumerate(tg):
            b.set_mass_target(k, t)
        res[prec] = _adjoint(b, mcases, wts)
        b.close()
    for k in range(len(mcases)):
        assert _rel(res["fp32"][0][k], res["fp64"][0][k]) <= 1e-3
        assert _rel(res["fp32"][1][k], res["fp64"][1][k]) <= 1e-3


def test_mass_target_needs_the_correction(mcases):
    from nslsm import LsmError
    from nslsm.batch import LevelSetBatch
    c = mcases[0]
    b = LevelSetBatch([(*c["it"].grid.shape, c["dt"], c["it"].dtau, c["it"].eps)], RNitermax=2)
    with pytest.raises(LsmError):
        b.set_mass_target(0, 1.0)
    b.close()
