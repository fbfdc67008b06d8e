"""Adjoint of the batched level-set path (lsm_batch_forward_record /
lsm_batch_backward) on the GPU.

  * the FP64 batch forward equals the FP64 oracle's levelsetmethod;
  * the FP64 adjoint kernels equal the autograd gradient of the FP64 torch
    tape (tests/lsm_tape.py, itself pinned to the oracle and to central
    differences on CPU) for phi0 and q, RNitermax 0 and 3, three steps with
    a checkpoint every two steps;
  * the FP64 adjoint equals central differences of the batch's own forward
    along 24 seeded directions, step 1e-7 (relative error <= 1e-4;
    directions whose difference quotient changes between steps h and h/2
    crossed a branch point of the piecewise-smooth step and are not scored;
    at least 16 must be scored);
  * the checkpoint interval does not change the gradient (bit-identical);
  * the FP32 adjoint follows the FP64 one;
  * nslsm.batch.transport (torch.autograd.Function) returns the same
    gradients as the direct C-ABI calls.
"""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
import lsm_tape as T  # noqa: E402

NSTEPS = 3
CKPT = 2


@pytest.fixture(scope="module")
def adj_cases(oracle, lib_built):
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
                      btype=(1,) * 6, BigPhi=5.0, precision=precision, **kw)
    for k, c in enumerate(cases):
        it = c["it"]
        b.set_geometry(k, it.x, it.y, it.z, c["csi"], c["eta"], c["zet"])
        b.set_velocity(k, it.q)
        b.set_phi(k, it.phi0)
    return b


def _weights(cases, seed=11):
    rng = np.random.default_rng(seed)
    return [np.asfortranarray(rng.standard_normal(c["it"].grid.shape)) for c in cases]


def _adjoint(b, cases, wts, nsteps=NSTEPS, ck=CKPT):
    for k, c in enumerate(cases):
        b.set_phi(k, c["it"].phi0)
    b.forward_record(nsteps, ck)
    for k, w in enumerate(wts):
        b.set_grad_phi(k, w)
    b.backward()
    return [b.get_grad_phi0(k) for k in range(len(cases))], [b.get_grad_velocity(k) for k in range(len(cases))]


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


@pytest.mark.parametrize("R", [0, 3])
def test_fp64_batch_forward_matches_oracle(oracle, adj_cases, R):
    b = _batch(adj_cases, R)
    vols = b.step(NSTEPS)
    for k, c in enumerate(adj_cases):
        it = c["it"]
        op = O.make_params(epslsm=it.eps, delti_lsm=c["dt"], RNitermax=R, RNtimestep=it.dtau, BigPhi=5.0)
        phi = it.phi0
        for s in range(1, NSTEPS + 1):
            phi, rv = oracle.levelsetmethod(c["g"], op, it.q, c["csi"], c["eta"], c["zet"], c["aj"], phi, phi, it.x,
                                            it.y, it.z, s)
        assert float(np.abs(b.get_phi(k) - phi).max()) <= 1e-12
        # pre-advection volumes of the last step (64-bit fixed point, 2^-48 per cell)
        assert np.allclose(vols[k], rv, rtol=1e-10, atol=0), (vols[k], rv)
    b.close()


@pytest.mark.parametrize("mode", ["store", "recompute"])
@pytest.mark.parametrize("R", [0, 3])
def test_fp64_adjoint_matches_torch_tape(adj_cases, R, mode):
    b = _batch(adj_cases, R, adjoint_mode=mode)
    wts = _weights(adj_cases)
    gphi, gq = _adjoint(b, adj_cases, wts)
    b.close()
    for k, c in enumerate(adj_cases):
        it = c["it"]
        M = T.metrics_torch(c["csi"], c["eta"], c["zet"], "cuda")
        p = T.to_torch(it.phi0, "cuda").requires_grad_(True)
        q = T.to_torch(it.q, "cuda").requires_grad_(True)
        out = T.run(p, q, M, c["dt"], it.dtau, it.eps, R, NSTEPS)
        (out * T.to_torch(wts[k], "cuda")).sum().backward()
        ref_phi = np.asfortranarray(p.grad.cpu().numpy().T)
        ref_q = np.asfortranarray(q.grad.cpu().numpy().T)
        assert _rel(gphi[k], ref_phi) <= 1e-10, (k, _rel(gphi[k], ref_phi))
        assert _rel(gq[k], ref_q) <= 1e-10, (k, _rel(gq[k], ref_q))
        assert float(np.abs(gq[k][0]).max()) == 0.0


def test_fp64_adjoint_matches_central_differences(adj_cases):
    R = 3
    b = _batch(adj_cases, R)
    wts = _weights(adj_cases)
    gphi, gq = _adjoint(b, adj_cases, wts)

    def loss(phis=None, qs=None):
        for k, c in enumerate(adj_cases):
            b.set_phi(k, c["it"].phi0 if phis is None else phis[k])
            b.set_velocity(k, c["it"].q if qs is None else qs[k])
        b.step(NSTEPS, volumes=False)
        return sum(float((b.get_phi(k) * wts[k]).sum()) for k in range(len(adj_cases)))

    rng = np.random.default_rng(5)
    h = 1e-7
    scored, worst = 0, 0.0
    for d in range(24):
        if d % 2 == 0:   # phi0 direction
            v = [np.asfortranarray(rng.standard_normal(c["it"].grid.shape)) for c in adj_cases]
            x0 = [c["it"].phi0 for c in adj_cases]
            f = lambda t: loss(phis=[x + t * vv for x, vv in zip(x0, v)])
            an = sum(float((g * vv).sum()) for g, vv in zip(gphi, v))
        else:            # velocity direction (q(2:4))
            v = []
            for c in adj_cases:
                vv = np.zeros_like(c["it"].q)
                vv[1:] = rng.standard_normal(vv[1:].shape)
                v.append(vv)
            x0 = [c["it"].q for c in adj_cases]
            f = lambda t: loss(qs=[x + t * vv for x, vv in zip(x0, v)])
            an = sum(float((g * vv).sum()) for g, vv in zip(gq, v))
        fd1 = (f(h) - f(-h)) / (2 * h)
        fd2 = (f(0.5 * h) - f(-0.5 * h)) / h
        if abs(fd1 - fd2) > 1e-5 * max(abs(fd1), 1e-12):
            continue
        scored += 1
        worst = max(worst, abs(an - fd1) / max(abs(fd1), 1e-12))
    b.close()
    assert scored >= 16 and worst <= 1e-4, (scored, worst)


@pytest.mark.parametrize("mode", ["store", "recompute"])
def test_checkpoint_interval_does_not_change_gradient(adj_cases, mode):
    wts = _weights(adj_cases)
    outs = []
    for ck in (1, 2, 5):
        b = _batch(adj_cases, 2, adjoint_mode=mode)
        outs.append(_adjoint(b, adj_cases, wts, nsteps=5, ck=ck))
        b.close()
    for o in outs[1:]:
        for a, c in zip(outs[0][0] + outs[0][1], o[0] + o[1]):
            assert np.array_equal(a, c)


def test_fp32_adjoint_follows_fp64(adj_cases):
    wts = _weights(adj_cases)
    res = {}
    for prec in ("fp64", "fp32"):
        b = _batch(adj_cases, 3, precision=prec, autotune=False)
        res[prec] = _adjoint(b, adj_cases, wts)
        b.close()
    for k in range(len(adj_cases)):
        assert _rel(res["fp32"][0][k], res["fp64"][0][k]) <= 1e-3
        assert _rel(res["fp32"][1][k], res["fp64"][1][k]) <= 1e-3


def test_autograd_function_matches_direct_calls(adj_cases):
    from nslsm.batch import transport
    b = _batch(adj_cases, 3)
    wts = _weights(adj_cases)
    gphi, gq = _adjoint(b, adj_cases, wts)
    phis = [T.to_torch(c["it"].phi0, "cuda").requires_grad_(True) for c in adj_cases]
    qs = [T.to_torch(c["it"].q, "cuda").requires_grad_(True) for c in adj_cases]
    outs = transport(b, NSTEPS, phis, qs, checkpoint_every=CKPT)
    sum((o * T.to_torch(w, "cuda")).sum() for o, w in zip(outs, wts)).backward()
    for k in range(len(adj_cases)):
        assert np.array_equal(np.asfortranarray(phis[k].grad.cpu().numpy().T), gphi[k])
        assert np.array_equal(np.asfortranarray(qs[k].grad.cpu().numpy().T), gq[k])
    b.close()


def test_batch_waits_for_torch_stream(adj_cases):
    """Inputs produced by torch on its current stream are read only after
    torch has written them (the batch runs on its own stream)."""
    c = adj_cases[0]
    b = _batch([c], 2)
    base = T.to_torch(c["it"].phi0, "cuda")
    for r in range(20):
        x = base.clone()
        for _ in range(50):          # a queue of kernels still running when set_phi is called
            x = x * 1.0000001 + 1e-9
        b.set_phi(0, x)
        got = b.get_phi(0, like=base)
        assert torch.equal(got, x), r
    b.close()


@pytest.mark.parametrize("btype", [(0, 2, 1, 0, 1, 0), (2, 2, 0, 0, 2, 1)])
def test_adjoint_other_boundary_types_match_tape(oracle, adj_cases, btype):
    """bcond_lsm types 0 (copy) and 2 (linear extrapolation on im; ignored on
    the other faces, as in the reference) in the forward against the oracle
    and in the adjoint against the torch tape."""
    from nslsm.batch import LevelSetBatch
    cases_ = adj_cases[:2]
    R = 2
    b = LevelSetBatch([(*c["it"].grid.shape, c["dt"], c["it"].dtau, c["it"].eps) for c in cases_], RNitermax=R,
                      btype=btype, BigPhi=5.0, precision="fp64")
    for k, c in enumerate(cases_):
        it = c["it"]
        b.set_geometry(k, it.x, it.y, it.z, c["csi"], c["eta"], c["zet"])
        b.set_velocity(k, it.q)
        b.set_phi(k, it.phi0)
    b.step(NSTEPS)
    for k, c in enumerate(cases_):
        it = c["it"]
        op = O.make_params(epslsm=it.eps, delti_lsm=c["dt"], RNitermax=R, RNtimestep=it.dtau, BigPhi=5.0,
                           btype_lsm=btype)
        phi = it.phi0
        for s in range(1, NSTEPS + 1):
            phi, _ = oracle.levelsetmethod(c["g"], op, it.q, c["csi"], c["eta"], c["zet"], c["aj"], phi, phi, it.x,
                                           it.y, it.z, s)
        assert float(np.abs(b.get_phi(k) - phi).max()) <= 1e-12
    wts = _weights(cases_)
    gphi, gq = _adjoint(b, cases_, wts)
    b.close()
    for k, c in enumerate(cases_):
        it = c["it"]
        M = T.metrics_torch(c["csi"], c["eta"], c["zet"], "cuda")
        p = T.to_torch(it.phi0, "cuda").requires_grad_(True)
        q = T.to_torch(it.q, "cuda").requires_grad_(True)
        out = T.run(p, q, M, c["dt"], it.dtau, it.eps, R, NSTEPS, btype=btype)
        (out * T.to_torch(wts[k], "cuda")).sum().backward()
        assert _rel(gphi[k], np.asfortranarray(p.grad.cpu().numpy().T)) <= 1e-10
        assert _rel(gq[k], np.asfortranarray(q.grad.cpu().numpy().T)) <= 1e-10


@pytest.mark.parametrize("ck", [CKPT, NSTEPS])
def test_second_backward_repeats_the_gradient(adj_cases, ck):
    """The forward keeps the last segment's internals; a second reverse
    sweep (after earlier segments were recomputed into the same slots, or
    with one segment only) gives the same gradient bit for bit."""
    cases_ = adj_cases[:2]
    b = _batch(cases_, 3)
    wts = _weights(cases_)
    g1, q1 = _adjoint(b, cases_, wts, ck=ck)
    for k, w in enumerate(wts):
        b.set_grad_phi(k, w)
    b.backward()
    for k in range(len(cases_)):
        assert np.array_equal(b.get_grad_phi0(k), g1[k])
        assert np.array_equal(b.get_grad_velocity(k), q1[k])
    b.close()


def test_adjoint_modes_agree(adj_cases):
    """Stored coefficients (the forward's own Godunov selections) and the
    reverse sweep's recomputation give the same FP64 gradient to rounding,
    and the same FP32 gradient to FP32 rounding."""
    wts = _weights(adj_cases)
    for prec, tol in (("fp64", 1e-13), ("fp32", 1e-5)):
        res = {}
        for mode in ("store", "recompute"):
            b = _batch(adj_cases, 3, precision=prec, adjoint_mode=mode, autotune=False)
            res[mode] = _adjoint(b, adj_cases, wts)
            b.close()
        for k in range(len(adj_cases)):
            assert _rel(res["store"][0][k], res["recompute"][0][k]) <= tol
            assert _rel(res["store"][1][k], res["recompute"][1][k]) <= tol


@pytest.mark.parametrize("mode", ["store", "recompute"])
def test_tiny_ragged_instances_adjoint(oracle, lib_built, mode):
    """The adjoint on instances of 4..9 nodes per axis (partial tiles in every
    kernel) against the FP64 torch tape."""
    from nslsm import configs
    cases_ = []
    for it in configs.batched_instances(n_inst=3, lo=4, hi=9, seed=8, cfl=0.5):
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = oracle.mg_metrics(g, it.x, it.y, it.z)
        cases_.append(dict(it=it, g=g, csi=csi, eta=eta, zet=zet, aj=aj, dt=it.time_step(csi, eta, zet)))
    R = 2
    b = _batch(cases_, R, adjoint_mode=mode)
    wts = _weights(cases_)
    gphi, gq = _adjoint(b, cases_, wts)
    b.close()
    for k, c in enumerate(cases_):
        it = c["it"]
        M = T.metrics_torch(c["csi"], c["eta"], c["zet"], "cuda")
        p = T.to_torch(it.phi0, "cuda").requires_grad_(True)
        q = T.to_torch(it.q, "cuda").requires_grad_(True)
        out = T.run(p, q, M, c["dt"], it.dtau, it.eps, R, NSTEPS)
        (out * T.to_torch(wts[k], "cuda")).sum().backward()
        assert _rel(gphi[k], np.asfortranarray(p.grad.cpu().numpy().T)) <= 1e-10
        assert _rel(gq[k], np.asfortranarray(q.grad.cpu().numpy().T)) <= 1e-10


def test_fp64_adjoint_thin_instances_match_torch_tape(oracle, lib_built):
    """Instances with fewer than 6 nodes along an axis: the adjoint then
    reverses that axis's two boundary faces one after the other instead of
    in one launch (their targets would overlap).  Gradients equal the torch
    tape to 1e-10 on a batch whose x and z axes take the sequential path and
    whose y axis takes the paired one."""
    from types import SimpleNamespace
    from nslsm.configs import _mesh
    cases = []
    for shape in ((16, 12, 5), (5, 14, 9)):
        XI, ET, ZE = _mesh(*shape)
        X, Y, Z = XI + 0.05 * ET, ET - 0.03 * ZE, ZE + 0.04 * XI
        F = lambda a: np.asfortranarray(a, dtype=np.float64)  # noqa: E731
        q = np.zeros((4,) + shape, order="F")
        q[1] = 0.6 + 0.3 * np.sin(2 * np.pi * Y)
        q[2] = -0.4 * np.cos(2 * np.pi * X)
        q[3] = 0.2 * np.sin(2 * np.pi * X)
        h = 1.0 / (max(shape) - 1)
        it = SimpleNamespace(grid=SimpleNamespace(shape=shape), x=F(X), y=F(Y), z=F(Z),
                             phi0=F(Z - 0.5 - 0.04 * np.cos(2 * np.pi * (2 * X + Y))), q=F(q), dtau=0.5 * h,
                             eps=1.5 * h)
        g = O.make_grid(*shape)
        csi, eta, zet, aj = oracle.mg_metrics(g, it.x, it.y, it.z)
        smax = max(float(np.abs(m[0] * q[1] + m[1] * q[2] + m[2] * q[3]).max()) for m in (csi, eta, zet))
        cases.append(dict(it=it, g=g, csi=csi, eta=eta, zet=zet, aj=aj, dt=0.4 / smax))
    R = 3
    b = _batch(cases, R)
    wts = _weights(cases)
    gphi, gq = _adjoint(b, cases, wts)
    b.close()
    for k, c in enumerate(cases):
        it = c["it"]
        M = T.metrics_torch(c["csi"], c["eta"], c["zet"], "cuda")
        p = T.to_torch(it.phi0, "cuda").requires_grad_(True)
        q = T.to_torch(it.q, "cuda").requires_grad_(True)
        out = T.run(p, q, M, c["dt"], it.dtau, it.eps, R, NSTEPS)
        (out * T.to_torch(wts[k], "cuda")).sum().backward()
        ref_phi = np.asfortranarray(p.grad.cpu().numpy().T)
        ref_q = np.asfortranarray(q.grad.cpu().numpy().T)
        assert _rel(gphi[k], ref_phi) <= 1e-10, (k, _rel(gphi[k], ref_phi))
        assert _rel(gq[k], ref_q) <= 1e-10, (k, _rel(gq[k], ref_q))
