"""The FP64 torch tape of the batched step (tests/lsm_tape.py), pinned on CPU.

1. Its forward equals the FP64 oracle's `levelsetmethod` (no volume) to
   rounding, for RNitermax 0 and 3 over three steps on two uneven instances.
2. Its autograd gradient equals central finite differences of its own
   forward (16 seeded directions for phi0 and for q, relative error <= 1e-4).
   The step is piecewise smooth (the band sign threshold, the BigPhi switch
   and the upwind / Godunov selections are branch points); a direction whose
   finite difference changes between steps h and h/2 crossed a branch point
   and is not scored.

The GPU adjoint kernels are compared with this tape in test_gpu_adjoint.py.
"""
import numpy as np
import pytest

import oracle as O

torch = pytest.importorskip("torch")
import lsm_tape as T  # noqa: E402

NSTEPS = 3
FD_TOL = 1e-4


@pytest.fixture(scope="module")
def tape_cases(oracle):
    from nslsm import configs
    out = []
    for it in configs.batched_instances(n_inst=2, lo=12, hi=18, seed=3, cfl=0.5):
        g = O.make_grid(*it.grid.shape)
        csi, eta, zet, aj = oracle.mg_metrics(g, it.x, it.y, it.z)
        out.append(dict(it=it, g=g, csi=csi, eta=eta, zet=zet, aj=aj, dt=it.time_step(csi, eta, zet)))
    return out


@pytest.mark.parametrize("R", [0, 3])
def test_tape_forward_matches_oracle(oracle, tape_cases, R):
    for c in tape_cases:
        it = c["it"]
        op = O.make_params(epslsm=it.eps, delti_lsm=c["dt"], RNitermax=R, RNtimestep=it.dtau, BigPhi=5.0)
        phi = it.phi0
        for s in range(1, NSTEPS + 1):
            phi, _ = oracle.levelsetmethod(c["g"], op, it.q, c["csi"], c["eta"], c["zet"], c["aj"], phi, phi, it.x,
                                           it.y, it.z, s)
        M = T.metrics_torch(c["csi"], c["eta"], c["zet"])
        got = T.run(T.to_torch(it.phi0), T.to_torch(it.q), M, c["dt"], it.dtau, it.eps, R, NSTEPS)
        assert float((got - T.to_torch(phi)).abs().max()) <= 1e-13


def _loss(c, R, phi0, q, wts):
    it = c["it"]
    M = T.metrics_torch(c["csi"], c["eta"], c["zet"])
    return (T.run(phi0, q, M, c["dt"], it.dtau, it.eps, R, NSTEPS) * wts).sum()


def fd_check(f, x0, grad, ndir, seed, h=1e-6, mask=None):
    """central differences of f along seeded directions; returns (scored, worst rel err)"""
    gen = torch.Generator().manual_seed(seed)
    worst, scored = 0.0, 0
    for _ in range(ndir):
        v = torch.randn(x0.shape, generator=gen, dtype=torch.float64)
        if mask is not None:
            v = v * mask
        fd1 = (f(x0 + h * v) - f(x0 - h * v)) / (2 * h)
        fd2 = (f(x0 + 0.5 * h * v) - f(x0 - 0.5 * h * v)) / h
        if abs(fd1 - fd2) > 1e-5 * max(abs(fd1), 1e-12):
            continue   # a branch point between x0 - h v and x0 + h v
        an = float((grad * v).sum())
        worst = max(worst, abs(an - fd1) / max(abs(fd1), 1e-12))
        scored += 1
    return scored, worst


@pytest.mark.parametrize("R", [0, 3])
def test_tape_gradient_matches_central_differences(tape_cases, R):
    c = tape_cases[0]
    it = c["it"]
    gen = torch.Generator().manual_seed(11)
    phi0 = T.to_torch(it.phi0)
    q = T.to_torch(it.q)
    wts = torch.randn(phi0.shape, generator=gen, dtype=torch.float64)
    p = phi0.clone().requires_grad_(True)
    qq = q.clone().requires_grad_(True)
    _loss(c, R, p, qq, wts).backward()
    with torch.no_grad():
        n, worst = fd_check(lambda x: float(_loss(c, R, x, q, wts)), phi0, p.grad, 16, 5)
        assert n >= 12 and worst <= FD_TOL, (n, worst)
        qmask = torch.zeros(q.shape, dtype=torch.float64)
        qmask[..., 1:] = 1.0
        n, worst = fd_check(lambda x: float(_loss(c, R, phi0, x, wts)), q, qq.grad, 16, 6, mask=qmask)
        assert n >= 12 and worst <= FD_TOL, (n, worst)
    assert float(qq.grad[..., 0].abs().max()) == 0.0


@pytest.mark.parametrize("btype", [(0, 2, 1, 0, 1, 0), (2, 2, 0, 0, 2, 1)])
def test_tape_forward_other_boundary_types(oracle, tape_cases, btype):
    c = tape_cases[1]
    it = c["it"]
    op = O.make_params(epslsm=it.eps, delti_lsm=c["dt"], RNitermax=2, RNtimestep=it.dtau, BigPhi=5.0,
                       btype_lsm=btype)
    phi = it.phi0
    for s in range(1, NSTEPS + 1):
        phi, _ = oracle.levelsetmethod(c["g"], op, it.q, c["csi"], c["eta"], c["zet"], c["aj"], phi, phi, it.x,
                                       it.y, it.z, s)
    M = T.metrics_torch(c["csi"], c["eta"], c["zet"])
    got = T.run(T.to_torch(it.phi0), T.to_torch(it.q), M, c["dt"], it.dtau, it.eps, 2, NSTEPS, btype=btype)
    assert float((got - T.to_torch(phi)).abs().max()) <= 1e-13
