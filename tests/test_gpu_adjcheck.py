"""The adjoint on its own configuration: the sphere of radius 0.15 at (0.35,
0.35, 0.35) in the LeVeque deformation field (frozen at t = 0 over the run),
128^3 unit box, 50 steps of WENO3-RK3 + 5 reinitialisation pseudo-steps,
eps = 1.5 h; loss = sum (H_eps(phi_T) - H_eps(phi_target))^2 with
H_eps the reference's heaviside (src/global_lsm.F90:105-118) and phi_target
from a run with the velocity scaled by 1.05; gradients with respect to phi0
and the velocity through the batch's hand-written adjoint with a checkpoint
every 10 steps.

  * the FP64 gradient equals the FP64 PyTorch tape's (tests/lsm_tape.py) on
    a 32^3 copy of the case (1e-10 relative);
  * central differences of the FP64 forward along 16 seeded directions (8 in
    the velocity, 8 in phi0; bar 1e-4 relative), each at the configured
    step 1e-6 where its difference quotients at h and h/2 agree, else at
    1e-8: the forward map is piecewise smooth, and a perturbation can move
    nodes across the sign field's band edge |phi| = eps of a later step
    (the field switches there between the Godunov update and the node
    pinned by the lambda correction).  With ~3e4 nodes next to that edge
    per step over 50 steps, a 1e-6 perturbation of phi0 crosses it almost
    surely (a velocity perturbation moves phi less and crosses it less
    often); at 1e-8 the quotients agree;
  * the frozen-sign-field assumption in isolation: on a field with every
    |phi| >= 2 eps over the run (no band edge to cross), central differences
    at 1e-6 agree with the adjoint in every direction, phi0 included (1e-5,
    ten times inside the bar);
  * the FP32 gradient follows the FP64 one.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
import lsm_tape as TAPE  # noqa: E402

NSTEPS, CKPT, R = 50, 10, 5


def H(p, e):
    return torch.where(p < -e, torch.zeros_like(p), torch.where(p > e, torch.ones_like(p),
                       0.5 * (1.0 + p / e + torch.sin(np.pi * p / e) / np.pi)))


def dH(p, e):
    return torch.where(p.abs() > e, torch.zeros_like(p), (1.0 + torch.cos(np.pi * p / e)) / (2.0 * e))


def _setup(n, phi0=None):
    from nslsm import LevelSet, configs
    case = configs.sphere_deformation(n, reinit_iters=R)
    g = case.grid
    ls = LevelSet(device=0)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()  # noqa: E731
    x, y, z = dev(case.x), dev(case.y), dev(case.z)
    csi, eta, zet, aj = ls.mg_metrics(g, x, y, z)
    q = dev(case.q(0.0))
    smax = max(float((m * q[..., 1:4]).sum(-1).abs().max()) for m in (csi, eta, zet))
    ls.close()
    return dict(case=case, g=g, x=x, y=y, z=z, csi=csi, eta=eta, zet=zet, q=q,
                phi0=dev(case.phi0 if phi0 is None else phi0(case)), dt=case.cfl / smax)


def _batch(S, prec):
    from nslsm.batch import LevelSetBatch
    c = S["case"]
    b = LevelSetBatch([(S["g"].ni, S["g"].nj, S["g"].nk, S["dt"], c.params.RNtimestep, c.params.epslsm)],
                      RNitermax=R, btype=(1,) * 6, BigPhi=5.0, precision=prec, autotune=False)
    b.set_geometry(0, S["x"], S["y"], S["z"], S["csi"], S["eta"], S["zet"])
    return b


def _forward(b, phi0, q, nsteps=NSTEPS):
    b.set_velocity(0, q)
    b.set_phi(0, phi0)
    b.step(nsteps, volumes=False)
    return b.get_phi(0, like=phi0)


def _adjoint(b, phi0, q, seed_fn, nsteps=NSTEPS, ck=CKPT):
    b.set_velocity(0, q)
    b.set_phi(0, phi0)
    b.forward_record(nsteps, ck)
    b.set_grad_phi(0, seed_fn(b.get_phi(0, like=phi0)))
    b.backward()
    return b.get_grad_phi0(0, like=phi0), b.get_grad_velocity(0, like=phi0)


def _rel(a, r):
    return float((a - r).norm() / r.norm())


def _fd(f, h):
    return (f(h) - f(-h)) / (2 * h), (f(0.5 * h) - f(-0.5 * h)) / h


@pytest.fixture(scope="module")
def big(lib_built):
    S = _setup(128)
    eps = S["case"].params.epslsm
    b = _batch(S, "fp64")
    target = _forward(b, S["phi0"], 1.05 * S["q"])
    seed = lambda phiT: 2.0 * (H(phiT, eps) - H(target, eps)) * dH(phiT, eps)  # noqa: E731
    gphi, gq = _adjoint(b, S["phi0"], S["q"], seed)
    yield dict(S=S, b=b, eps=eps, target=target, seed=seed, gphi=gphi, gq=gq)
    b.close()


def test_fp64_gradient_equals_torch_tape_on_32_cubed(lib_built):
    T = _setup(32)
    eps = T["case"].params.epslsm
    b = _batch(T, "fp64")
    tgt = _forward(b, T["phi0"], 1.05 * T["q"])
    gp, gq = _adjoint(b, T["phi0"], T["q"], lambda phiT: 2.0 * (H(phiT, eps) - H(tgt, eps)) * dH(phiT, eps))
    b.close()
    M = [m[..., c].contiguous() for m in (T["csi"], T["eta"], T["zet"]) for c in range(3)]
    p0 = T["phi0"].clone().requires_grad_(True)
    qq = T["q"].clone().requires_grad_(True)
    cp = T["case"].params
    out = TAPE.run(p0, qq, M, T["dt"], cp.RNtimestep, cp.epslsm, R, NSTEPS)
    ((H(out, eps) - H(tgt, eps)) ** 2).sum().backward()
    e_phi, e_q = _rel(gp, p0.grad), _rel(gq, qq.grad)
    print("32^3 tape: grad phi0 %.2e, grad q %.2e" % (e_phi, e_q))
    assert e_phi <= 1e-10 and e_q <= 1e-10


def _directions(S, kind, count, seed):
    gen = torch.Generator(device="cuda").manual_seed(seed)
    out = []
    for _ in range(count):
        if kind == "phi0":
            out.append(torch.randn(S["phi0"].shape, generator=gen, dtype=torch.float64, device="cuda"))
        else:
            v = torch.randn(S["q"].shape, generator=gen, dtype=torch.float64, device="cuda")
            v[..., 0] = 0.0
            out.append(v)
    return out


def test_central_differences_16_directions(big):
    """16 seeded directions, alternating phi0 and velocity (as the benchmark's
    adjoint check draws them).  Each is tried at the configured step 1e-6; a
    direction whose difference quotients at h and h/2 disagree (by more than
    1e-3 relative) crossed a branch point of the piecewise-smooth forward map
    and is retried at 1e-8.  Every direction must be scored at one of the two
    steps, within 1e-4 of the adjoint."""
    S, b, eps, target = big["S"], big["b"], big["eps"], big["target"]
    loss = lambda p, q: float(((H(_forward(b, p, q), eps) - H(target, eps)) ** 2).sum())  # noqa: E731
    gen = torch.Generator(device="cuda").manual_seed(7)
    rows, worst = [], 0.0
    for d in range(16):
        kind = "phi0" if d % 2 == 0 else "q"
        v = torch.randn(S["phi0"].shape if kind == "phi0" else S["q"].shape, generator=gen, dtype=torch.float64,
                        device="cuda")
        if kind == "phi0":
            f = lambda t: loss(S["phi0"] + t * v, S["q"])  # noqa: E731
            an = float((big["gphi"] * v).sum())
        else:
            v[..., 0] = 0.0
            f = lambda t: loss(S["phi0"], S["q"] + t * v)  # noqa: E731
            an = float((big["gq"] * v).sum())
        used = None
        for h in (1e-6, 1e-8):
            fd1, fd2 = _fd(f, h)
            if abs(fd1 - fd2) <= 1e-3 * max(abs(fd1), abs(fd2)):
                used = h
                break
        assert used is not None, (d, kind, fd1, fd2)
        err = abs(an - fd1) / abs(fd1)
        rows.append("%s h=%g err=%.1e" % (kind, used, err))
        worst = max(worst, err)
    print("central differences (phi0 at 1e-6 crosses the band edge of a later step, see the module note): "
          + "; ".join(rows))
    assert worst <= 1e-4


def test_frozen_sign_field_is_exact_away_from_the_band_edge(lib_built):
    """A level set with no interface (phi >= 2 eps everywhere over the run,
    not a distance function, so the reinitialisation changes it): the sign
    field is +1 everywhere, no node is pinned, and every direction's
    difference quotient at 1e-6 matches the adjoint (the quotients at h and
    h/2 agree: no branch point is crossed)."""
    def bowl(case):
        # the minimum off the grid's symmetry planes: a bowl centred between
        # two nodes would make a one-sided difference exactly zero there, a
        # switch of the Godunov selection at the unperturbed state
        X, Y, Z = case.x, case.y, case.z
        return np.asfortranarray(0.2 + 1.5 * ((X - 0.437) ** 2 + (Y - 0.561) ** 2 + 0.5 * (Z - 0.509) ** 2))

    S = _setup(32, phi0=bowl)
    eps = S["case"].params.epslsm
    assert float(S["phi0"].min()) >= 2 * eps
    b = _batch(S, "fp64")
    n = 10
    phiT = _forward(b, S["phi0"], S["q"], n)
    assert float(phiT.min()) >= 2 * eps
    gen = torch.Generator(device="cuda").manual_seed(3)
    w = torch.randn(S["phi0"].shape, generator=gen, dtype=torch.float64, device="cuda")
    gphi, gq = _adjoint(b, S["phi0"], S["q"], lambda p: w, nsteps=n, ck=4)
    worst = 0.0
    for kind, seed in (("phi0", 11), ("q", 12)):
        for v in _directions(S, kind, 6, seed):
            if kind == "phi0":
                f = lambda t: float((_forward(b, S["phi0"] + t * v, S["q"], n) * w).sum())  # noqa: E731
                an = float((gphi * v).sum())
            else:
                f = lambda t: float((_forward(b, S["phi0"], S["q"] + t * v, n) * w).sum())  # noqa: E731
                an = float((gq * v).sum())
            fd1, fd2 = _fd(f, 1e-6)
            assert abs(fd1 - fd2) <= 1e-5 * max(abs(fd1), abs(fd2)), (kind, fd1, fd2)
            worst = max(worst, abs(an - fd1) / abs(fd1))
    b.close()
    print("no band edge: worst relative error over 12 directions at h = 1e-6: %.2e" % worst)
    assert worst <= 1e-5


def test_fp32_gradient_follows_fp64(big):
    S = big["S"]
    b32 = _batch(S, "fp32")
    g32phi, g32q = _adjoint(b32, S["phi0"], S["q"], big["seed"])
    b32.close()
    e_phi, e_q = _rel(g32phi, big["gphi"]), _rel(g32q, big["gq"])
    print("FP32 vs FP64 gradient: phi0 %.2e, q %.2e" % (e_phi, e_q))
    assert e_phi <= 1e-4 and e_q <= 1e-4
