"""FP64 PyTorch restatement of one batched level-set step (test infrastructure).

The forward is written with differentiable torch operations so that
torch.autograd gives an independent "tape" gradient for the hand-written
adjoint kernels of the batched path.  It follows the batched formulation:

  W_m      = dt (grad xi_m . u)                       (rhs_contra_j x dt)
  stage s  = c1 phi^n + c2 in - c3 sum_m W_m (Phi+ - Phi-)_m   (interior)
             WENO3 (GetWENO3Reconstruction, src/AdvectionMethods.F90:195-245),
             one-sided stencils forced on the first / last interior node
             (src/calc_RH_AD_WENO3.F90:201-245), then bcond_lsm
             (src/bcond_lsm.F90, faces i1, im, j1, jm, k1, km in order)
  sign     = Kang sign of the advected field with the lambda-corrected band
             frozen (s = 0 where |phi0| < eps and |grad phi0| > 0)
  reinit   = RNitermax pseudo-steps d - dtau s (|grad d|_G - 1)
             (src/calc_RH_RN.F90 Godunov norm), then bcond_lsm.

The upwind side of every WENO face, the Godunov max / clip selections, the
BigPhi switch and the sign field are evaluated on the forward values (torch
`where` passes the gradient through the selected branch only), which is the
same piecewise-smooth function the adjoint kernels differentiate.

Tensors are C-contiguous (nk, nj, ni); metrics are nine tensors ordered
csi_x, csi_y, csi_z, eta_x, ..., zet_z; q has shape (nk, nj, ni, 4).
"""
from __future__ import annotations

import math

import torch

_DIM = {0: 2, 1: 1, 2: 0}   # reference axis (i, j, k) -> torch dimension


def _shift(a: torch.Tensor, o: int, dim: int) -> torch.Tensor:
    """b[.., c, ..] = a[.., c + o, ..] along `dim`, zero outside."""
    n = a.shape[dim]
    pad = [0, 0] * a.dim()
    p = 2 * (a.dim() - 1 - dim)
    pad[p], pad[p + 1] = 2, 2
    ap = torch.nn.functional.pad(a, pad)
    return ap.narrow(dim, 2 + o, n)


def _rec3(fL, fC, fR):
    b0 = (fC - fR) * (fC - fR)
    b1 = (fL - fC) * (fL - fC)
    t0 = b0 + 1.0e-6
    t1 = b1 + 1.0e-6
    a0 = 2.0 * t1 * t1
    a1 = t0 * t0
    w0 = a0 / (a0 + a1)
    u1 = 1.5 * fC - 0.5 * fL
    return w0 * (0.5 * (fL + fR) - fC) + u1


def _coord(n, dim, ndim, device):
    shape = [1] * ndim
    shape[dim] = n
    return torch.arange(n, device=device).view(shape)


def _interior(shape, device):
    nk, nj, ni = shape
    m = torch.zeros(shape, dtype=torch.bool, device=device)
    m[1:-1, 1:-1, 1:-1] = True
    return m


def stage_rhs(phi, W):
    R = torch.zeros_like(phi)
    for ax in range(3):
        dim = _DIM[ax]
        n = phi.shape[dim]
        idx = _coord(n, dim, 3, phi.device)
        lo, hi = idx == 1, idx == n - 2
        m2 = torch.where(idx > 1, _shift(phi, -2, dim), torch.zeros_like(phi))
        p2 = torch.where(idx < n - 2, _shift(phi, 2, dim), torch.zeros_like(phi))
        m1, p1 = _shift(phi, -1, dim), _shift(phi, 1, dim)
        w = W[ax]
        up = w > 0
        fp = torch.where(up | hi, _rec3(m1, phi, p1), _rec3(p2, p1, phi))
        fm = torch.where(up & ~lo, _rec3(m2, m1, phi), _rec3(p1, phi, m1))
        R = R + w * (fp - fm)
    return torch.where(_interior(phi.shape, phi.device), R, torch.zeros_like(R))


def bcond(phi, btype, BigPhi):
    """bcond_lsm, faces in the reference's order, each from the current values."""
    for face in range(6):
        t = btype[face]
        if not (t in (0, 1) or (t == 2 and face == 1)):
            continue
        dim = _DIM[face >> 1]
        n = phi.shape[dim]
        b, n1, n2 = (0, 1, 2) if face % 2 == 0 else (n - 1, n - 2, n - 3)
        v1, v2 = phi.select(dim, n1), phi.select(dim, n2)
        if t == 0:
            val = v1
        elif t == 1:
            val = torch.where(v2.abs() >= BigPhi, v1, (4.0 / 3.0) * v1 - (1.0 / 3.0) * v2)
        else:
            val = 2.0 * v1 - v2
        phi = phi.clone()
        phi.select(dim, b).copy_(val)
    return phi


def _diffs(d):
    """one-sided differences per axis: (mas, men), physical faces take the one available"""
    mas, men = [], []
    for ax in range(3):
        dim = _DIM[ax]
        n = d.shape[dim]
        idx = _coord(n, dim, 3, d.device)
        fwd = _shift(d, 1, dim) - d
        bwd = d - _shift(d, -1, dim)
        mas.append(torch.where(idx < n - 1, fwd, bwd))
        men.append(torch.where(idx > 0, bwd, fwd))
    return mas, men


def godunov(d, M, s):
    mas, men = _diffs(d)
    acc = torch.zeros_like(d)
    pos = s > 0
    zero = torch.zeros_like(d)
    for x in range(3):
        bb = M[x] * men[0] + M[3 + x] * men[1] + M[6 + x] * men[2]
        ff = M[x] * mas[0] + M[3 + x] * mas[1] + M[6 + x] * mas[2]
        P = torch.where(pos, torch.where(bb > 0, bb, zero), torch.where(bb < 0, bb, zero))
        Q = torch.where(pos, torch.where(ff < 0, ff, zero), torch.where(ff > 0, ff, zero))
        acc = acc + torch.where(P * P >= Q * Q, P * P, Q * Q)
    safe = torch.where(acc > 0, acc, torch.ones_like(acc))
    return torch.where(acc > 0, torch.sqrt(safe), zero)


@torch.no_grad()
def sign_field(phi0, M, eps):
    g = godunov(phi0, M, torch.where(phi0 > 0, torch.ones_like(phi0), -torch.ones_like(phi0)))
    smooth = phi0 / eps - (1.0 / math.pi) * torch.sin(math.pi * phi0 / eps)
    s = torch.where((phi0 != 0) & (g > 0), torch.zeros_like(phi0), smooth)
    s = torch.where(phi0 <= -eps, -torch.ones_like(phi0), s)
    return torch.where(phi0 >= eps, torch.ones_like(phi0), s)


def step(phin, W, M, dtau, eps, R, btype, BigPhi):
    C = ((1.0, 0.0, 1.0), (0.75, 0.25, 0.25), (1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0))
    cur = phin
    for c1, c2, c3 in C:
        cur = bcond(c1 * phin + c2 * cur - c3 * stage_rhs(cur, W), btype, BigPhi)
    if R > 0:
        s = sign_field(cur.detach(), M, eps)
        d = cur
        for _ in range(R):
            d = torch.where(s == 0, d, d - dtau * s * (godunov(d, M, s) - 1.0))
        return bcond(d, btype, BigPhi)
    return bcond(cur, btype, BigPhi)


def contra(q, M, dt):
    u, v, w = q[..., 1], q[..., 2], q[..., 3]
    return [dt * (M[3 * m] * u + M[3 * m + 1] * v + M[3 * m + 2] * w) for m in range(3)]


def run(phi0, q, M, dt, dtau, eps, R, nsteps, btype=(1,) * 6, BigPhi=5.0):
    """phi^nsteps from phi0 with velocity q held fixed."""
    W = contra(q, M, dt)
    phi = phi0
    for _ in range(nsteps):
        phi = step(phi, W, M, dtau, eps, R, btype, BigPhi)
    return phi


def metrics_torch(csi, eta, zet, device="cpu"):
    """numpy (3, ni, nj, nk) Fortran metrics -> nine (nk, nj, ni) float64 tensors."""
    out = []
    for m in (csi, eta, zet):
        t = torch.from_numpy(m.T.copy()).to(device)   # (nk, nj, ni, 3)
        out += [t[..., c].contiguous() for c in range(3)]
    return out


def to_torch(a, device="cpu"):
    """numpy Fortran (ni, nj, nk[, ...]) or (c, ni, nj, nk) -> C-contiguous reversed-shape tensor."""
    return torch.from_numpy(a.T.copy()).to(device)
