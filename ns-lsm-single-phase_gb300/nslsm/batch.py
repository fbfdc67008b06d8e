"""Batched level-set transport (include/lsm_batch.h) from Python.

    b = LevelSetBatch(instances, RNitermax=5, btype=(1,)*6, BigPhi=5.0)
    b.set_geometry(k, x, y, z, csi, eta, zet); b.set_velocity(k, q); b.set_phi(k, phi)
    vols = b.step(100)          # (ninst, 4) pre-advection volumes of the last step
    phi_k = b.get_phi(k)

    # adjoint: dL/dphi0 and dL/dq through `nsteps` steps
    b.forward_record(nsteps, checkpoint_every=4)
    b.set_grad_phi(k, dL_dphi_k); b.backward()
    g_phi0, g_q = b.get_grad_phi0(k), b.get_grad_velocity(k)

    # the same through torch.autograd
    outs = transport(b, nsteps, phi0_list, q_list)

    # FP64 mass correction towards each instance's target volume
    b = LevelSetBatch(instances, mass_correction=True)
    ...; b.set_mass_target(k, b.water_volume()[k, 3])

Arrays follow the same conventions as nslsm.api: numpy in the reference's
Fortran layout or CUDA tensors with the reversed shape.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import numpy as np

from . import _lib
from .api import _addr, _is_torch, Grid


def _torch_sync(*arrays) -> None:
    """The batch runs on its own stream: work torch has queued on its current
    stream for these tensors (producing an input, zero-filling an output)
    must finish before the library touches them."""
    for a in arrays:
        if a is not None and _is_torch(a) and a.is_cuda:
            import torch
            torch.cuda.current_stream(a.device).synchronize()
            return


class LevelSetBatch:
    def __init__(self, instances: Sequence[Tuple[int, int, int, float, float, float]], RNitermax: int = 5,
                 btype: Sequence[int] = (1, 1, 1, 1, 1, 1), BigPhi: float = 5.0, device: int = 0, stream=None,
                 use_graph: bool = True, autotune: bool = True, shape: int = 0, precision: str = "fp32",
                 adjoint_mode: str = "store", mass_correction: bool = False):
        """instances: (ni, nj, nk, dt, dtau, eps) per instance; precision "fp32" or "fp64";
        adjoint_mode "store" (recorded pseudo-steps keep their adjoint coefficients: 6 arrays each)
        or "recompute" (the reverse sweep re-derives them: 1 array each); mass_correction: after
        every step shift phi by C = (target - V) / (dV/dC) towards the targets of set_mass_target."""
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        if adjoint_mode not in ("store", "recompute"):
            raise ValueError("adjoint_mode must be 'store' or 'recompute'")
        self.lib = _lib.load()
        n = len(instances)
        arr = (_lib.LsmBatchInstance * n)()
        for k, (ni, nj, nk, dt, dtau, eps) in enumerate(instances):
            arr[k].ni, arr[k].nj, arr[k].nk = int(ni), int(nj), int(nk)
            arr[k].dt, arr[k].dtau, arr[k].eps = float(dt), float(dtau), float(eps)
        cfg = _lib.LsmBatchConfig()
        cfg.RNitermax = int(RNitermax)
        for f in range(6):
            cfg.btype_lsm[f] = int(btype[f])
        cfg.BigPhi = float(BigPhi)
        cfg.use_graph, cfg.autotune, cfg.shape = int(use_graph), int(autotune), int(shape)
        cfg.precision = 1 if precision == "fp64" else 0
        cfg.adjoint_mode = 0 if adjoint_mode == "store" else 1
        cfg.mass_correction = int(bool(mass_correction))
        self.mass_correction = bool(mass_correction)
        self.precision = precision
        self.adjoint_mode = adjoint_mode
        h = C.c_void_p()
        st = self.lib.lsm_batch_create(C.byref(h), int(device), stream, n, arr, C.byref(cfg))
        if st != 0:
            raise _lib.LsmError(st, "lsm_batch_create", "")
        self.h = h
        self.grids = [Grid(ni, nj, nk) for (ni, nj, nk, *_rest) in instances]
        self.ninst = n

    def close(self):
        if self.h:
            self.lib.lsm_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, st, where):
        if st != 0:
            raise _lib.LsmError(st, where, (self.lib.lsm_batch_last_error(self.h) or b"").decode())

    def set_geometry(self, k, x, y, z, csi, eta, zet):
        g = self.grids[k]
        _torch_sync(x, y, z, csi, eta, zet)
        self._chk(self.lib.lsm_batch_set_geometry(self.h, k, _addr(x, g, 1, np.float64), _addr(y, g, 1, np.float64),
                                                  _addr(z, g, 1, np.float64), _addr(csi, g, 3, np.float64),
                                                  _addr(eta, g, 3, np.float64), _addr(zet, g, 3, np.float64)),
                  "lsm_batch_set_geometry")

    def set_velocity(self, k, q):
        g = self.grids[k]
        _torch_sync(q)
        self._chk(self.lib.lsm_batch_set_velocity(self.h, k, _addr(q, g, 4, np.float64)), "lsm_batch_set_velocity")

    def set_velocities(self, qs):
        """Every instance's velocity in one call (qs[k]: instance k's q)."""
        if len(qs) != self.ninst:
            raise ValueError("one velocity array per instance")
        _torch_sync(*qs)
        ptrs = (C.c_void_p * self.ninst)(*[_addr(q, g, 4, np.float64) for q, g in zip(qs, self.grids)])
        self._chk(self.lib.lsm_batch_set_velocities(self.h, ptrs), "lsm_batch_set_velocities")

    def get_phis(self, outs):
        """Every instance's phi into outs[k] (Fortran-ordered numpy arrays or
        CUDA tensors of the reversed shape) in one call."""
        if len(outs) != self.ninst:
            raise ValueError("one output array per instance")
        _torch_sync(*outs)
        ptrs = (C.c_void_p * self.ninst)(*[_addr(o, g, 1, np.float64) for o, g in zip(outs, self.grids)])
        self._chk(self.lib.lsm_batch_get_phis(self.h, ptrs), "lsm_batch_get_phis")
        return outs

    def set_phi(self, k, phi):
        g = self.grids[k]
        _torch_sync(phi)
        self._chk(self.lib.lsm_batch_set_phi(self.h, k, _addr(phi, g, 1, np.float64)), "lsm_batch_set_phi")

    def get_phi(self, k, like=None):
        g = self.grids[k]
        if like is not None and _is_torch(like):
            import torch
            out = torch.zeros((g.nk, g.nj, g.ni), dtype=torch.float64, device=like.device)
            _torch_sync(out)
        else:
            out = np.zeros(g.shape, order="F")
        self._chk(self.lib.lsm_batch_get_phi(self.h, k, _addr(out, g, 1, np.float64)), "lsm_batch_get_phi")
        return out

    def step(self, nsteps: int = 1, volumes: bool = True):
        v = np.zeros((self.ninst, 4)) if volumes else None
        self._chk(self.lib.lsm_batch_step(self.h, int(nsteps), None if v is None else v.ctypes.data),
                  "lsm_batch_step")
        return v

    def water_volume(self):
        """(ninst, 4) water volumes (K, S, bulk, total) of the current phi."""
        v = np.zeros((self.ninst, 4))
        self._chk(self.lib.lsm_batch_water_volume(self.h, v.ctypes.data), "lsm_batch_water_volume")
        return v

    def set_mass_target(self, k, volume: float):
        """Target water volume of instance k for the mass correction (nan: none)."""
        self._chk(self.lib.lsm_batch_set_mass_target(self.h, int(k), float(volume)), "lsm_batch_set_mass_target")

    def mass_state(self):
        """(ninst, 4): the last step's volume before the correction V, slope dV/dC, shift C, target."""
        v = np.zeros((self.ninst, 4))
        self._chk(self.lib.lsm_batch_mass_state(self.h, v.ctypes.data), "lsm_batch_mass_state")
        return v

    # ------------------------------------------------------------ adjoint
    @staticmethod
    def adjoint_bytes(nodes: int, RNitermax: int, nsteps: int, checkpoint_every: int, precision: str = "fp32",
                      adjoint_mode: str = "store", mass_correction: bool = False) -> int:
        """Device bytes forward_record allocates for the adjoint state (padding ignored):
        N (ceil(nsteps / k) + k (5 + m + c R) + 9) elements, c = 6 (store) or 1 (recompute), m = 2
        with the mass correction (the pre-correction field and its interface-cell list per step,
        plus N 8-byte words of scratch)."""
        c = 6 if adjoint_mode == "store" else 1
        m = 2 if mass_correction else 0
        k = min(int(checkpoint_every), int(nsteps))
        arrays = -(-int(nsteps) // k) + k * (5 + m + c * int(RNitermax)) + 9
        return int(nodes) * arrays * (8 if precision == "fp64" else 4) + (8 * int(nodes) if m else 0)

    def forward_record(self, nsteps: int, checkpoint_every: int = 4):
        self._chk(self.lib.lsm_batch_forward_record(self.h, int(nsteps), int(checkpoint_every)),
                  "lsm_batch_forward_record")

    def set_grad_phi(self, k, grad):
        g = self.grids[k]
        _torch_sync(grad)
        self._chk(self.lib.lsm_batch_set_grad_phi(self.h, k, _addr(grad, g, 1, np.float64)), "lsm_batch_set_grad_phi")

    def backward(self):
        self._chk(self.lib.lsm_batch_backward(self.h), "lsm_batch_backward")

    def _out(self, k, ncomp, like):
        g = self.grids[k]
        if like is not None and _is_torch(like):
            import torch
            shp = (g.nk, g.nj, g.ni) + ((ncomp,) if ncomp > 1 else ())
            out = torch.zeros(shp, dtype=torch.float64, device=like.device)
            _torch_sync(out)
            return out
        return np.zeros(((ncomp,) if ncomp > 1 else ()) + g.shape, order="F")

    def get_grad_phi0(self, k, like=None):
        out = self._out(k, 1, like)
        self._chk(self.lib.lsm_batch_get_grad_phi0(self.h, k, _addr(out, self.grids[k], 1, np.float64)),
                  "lsm_batch_get_grad_phi0")
        return out

    def get_grad_velocity(self, k, like=None):
        out = self._out(k, 4, like)
        self._chk(self.lib.lsm_batch_get_grad_velocity(self.h, k, _addr(out, self.grids[k], 4, np.float64)),
                  "lsm_batch_get_grad_velocity")
        return out

    @property
    def nodes(self) -> int:
        return int(self.lib.lsm_batch_nodes(self.h))

    @property
    def stage_kernel(self) -> str:
        """RK stage kernel in use: "tma" (plane tiles staged by TMA copies) or "smem"."""
        return "tma" if self.lib.lsm_batch_stage_kernel(self.h) == 1 else "smem"

    @property
    def launches_per_step(self) -> int:
        return int(self.lib.lsm_batch_launches_per_step(self.h))

    @property
    def shape(self):
        i, x, y, z = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._chk(self.lib.lsm_batch_shape(self.h, C.byref(i), C.byref(x), C.byref(y), C.byref(z)), "shape")
        return i.value, (x.value, y.value, z.value)


def _transport_function():
    import torch

    class _Transport(torch.autograd.Function):
        """phi^0 (per instance), q (per instance) -> phi^nsteps through the
        batch's level-set steps; backward runs the hand-written adjoint."""

        @staticmethod
        def forward(ctx, batch, nsteps, ckpt, *tensors):
            n = batch.ninst
            phis, qs = tensors[:n], tensors[n:]
            for k in range(n):
                batch.set_velocity(k, qs[k].detach().contiguous())
                batch.set_phi(k, phis[k].detach().contiguous())
            batch.forward_record(nsteps, ckpt)
            ctx.batch = batch
            ctx.like = phis[0]
            return tuple(batch.get_phi(k, like=phis[k]) for k in range(n))

        @staticmethod
        def backward(ctx, *grads):
            b = ctx.batch
            for k, g in enumerate(grads):
                if g is None:
                    g = torch.zeros((b.grids[k].nk, b.grids[k].nj, b.grids[k].ni), dtype=torch.float64,
                                    device=ctx.like.device)
                b.set_grad_phi(k, g.detach().to(torch.float64).contiguous())
            b.backward()
            gphi = [b.get_grad_phi0(k, like=ctx.like) for k in range(b.ninst)]
            gq = [b.get_grad_velocity(k, like=ctx.like) for k in range(b.ninst)]
            return (None, None, None, *gphi, *gq)

    return _Transport


_TRANSPORT = None


def transport(batch: LevelSetBatch, nsteps: int, phi0, q, checkpoint_every: int = 4):
    """Differentiable batched transport: lists of CUDA float64 tensors phi0[k]
    (nk, nj, ni) and q[k] (nk, nj, ni, 4) -> list of phi^nsteps[k].  The
    geometry must already be set on `batch`; its state is overwritten."""
    global _TRANSPORT
    if _TRANSPORT is None:
        _TRANSPORT = _transport_function()
    outs = _TRANSPORT.apply(batch, int(nsteps), int(checkpoint_every), *phi0, *q)
    return list(outs)
