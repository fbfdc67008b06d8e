"""Batched FP32 level-set transport (include/lsm_batch.h) from Python.

    b = LevelSetBatch(instances, RNitermax=5, btype=(1,)*6, BigPhi=5.0)
    b.set_geometry(k, x, y, z, csi, eta, zet); b.set_velocity(k, q); b.set_phi(k, phi)
    vols = b.step(100)          # (ninst, 4) pre-advection volumes of the last step
    phi_k = b.get_phi(k)

Arrays follow the same conventions as nslsm.api: numpy in the reference's
Fortran layout or CUDA tensors with the reversed shape.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence, Tuple

import numpy as np

from . import _lib
from .api import _addr, _is_torch, Grid


class LevelSetBatch:
    def __init__(self, instances: Sequence[Tuple[int, int, int, float, float, float]], RNitermax: int = 5,
                 btype: Sequence[int] = (1, 1, 1, 1, 1, 1), BigPhi: float = 5.0, device: int = 0, stream=None,
                 use_graph: bool = True, autotune: bool = True, shape: int = 0):
        """instances: (ni, nj, nk, dt, dtau, eps) per instance."""
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
        self._chk(self.lib.lsm_batch_set_geometry(self.h, k, _addr(x, g, 1, np.float64), _addr(y, g, 1, np.float64),
                                                  _addr(z, g, 1, np.float64), _addr(csi, g, 3, np.float64),
                                                  _addr(eta, g, 3, np.float64), _addr(zet, g, 3, np.float64)),
                  "lsm_batch_set_geometry")

    def set_velocity(self, k, q):
        g = self.grids[k]
        self._chk(self.lib.lsm_batch_set_velocity(self.h, k, _addr(q, g, 4, np.float64)), "lsm_batch_set_velocity")

    def set_phi(self, k, phi):
        g = self.grids[k]
        self._chk(self.lib.lsm_batch_set_phi(self.h, k, _addr(phi, g, 1, np.float64)), "lsm_batch_set_phi")

    def get_phi(self, k, like=None):
        g = self.grids[k]
        if like is not None and _is_torch(like):
            import torch
            out = torch.zeros((g.nk, g.nj, g.ni), dtype=torch.float64, device=like.device)
        else:
            out = np.zeros(g.shape, order="F")
        self._chk(self.lib.lsm_batch_get_phi(self.h, k, _addr(out, g, 1, np.float64)), "lsm_batch_get_phi")
        return out

    def step(self, nsteps: int = 1, volumes: bool = True):
        v = np.zeros((self.ninst, 4)) if volumes else None
        self._chk(self.lib.lsm_batch_step(self.h, int(nsteps), None if v is None else v.ctypes.data),
                  "lsm_batch_step")
        return v

    @property
    def nodes(self) -> int:
        return int(self.lib.lsm_batch_nodes(self.h))

    @property
    def launches_per_step(self) -> int:
        return int(self.lib.lsm_batch_launches_per_step(self.h))

    @property
    def shape(self):
        i, x, y, z = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self._chk(self.lib.lsm_batch_shape(self.h, C.byref(i), C.byref(x), C.byref(y), C.byref(z)), "shape")
        return i.value, (x.value, y.value, z.value)
