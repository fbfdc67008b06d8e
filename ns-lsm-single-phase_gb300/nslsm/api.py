"""Python mirror of the reference's level-set routines over the C-ABI.

Each method carries the name and argument meaning of the Fortran routine it
replaces (see include/lsm_c.h for the file:line of every routine) and calls
liblsm_gb300.so.  Arrays may be

  * numpy arrays on the host, Fortran-ordered with shape (ni, nj, nk), vector
    fields (3, ni, nj, nk), q (4, ni, nj, nk) -- the reference's own layout;
  * torch CUDA tensors, C-contiguous with the reversed shape (nk, nj, ni),
    vector fields (nk, nj, ni, 3), q (nk, nj, ni, 4) -- the same bytes.

Outputs are allocated like the first array argument.  Host arrays are staged
through the library's device pool; CUDA tensors are used in place on torch's
current stream.  Errors raise `LsmError` with the library's status code.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .params import LsmParams

try:  # torch is optional for host-array use
    import torch
except Exception:  # pragma: no cover
    torch = None


class Grid:
    """Python mirror of struct lsm_grid: Fortran bounds (il:iu, jl:ju, kl:ku)."""

    def __init__(self, ni: int, nj: int, nk: int, igp: int = 0, jgp: int = 0, kgp: int = 0,
                 physical: Sequence[int] = (1, 1, 1, 1, 1, 1), dc: float = 1.0, de: float = 1.0,
                 dz: float = 1.0, il: int = 1, jl: int = 1, kl: int = 1):
        self.ni, self.nj, self.nk = int(ni), int(nj), int(nk)
        self.igp, self.jgp, self.kgp = igp, jgp, kgp
        self.physical = tuple(int(p) for p in physical)
        self.dc, self.de, self.dz = dc, de, dz
        self.il, self.jl, self.kl = il, jl, kl

    @property
    def shape(self) -> Tuple[int, int, int]:
        return (self.ni, self.nj, self.nk)

    @property
    def n(self) -> int:
        return self.ni * self.nj * self.nk

    def to_c(self) -> _lib.LsmGrid:
        g = _lib.LsmGrid()
        g.il, g.iu = self.il, self.il + self.ni - 1
        g.jl, g.ju = self.jl, self.jl + self.nj - 1
        g.kl, g.ku = self.kl, self.kl + self.nk - 1
        g.igp, g.jgp, g.kgp = self.igp, self.jgp, self.kgp
        g.dc, g.de, g.dz = self.dc, self.de, self.dz
        for f in range(6):
            g.physical_face[f] = self.physical[f]
        return g


def _is_torch(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor)


def _addr(a, grid: Grid, comps: int, dtype) -> Optional[int]:
    """Raw address of an array after checking its layout and size."""
    if a is None:
        return None
    n = grid.n * comps
    if _is_torch(a):
        want = torch.float64 if dtype == np.float64 else torch.int32
        if a.dtype != want or not a.is_contiguous() or a.numel() != n:
            raise ValueError(f"tensor must be contiguous {want} with {n} elements")
        return a.data_ptr()
    if not isinstance(a, np.ndarray) or a.dtype != dtype or a.size != n or not a.flags.f_contiguous:
        raise ValueError(f"array must be Fortran-contiguous {np.dtype(dtype)} with {n} elements")
    return a.ctypes.data


def _new(like, grid: Grid, comps: int = 1, dtype=np.float64):
    if _is_torch(like):
        tdt = torch.float64 if dtype == np.float64 else torch.int32
        shape = (grid.nk, grid.nj, grid.ni) + ((comps,) if comps > 1 else ())
        return torch.zeros(shape, dtype=tdt, device=like.device)
    shape = ((comps,) if comps > 1 else ()) + grid.shape
    return np.zeros(shape, dtype=dtype, order="F")


class LevelSet:
    """One library handle (device + stream + device pool)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        self.lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self.lib.lsm_create(C.byref(h), int(device), stream), "lsm_create")
        self.h = h
        self.device = device
        self._cb = None

    def close(self) -> None:
        if self.h:
            self.lib.lsm_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream: Optional[int]) -> None:
        _lib.check(self.lib.lsm_set_stream(self.h, stream), "lsm_set_stream", self.h)

    def set_exchange_callback(self, fn) -> None:
        """fn(field_device_ptr: int, grid) -> int, called where the reference
        calls rhs_exchng3_3d."""
        if fn is None:
            self._cb = None
            self.lib.lsm_set_exchange_callback(self.h, _lib.EXCHANGE_FN(), None)
            return

        def tramp(user, field, g):
            return int(fn(field, g.contents))

        self._cb = _lib.EXCHANGE_FN(tramp)
        _lib.check(self.lib.lsm_set_exchange_callback(self.h, self._cb, None), "exchange", self.h)

    @property
    def launches(self) -> int:
        return int(self.lib.lsm_kernel_launch_count(self.h))

    def _sync_stream(self, *arrays) -> None:
        if any(_is_torch(a) and a.is_cuda for a in arrays if a is not None):
            self.set_stream(torch.cuda.current_stream().cuda_stream)

    def _call(self, name, *args):
        _lib.check(getattr(self.lib, name)(self.h, *args), name, self.h)

    # ---------------------------------------------------------------- A0
    def levelsetmethod(self, grid: Grid, p: LsmParams, q, csi, eta, zet, aj, phi, phi_n, x, y, z,
                       iteraciontiempo: int) -> np.ndarray:
        """levelsetmethod: advance phi in place; returns the pre-advection
        volumes (K-tetrahedra, second tetrahedra, bulk, total)."""
        self._sync_stream(phi)
        vols = np.zeros(4)
        g, cp = grid.to_c(), p.to_c()
        self._call("lsm_levelsetmethod", C.byref(g), C.byref(cp), _addr(q, grid, 4, np.float64),
                   _addr(csi, grid, 3, np.float64), _addr(eta, grid, 3, np.float64),
                   _addr(zet, grid, 3, np.float64), _addr(aj, grid, 1, np.float64),
                   _addr(phi, grid, 1, np.float64), _addr(phi_n, grid, 1, np.float64),
                   _addr(x, grid, 1, np.float64), _addr(y, grid, 1, np.float64),
                   _addr(z, grid, 1, np.float64), int(iteraciontiempo), vols.ctypes.data)
        return vols

    def convergence_volume(self) -> float:
        """ConvergenceVolume of the last levelsetmethod call
        (src/levelsetmethod.F90:245-264): the pre-advection total minus the
        K- and second-tetrahedra volumes of the advected phi when
        GlobalMassCorrection is set, else the pre-advection total."""
        v = C.c_double(0.0)
        self._call("lsm_convergence_volume", C.byref(v))
        return v.value

    # ---------------------------------------------------------------- A1
    def rhs_contra_j(self, grid: Grid, q, csi, eta, zet, aj):
        self._sync_stream(q)
        u = _new(aj, grid, 3)
        g = grid.to_c()
        self._call("lsm_rhs_contra_j", C.byref(g), _addr(q, grid, 4, np.float64),
                   _addr(csi, grid, 3, np.float64), _addr(eta, grid, 3, np.float64),
                   _addr(zet, grid, 3, np.float64), _addr(aj, grid, 1, np.float64), _addr(u, grid, 3, np.float64))
        return u

    # ----------------------------------------------------------- A2 / A7
    def calc_rh_ad_weno3(self, grid: Grid, phi, ucn, mask=None):
        return self._rh(grid, "lsm_calc_rh_ad_weno3", phi, ucn, mask)

    def calc_rh_ad(self, grid: Grid, phi, ucn, mask=None):
        return self._rh(grid, "lsm_calc_rh_ad", phi, ucn, mask)

    def _rh(self, grid, name, phi, ucn, mask):
        self._sync_stream(phi)
        rh = _new(phi, grid)
        g = grid.to_c()
        self._call(name, C.byref(g), _addr(phi, grid, 1, np.float64), _addr(ucn, grid, 3, np.float64),
                   _addr(mask, grid, 1, np.int32), _addr(rh, grid, 1, np.float64))
        return rh

    # ---------------------------------------------------------------- A4
    def ad_rktvd3(self, grid: Grid, p: LsmParams, phi_n, ucn, aj, mask=None):
        self._sync_stream(phi_n)
        out = _new(phi_n, grid)
        g, cp = grid.to_c(), p.to_c()
        self._call("lsm_ad_rktvd3", C.byref(g), C.byref(cp), _addr(out, grid, 1, np.float64),
                   _addr(phi_n, grid, 1, np.float64), _addr(mask, grid, 1, np.int32),
                   _addr(ucn, grid, 3, np.float64), _addr(aj, grid, 1, np.float64))
        return out

    # ---------------------------------------------------------------- A5
    def bcond_lsm(self, grid: Grid, p: LsmParams, phi) -> None:
        self._sync_stream(phi)
        g, cp = grid.to_c(), p.to_c()
        self._call("lsm_bcond_lsm", C.byref(g), C.byref(cp), _addr(phi, grid, 1, np.float64))

    # ----------------------------------------------------------- R0 - R3
    def calc_sign_ini(self, grid: Grid, phi0, csi, eta, zet, epslsm: float, M_Sphi0: int = 1):
        self._sync_stream(phi0)
        s, n = _new(phi0, grid), _new(phi0, grid)
        g = grid.to_c()
        self._call("lsm_calc_sign_ini", C.byref(g), _addr(phi0, grid, 1, np.float64),
                   _addr(csi, grid, 3, np.float64), _addr(eta, grid, 3, np.float64),
                   _addr(zet, grid, 3, np.float64), float(epslsm), int(M_Sphi0),
                   _addr(s, grid, 1, np.float64), _addr(n, grid, 1, np.float64))
        return s, n

    def calc_rh_rn(self, grid: Grid, d, sign, csi, eta, zet):
        self._sync_stream(d)
        rh = _new(d, grid)
        g = grid.to_c()
        self._call("lsm_calc_rh_rn", C.byref(g), _addr(d, grid, 1, np.float64), _addr(sign, grid, 1, np.float64),
                   _addr(csi, grid, 3, np.float64), _addr(eta, grid, 3, np.float64),
                   _addr(zet, grid, 3, np.float64), _addr(rh, grid, 1, np.float64))
        return rh

    def calc_lambda_rn(self, grid: Grid, p: LsmParams, phi0, normgrad0, d, time_step: float):
        self._sync_stream(d)
        lam = _new(d, grid)
        g, cp = grid.to_c(), p.to_c()
        self._call("lsm_calc_lambda_rn", C.byref(g), C.byref(cp), _addr(phi0, grid, 1, np.float64),
                   _addr(normgrad0, grid, 1, np.float64), _addr(d, grid, 1, np.float64), float(time_step),
                   _addr(lam, grid, 1, np.float64))
        return lam

    def reinitialization(self, grid: Grid, p: LsmParams, phi0, csi, eta, zet):
        self._sync_stream(phi0)
        out = _new(phi0, grid)
        g, cp = grid.to_c(), p.to_c()
        self._call("lsm_reinitialization", C.byref(g), C.byref(cp), _addr(phi0, grid, 1, np.float64),
                   _addr(csi, grid, 3, np.float64), _addr(eta, grid, 3, np.float64),
                   _addr(zet, grid, 3, np.float64), _addr(out, grid, 1, np.float64))
        return out

    # ------------------------------------------------------------ L0
    def calc_normgrad_d(self, grid: Grid, p: LsmParams, phi_rn, phizero, csi, eta, zet):
        self._sync_stream(phi_rn)
        out = _new(phi_rn, grid)
        g, cp = grid.to_c(), p.to_c()
        self._call("lsm_calc_normgrad_d", C.byref(g), C.byref(cp), _addr(phi_rn, grid, 1, np.float64),
                   _addr(phizero, grid, 1, np.float64), _addr(csi, grid, 3, np.float64),
                   _addr(eta, grid, 3, np.float64), _addr(zet, grid, 3, np.float64), _addr(out, grid, 1, np.float64))
        return out

    def reinitialisation_test2(self, grid: Grid, p: LsmParams, phizero, csi, eta, zet):
        """-> (phi reinitialised, pseudo-time iterations run)"""
        self._sync_stream(phizero)
        out = _new(phizero, grid)
        g, cp = grid.to_c(), p.to_c()
        it = C.c_int(0)
        self._call("lsm_reinitialisation_test2", C.byref(g), C.byref(cp), _addr(phizero, grid, 1, np.float64),
                   _addr(csi, grid, 3, np.float64), _addr(eta, grid, 3, np.float64),
                   _addr(zet, grid, 3, np.float64), _addr(out, grid, 1, np.float64), C.byref(it))
        return out, it.value

    def geometric_reinitialisation(self, grid: Grid, p: LsmParams, phizero, x, y, z, total_water_volume: float,
                                   phicorrected):
        """geometric_reinitialisation (the hybrid path): -> (phicorrected, InterfaceNodesID, info dict).
        `phicorrected` is not modified; nodes away from the interface keep its values."""
        self._sync_stream(phizero)
        out = _new(phizero, grid)
        if _is_torch(out):
            out.copy_(phicorrected)
            self._sync_stream(out)
        else:
            out[...] = phicorrected
        ids = _new(phizero, grid, dtype=np.int32)
        g, cp = grid.to_c(), p.to_c()
        info = _lib.LsmGeomInfo()
        self._call("lsm_geometric_reinitialisation", C.byref(g), C.byref(cp), _addr(phizero, grid, 1, np.float64),
                   _addr(x, grid, 1, np.float64), _addr(y, grid, 1, np.float64), _addr(z, grid, 1, np.float64),
                   float(total_water_volume), _addr(out, grid, 1, np.float64), _addr(ids, grid, 1, np.int32),
                   C.byref(info))
        return out, ids, {f: getattr(info, f) for f, _ in _lib.LsmGeomInfo._fields_}

    # ------------------------------------------------------------ N1 - N3
    def narrowband(self, grid: Grid, p: LsmParams, phi_n):
        self._sync_stream(phi_n)
        nb = _new(phi_n, grid, dtype=np.int32)
        g, cp = grid.to_c(), p.to_c()
        self._call("lsm_narrowband", C.byref(g), C.byref(cp), _addr(phi_n, grid, 1, np.float64),
                   _addr(nb, grid, 1, np.int32))
        return nb

    def get_gfm_list(self, grid: Grid, p: LsmParams, phi) -> np.ndarray:
        """(count, 3) int32 array of Fortran (i, j, k), in k-j-i order."""
        self._sync_stream(phi)
        g, cp = grid.to_c(), p.to_c()
        cnt = C.c_int(0)
        self._call("lsm_get_gfm_list", C.byref(g), C.byref(cp), _addr(phi, grid, 1, np.float64), C.byref(cnt),
                   None, 0)
        n = cnt.value
        lst = np.zeros((max(n, 1), 3), dtype=np.int32, order="F")
        self._call("lsm_get_gfm_list", C.byref(g), C.byref(cp), _addr(phi, grid, 1, np.float64), C.byref(cnt),
                   lst.ctypes.data, max(n, 1))
        return lst[:n]

    # ---------------------------------------------------------------- V1
    def total_water_volume(self, grid: Grid, phi, x, y, z, with_nodes: bool = False):
        self._sync_stream(phi)
        vols = np.zeros(4)
        adv = _new(phi, grid, dtype=np.int32) if with_nodes else None
        g = grid.to_c()
        self._call("lsm_total_water_volume", C.byref(g), _addr(phi, grid, 1, np.float64),
                   _addr(x, grid, 1, np.float64), _addr(y, grid, 1, np.float64), _addr(z, grid, 1, np.float64),
                   vols.ctypes.data, _addr(adv, grid, 1, np.int32))
        return (vols, adv) if with_nodes else vols

    def cell_water_volumes(self, grid: Grid, phi, x, y, z):
        self._sync_stream(phi)
        cv = _new(phi, grid)
        g = grid.to_c()
        self._call("lsm_cell_water_volumes", C.byref(g), _addr(phi, grid, 1, np.float64),
                   _addr(x, grid, 1, np.float64), _addr(y, grid, 1, np.float64), _addr(z, grid, 1, np.float64),
                   _addr(cv, grid, 1, np.float64))
        return cv

    # ---------------------------------------------------------------- M0
    def mg_metrics(self, grid: Grid, x, y, z):
        self._sync_stream(x)
        csi, eta, zet, aj = _new(x, grid, 3), _new(x, grid, 3), _new(x, grid, 3), _new(x, grid)
        g = grid.to_c()
        self._call("lsm_mg_metrics", C.byref(g), _addr(x, grid, 1, np.float64), _addr(y, grid, 1, np.float64),
                   _addr(z, grid, 1, np.float64), _addr(csi, grid, 3, np.float64),
                   _addr(eta, grid, 3, np.float64), _addr(zet, grid, 3, np.float64),
                   _addr(aj, grid, 1, np.float64))
        return csi, eta, zet, aj


def write_total_water_volume(volume: float, path: Optional[str] = None) -> None:
    """WriteTotalWaterVolume: append one list-directed REAL(8) line."""
    lib = _lib.load()
    _lib.check(lib.lsm_write_total_water_volume(float(volume), None if path is None else path.encode()),
               "lsm_write_total_water_volume")
