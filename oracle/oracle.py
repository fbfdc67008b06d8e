"""TEST INFRASTRUCTURE ONLY: ctypes binding of the CPU FP64 oracle.

The oracle (oracle/lsm_oracle.cpp) restates the level-set transport routines
of NS-LSM-Single-Phase in C++ with the reference's FP64 operation order.  It
is the checker for the CUDA path and the timed CPU baseline; the product
never imports this module.  Parity is pinned only by analytic known-answer
tests because the Fortran reference cannot be built here (parity unpinned
against the reference's own outputs).

Arrays are numpy float64 / int32 in Fortran order with the grid's shape
(ni, nj, nk); vector fields have shape (3, ni, nj, nk), q has (4, ni, nj, nk).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))


def build(quiet: bool = True) -> None:
    """Compile the serial and OpenMP oracle libraries (make -C oracle)."""
    out = subprocess.run(["make", "-C", _HERE, "-j2"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


class Grid(C.Structure):
    _fields_ = [("il", C.c_int), ("iu", C.c_int), ("jl", C.c_int), ("ju", C.c_int),
                ("kl", C.c_int), ("ku", C.c_int), ("igp", C.c_int), ("jgp", C.c_int),
                ("kgp", C.c_int), ("dc", C.c_double), ("de", C.c_double), ("dz", C.c_double),
                ("physical_face", C.c_int * 6)]


class Params(C.Structure):
    _fields_ = [("epslsm", C.c_double), ("numiter_lsm", C.c_int), ("delti_lsm", C.c_double),
                ("RNitermax", C.c_int), ("RNtimestep", C.c_double), ("RNfreq", C.c_int),
                ("btype_lsm", C.c_int * 6), ("bc_extrapolation_order", C.c_int),
                ("isnarrow", C.c_int), ("narrowcoef", C.c_double), ("orderAD", C.c_int),
                ("sussman_correction_method", C.c_int), ("call_levelsetmethod", C.c_int),
                ("call_reinitialisation", C.c_int), ("hybrid_reinitialisation", C.c_int),
                ("TotalVolumeComputation", C.c_int), ("GlobalMassCorrection", C.c_int),
                ("BigPhi", C.c_double), ("epsReinitialisation", C.c_double),
                ("M_Sphi0", C.c_int), ("reinit_scheme", C.c_int),
                ("write_global_volume", C.c_int), ("OrderReinitialisationBoundaries", C.c_int),
                ("ENOBCReinitialisation", C.c_int), ("ConvergenceToleranceGeomReini", C.c_double)]


def make_grid(ni, nj, nk, igp=0, jgp=0, kgp=0, physical=(1, 1, 1, 1, 1, 1), dc=1.0, de=1.0, dz=1.0):
    g = Grid()
    g.il, g.iu, g.jl, g.ju, g.kl, g.ku = 1, ni, 1, nj, 1, nk
    g.igp, g.jgp, g.kgp = igp, jgp, kgp
    g.dc, g.de, g.dz = dc, de, dz
    for f in range(6):
        g.physical_face[f] = int(physical[f])
    return g


def make_params(**kw):
    p = Params()
    p.epslsm = 0.0
    p.numiter_lsm = 1
    p.delti_lsm = 0.0
    p.RNitermax = 5
    p.RNtimestep = 0.0
    p.RNfreq = 1
    for f in range(6):
        p.btype_lsm[f] = 1
    p.bc_extrapolation_order = 1
    p.isnarrow = 1
    p.narrowcoef = 4.0
    p.orderAD = 1
    p.sussman_correction_method = 0
    p.call_levelsetmethod = 1
    p.call_reinitialisation = 1
    p.hybrid_reinitialisation = 0
    p.TotalVolumeComputation = 1
    p.GlobalMassCorrection = 0
    p.BigPhi = 5.0
    p.epsReinitialisation = 1e-3
    p.M_Sphi0 = 1
    p.reinit_scheme = 0
    p.write_global_volume = 0
    p.OrderReinitialisationBoundaries = 1
    p.ENOBCReinitialisation = 0
    p.ConvergenceToleranceGeomReini = 1.0e-9
    for k, v in kw.items():
        if k == "btype_lsm":
            for f in range(6):
                p.btype_lsm[f] = int(v[f])
        else:
            setattr(p, k, v)
    return p


_D = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_I = np.ctypeslib.ndpointer(dtype=np.int32, flags="F_CONTIGUOUS")
_GP = C.POINTER(Grid)
_PP = C.POINTER(Params)


def _opt_int(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


class Oracle:
    """One loaded oracle library (serial by default, or the OpenMP build)."""

    def __init__(self, omp: bool = False):
        name = "liblsm_oracle_omp.so" if omp else "liblsm_oracle.so"
        path = os.path.join(_HERE, name)
        if not os.path.exists(path):
            build()
        self.lib = C.CDLL(path)
        L = self.lib
        vp = C.c_void_p
        sig = {
            "oracle_rhs_contra_j": [_GP, _D, _D, _D, _D, _D, _D],
            "oracle_calc_rh_ad_weno3": [_GP, _D, _D, vp, _D],
            "oracle_calc_rh_ad": [_GP, _D, _D, vp, _D],
            "oracle_bcond_lsm": [_GP, _PP, _D],
            "oracle_ad_rktvd3": [_GP, _PP, _D, _D, vp, _D, _D],
            "oracle_calc_sign_ini": [_GP, _D, _D, _D, _D, C.c_double, C.c_int, _D, _D],
            "oracle_calc_rh_rn": [_GP, _D, _D, _D, _D, _D, _D],
            "oracle_calc_lambda_rn": [_GP, _PP, _D, _D, _D, C.c_double, _D],
            "oracle_reinitialization": [_GP, _PP, _D, _D, _D, _D, _D],
            "oracle_calc_normgrad_d": [_GP, _PP, _D, _D, _D, _D, _D, _D],
            "oracle_reinitialisation_test2": [_GP, _PP, _D, _D, _D, _D, _D, C.POINTER(C.c_int)],
            "oracle_narrowband": [_GP, _PP, _D, _I],
            "oracle_get_gfm_list": [_GP, _PP, _D, C.POINTER(C.c_int), vp, C.c_int],
            "oracle_total_water_volume": [_GP, _D, _D, _D, _D, _D, vp],
            "oracle_total_water_volume_par": [_GP, _D, _D, _D, _D, _D],
            "oracle_cell_water_volumes": [_GP, _D, _D, _D, _D, _D],
            "oracle_mg_metrics": [_GP, _D, _D, _D, _D, _D, _D, _D],
            "oracle_levelsetmethod": [_GP, _PP, _D, _D, _D, _D, _D, _D, _D, _D, _D, _D, C.c_int, _D],
            "oracle_geometric_reinitialisation": [_GP, _PP, _D, _D, _D, _D, C.c_double, _D, _I,
                                                  C.POINTER(C.c_int), C.POINTER(C.c_double)],
        }
        for fn, args in sig.items():
            f = getattr(L, fn)
            f.argtypes = args
            f.restype = C.c_int
        L.oracle_num_threads.restype = C.c_int

    @property
    def threads(self) -> int:
        return int(self.lib.oracle_num_threads())

    @staticmethod
    def _chk(st, name):
        if st != 0:
            raise RuntimeError(f"{name} returned status {st}")

    def rhs_contra_j(self, g, q, csi, eta, zet, aj):
        u = np.zeros((3,) + aj.shape, order="F")
        self._chk(self.lib.oracle_rhs_contra_j(C.byref(g), q, csi, eta, zet, aj, u), "contra")
        return u

    def calc_rh_ad_weno3(self, g, phi, ucn, mask=None):
        rh = np.zeros(phi.shape, order="F")
        self._chk(self.lib.oracle_calc_rh_ad_weno3(C.byref(g), phi, ucn, _opt_int(mask), rh), "weno3")
        return rh

    def calc_rh_ad(self, g, phi, ucn, mask=None):
        rh = np.zeros(phi.shape, order="F")
        self._chk(self.lib.oracle_calc_rh_ad(C.byref(g), phi, ucn, _opt_int(mask), rh), "upwind")
        return rh

    def bcond_lsm(self, g, p, phi):
        out = np.array(phi, order="F", copy=True)
        self._chk(self.lib.oracle_bcond_lsm(C.byref(g), C.byref(p), out), "bcond")
        return out

    def ad_rktvd3(self, g, p, phin, ucn, aj, mask=None):
        out = np.zeros(phin.shape, order="F")
        self._chk(self.lib.oracle_ad_rktvd3(C.byref(g), C.byref(p), out, phin, _opt_int(mask), ucn, aj), "rk3")
        return out

    def calc_sign_ini(self, g, phi0, csi, eta, zet, eps, M_Sphi0=1):
        s = np.zeros(phi0.shape, order="F")
        n = np.zeros(phi0.shape, order="F")
        self._chk(self.lib.oracle_calc_sign_ini(C.byref(g), phi0, csi, eta, zet, eps, M_Sphi0, s, n), "sign")
        return s, n

    def calc_rh_rn(self, g, d, s, csi, eta, zet):
        rh = np.zeros(d.shape, order="F")
        self._chk(self.lib.oracle_calc_rh_rn(C.byref(g), d, s, csi, eta, zet, rh), "rh_rn")
        return rh

    def calc_lambda_rn(self, g, p, phi0, ng, d, dt):
        lam = np.zeros(d.shape, order="F")
        self._chk(self.lib.oracle_calc_lambda_rn(C.byref(g), C.byref(p), phi0, ng, d, dt, lam), "lambda")
        return lam

    def reinitialization(self, g, p, phi0, csi, eta, zet):
        out = np.zeros(phi0.shape, order="F")
        self._chk(self.lib.oracle_reinitialization(C.byref(g), C.byref(p), phi0, csi, eta, zet, out), "reinit")
        return out

    def calc_normgrad_d(self, g, p, phi, phizero, csi, eta, zet):
        out = np.zeros(phi.shape, order="F")
        self._chk(self.lib.oracle_calc_normgrad_d(C.byref(g), C.byref(p), phi, phizero, csi, eta, zet, out),
                  "normgrad_d")
        return out

    def reinitialisation_test2(self, g, p, phizero, csi, eta, zet):
        """-> (phi reinitialised, pseudo-time iterations run)"""
        out = np.zeros(phizero.shape, order="F")
        it = C.c_int(0)
        self._chk(self.lib.oracle_reinitialisation_test2(C.byref(g), C.byref(p), phizero, csi, eta, zet, out,
                                                         C.byref(it)), "reinitialisation_test2")
        return out, it.value

    def narrowband(self, g, p, phin):
        nb = np.zeros(phin.shape, dtype=np.int32, order="F")
        self._chk(self.lib.oracle_narrowband(C.byref(g), C.byref(p), phin, nb), "narrowband")
        return nb

    def get_gfm_list(self, g, p, phi):
        cnt = C.c_int(0)
        self._chk(self.lib.oracle_get_gfm_list(C.byref(g), C.byref(p), phi, C.byref(cnt), None, 0), "gfm")
        n = cnt.value
        lst = np.zeros((max(n, 1), 3), dtype=np.int32, order="F")
        self._chk(self.lib.oracle_get_gfm_list(C.byref(g), C.byref(p), phi, C.byref(cnt),
                                               lst.ctypes.data_as(C.c_void_p), max(n, 1)), "gfm")
        return lst[:n]

    def total_water_volume(self, g, phi, x, y, z, with_nodes=False):
        v = np.zeros(4)
        adv = np.zeros(phi.shape, dtype=np.int32, order="F") if with_nodes else None
        self._chk(self.lib.oracle_total_water_volume(
            C.byref(g), phi, x, y, z, v, None if adv is None else adv.ctypes.data_as(C.c_void_p)), "volume")
        return (v, adv) if with_nodes else v

    def total_water_volume_par(self, g, phi, x, y, z):
        v = np.zeros(4)
        self._chk(self.lib.oracle_total_water_volume_par(C.byref(g), phi, x, y, z, v), "volume_par")
        return v

    def cell_water_volumes(self, g, phi, x, y, z):
        cv = np.zeros(phi.shape, order="F")
        self._chk(self.lib.oracle_cell_water_volumes(C.byref(g), phi, x, y, z, cv), "cellvol")
        return cv

    def mg_metrics(self, g, x, y, z):
        sh = x.shape
        csi = np.zeros((3,) + sh, order="F"); eta = np.zeros((3,) + sh, order="F")
        zet = np.zeros((3,) + sh, order="F"); aj = np.zeros(sh, order="F")
        self._chk(self.lib.oracle_mg_metrics(C.byref(g), x, y, z, csi, eta, zet, aj), "metrics")
        return csi, eta, zet, aj

    def geometric_reinitialisation(self, g, p, phi0, x, y, z, total_water_volume, phicorrected):
        """geometric_reinitialisation: returns (phicorrected, InterfaceNodesID, info dict)"""
        pc = np.array(phicorrected, order="F", copy=True)
        ids = np.zeros(phi0.shape, dtype=np.int32, order="F")
        ii = (C.c_int * 5)()
        cc = C.c_double(0.0)
        self._chk(self.lib.oracle_geometric_reinitialisation(C.byref(g), C.byref(p), phi0, x, y, z,
                                                             float(total_water_volume), pc, ids, ii, C.byref(cc)),
                  "geometric_reinitialisation")
        info = dict(nnodes=ii[0], ntetrahedra=ii[1], nsecond=ii[2], newton_iterations=ii[3],
                    newton_converged=ii[4], C=cc.value)
        return pc, ids, info

    def levelsetmethod(self, g, p, q, csi, eta, zet, aj, phi, phin, x, y, z, it):
        out = np.array(phi, order="F", copy=True)
        v = np.zeros(4)
        self._chk(self.lib.oracle_levelsetmethod(C.byref(g), C.byref(p), q, csi, eta, zet, aj, out, phin,
                                                 x, y, z, it, v), "levelsetmethod")
        return out, v
