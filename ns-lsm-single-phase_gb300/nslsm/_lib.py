"""ctypes binding of liblsm_gb300.so (the C-ABI declared in include/lsm_c.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback in this package.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LSM_OK = 0
LSM_ERR_NULL = 1
LSM_ERR_BAD_SHAPE = 2
LSM_ERR_BAD_PARAM = 3
LSM_ERR_UNSUPPORTED = 4
LSM_ERR_NONFINITE = 5
LSM_ERR_NEGATIVE_VOLUME = 6
LSM_ERR_MIXED_MEMORY = 7
LSM_ERR_CAPACITY = 8
LSM_ERR_CUDA = 9
LSM_ERR_NO_DEVICE = 10


class LsmGrid(C.Structure):
    """struct lsm_grid"""
    _fields_ = [("il", C.c_int), ("iu", C.c_int), ("jl", C.c_int), ("ju", C.c_int),
                ("kl", C.c_int), ("ku", C.c_int), ("igp", C.c_int), ("jgp", C.c_int),
                ("kgp", C.c_int), ("dc", C.c_double), ("de", C.c_double), ("dz", C.c_double),
                ("physical_face", C.c_int * 6)]


class LsmParams(C.Structure):
    """struct lsm_params"""
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


class LsmGeomInfo(C.Structure):
    """struct lsm_geom_info"""
    _fields_ = [("nnodes", C.c_int), ("ntetrahedra", C.c_int), ("nsecond", C.c_int),
                ("newton_iterations", C.c_int), ("newton_converged", C.c_int), ("C", C.c_double)]


class LsmBatchInstance(C.Structure):
    """struct lsm_batch_instance"""
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("dt", C.c_double), ("dtau", C.c_double),
                ("eps", C.c_double)]


class LsmBatchConfig(C.Structure):
    """struct lsm_batch_config"""
    _fields_ = [("RNitermax", C.c_int), ("btype_lsm", C.c_int * 6), ("BigPhi", C.c_double),
                ("use_graph", C.c_int), ("autotune", C.c_int), ("shape", C.c_int),
                ("precision", C.c_int), ("adjoint_mode", C.c_int), ("mass_correction", C.c_int)]


EXCHANGE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.POINTER(LsmGrid))

_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_G = C.POINTER(LsmGrid)
_P = C.POINTER(LsmParams)

# name -> (restype, argtypes); arrays are passed as raw addresses (host or device)
SIGNATURES = {
    "lsm_params_default": (None, [_P]),
    "lsm_create": (_i, [C.POINTER(_vp), _i, _vp]),
    "lsm_destroy": (_i, [_vp]),
    "lsm_set_stream": (_i, [_vp, _vp]),
    "lsm_set_exchange_callback": (_i, [_vp, EXCHANGE_FN, _vp]),
    "lsm_status_string": (C.c_char_p, [_i]),
    "lsm_last_error": (C.c_char_p, [_vp]),
    "lsm_kernel_launch_count": (C.c_longlong, [_vp]),
    "lsm_levelsetmethod": (_i, [_vp, _G, _P] + [_vp] * 10 + [_i, _vp]),
    "lsm_rhs_contra_j": (_i, [_vp, _G] + [_vp] * 6),
    "lsm_calc_rh_ad_weno3": (_i, [_vp, _G] + [_vp] * 4),
    "lsm_calc_rh_ad": (_i, [_vp, _G] + [_vp] * 4),
    "lsm_ad_rktvd3": (_i, [_vp, _G, _P] + [_vp] * 5),
    "lsm_bcond_lsm": (_i, [_vp, _G, _P, _vp]),
    "lsm_calc_sign_ini": (_i, [_vp, _G] + [_vp] * 4 + [_d, _i, _vp, _vp]),
    "lsm_calc_rh_rn": (_i, [_vp, _G] + [_vp] * 6),
    "lsm_calc_lambda_rn": (_i, [_vp, _G, _P, _vp, _vp, _vp, _d, _vp]),
    "lsm_reinitialization": (_i, [_vp, _G, _P] + [_vp] * 5),
    "lsm_calc_normgrad_d": (_i, [_vp, _G, _P] + [_vp] * 6),
    "lsm_reinitialisation_test2": (_i, [_vp, _G, _P] + [_vp] * 5 + [C.POINTER(_i)]),
    "lsm_narrowband": (_i, [_vp, _G, _P, _vp, _vp]),
    "lsm_total_water_volume": (_i, [_vp, _G] + [_vp] * 6),
    "lsm_cell_water_volumes": (_i, [_vp, _G] + [_vp] * 5),
    "lsm_get_gfm_list": (_i, [_vp, _G, _P, _vp, C.POINTER(_i), _vp, _i]),
    "lsm_write_total_water_volume": (_i, [_d, C.c_char_p]),
    "lsm_convergence_volume": (_i, [_vp, C.POINTER(C.c_double)]),
    "lsm_geometric_reinitialisation": (_i, [_vp, _G, _P] + [_vp] * 4 + [_d, _vp, _vp, C.POINTER(LsmGeomInfo)]),
    "lsm_mg_metrics": (_i, [_vp, _G] + [_vp] * 7),
    "lsm_total_water_volume_noalloc": (_i, [_G] + [_vp] * 6),
    "lsm_batch_create": (_i, [C.POINTER(_vp), _i, _vp, _i, C.POINTER(LsmBatchInstance),
                              C.POINTER(LsmBatchConfig)]),
    "lsm_batch_destroy": (_i, [_vp]),
    "lsm_batch_set_geometry": (_i, [_vp, _i] + [_vp] * 6),
    "lsm_batch_set_velocity": (_i, [_vp, _i, _vp]),
    "lsm_batch_set_phi": (_i, [_vp, _i, _vp]),
    "lsm_batch_get_phi": (_i, [_vp, _i, _vp]),
    "lsm_batch_set_velocities": (_i, [_vp, C.POINTER(_vp)]),
    "lsm_batch_get_phis": (_i, [_vp, C.POINTER(_vp)]),
    "lsm_batch_step": (_i, [_vp, _i, _vp]),
    "lsm_batch_water_volume": (_i, [_vp, _vp]),
    "lsm_batch_set_mass_target": (_i, [_vp, _i, _d]),
    "lsm_batch_mass_state": (_i, [_vp, _vp]),
    "lsm_batch_forward_record": (_i, [_vp, _i, _i]),
    "lsm_batch_set_grad_phi": (_i, [_vp, _i, _vp]),
    "lsm_batch_backward": (_i, [_vp]),
    "lsm_batch_get_grad_phi0": (_i, [_vp, _i, _vp]),
    "lsm_batch_get_grad_velocity": (_i, [_vp, _i, _vp]),
    "lsm_batch_shape": (_i, [_vp] + [C.POINTER(_i)] * 4),
    "lsm_batch_nodes": (C.c_longlong, [_vp]),
    "lsm_batch_stage_kernel": (_i, [_vp]),
    "lsm_batch_launches_per_step": (_i, [_vp]),
    "lsm_batch_last_error": (C.c_char_p, [_vp]),
    "lsm_profile_enable": (_i, [_i]),
    "lsm_profile_reset": (_i, []),
    "lsm_profile_count": (_i, []),
    "lsm_profile_entry": (_i, [_i, C.c_char_p, _i, C.POINTER(C.c_longlong), C.POINTER(_d)]),
}

_LIB = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False):
    """Load liblsm_gb300.so once; raise if it is missing (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"{path} is not built; run nslsm.build.build() (no CPU fallback exists)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


class LsmError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: status {status} ({detail})")


def check(status: int, where: str, handle=None) -> None:
    if status != LSM_OK:
        lib = load()
        detail = (lib.lsm_last_error(handle) or b"").decode(errors="replace")
        raise LsmError(status, where, detail or lib.lsm_status_string(status).decode())


class KernelTimer:
    """Per-kernel CUDA-event timing inside the library (lsm_profile_*)."""

    def __init__(self):
        self.lib = load()

    def __enter__(self):
        self.lib.lsm_profile_reset()
        self.lib.lsm_profile_enable(1)
        return self

    def __exit__(self, *exc):
        self.lib.lsm_profile_enable(0)

    def read(self) -> dict:
        """{kernel name: (launches, total_ms)}"""
        out = {}
        buf = C.create_string_buffer(128)
        for i in range(self.lib.lsm_profile_count()):
            n = C.c_longlong(0)
            ms = C.c_double(0.0)
            check(self.lib.lsm_profile_entry(i, buf, 128, C.byref(n), C.byref(ms)), "lsm_profile_entry")
            out[buf.value.decode()] = (int(n.value), float(ms.value))
        return out
