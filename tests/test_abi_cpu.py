"""C-ABI checks that need no GPU: the library builds and loads, exports
every entry point declared in include/*.h, and its host-only functions
behave (parameter defaults, status strings, the GlobalVolume.txt writer,
the no-device error path)."""
import ctypes as C
import glob
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(lsm\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_reference_routines():
    names = _declared()
    for n in ("lsm_levelsetmethod", "lsm_ad_rktvd3", "lsm_calc_rh_ad_weno3", "lsm_calc_rh_ad",
              "lsm_rhs_contra_j", "lsm_bcond_lsm", "lsm_reinitialization", "lsm_calc_sign_ini",
              "lsm_calc_rh_rn", "lsm_calc_lambda_rn", "lsm_narrowband", "lsm_total_water_volume",
              "lsm_get_gfm_list", "lsm_write_total_water_volume"):
        assert n in names


def test_library_exports_every_declared_symbol(lib_built):
    lib = C.CDLL(lib_built)
    missing = [n for n in sorted(_declared()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_every_symbol(lib_built):
    from nslsm import _lib
    declared = _declared()
    bound = set(_lib.SIGNATURES)
    assert declared <= bound, declared - bound


def test_host_only_functions(lib_built, tmp_path):
    from nslsm import _lib
    lib = _lib.load()
    p = _lib.LsmParams()
    lib.lsm_params_default(C.byref(p))
    assert p.orderAD == 1 and p.RNitermax == 15 and p.BigPhi == 5.0 and p.M_Sphi0 == 1
    assert list(p.btype_lsm) == [1] * 6
    assert lib.lsm_status_string(_lib.LSM_ERR_NEGATIVE_VOLUME) == b"negative tetrahedron water volume"
    path = str(tmp_path / "GlobalVolume.txt")
    assert lib.lsm_write_total_water_volume(0.0128813727994583, path.encode()) == 0
    assert lib.lsm_write_total_water_volume(1.5e-3, path.encode()) == 0
    lines = open(path).read().splitlines()
    assert len(lines) == 2
    assert float(lines[0]) == pytest.approx(0.0128813727994583, rel=1e-15)
    assert float(lines[1]) == 1.5e-3


def test_no_device_is_an_error_not_a_crash(lib_built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from nslsm import _lib
    lib = _lib.load()
    h = C.c_void_p()
    st = lib.lsm_create(C.byref(h), 0, None)
    assert st == _lib.LSM_ERR_NO_DEVICE


def test_batch_create_validates_before_touching_a_device(lib_built):
    """Empty and malformed batches are rejected with their status codes
    (checked before any device call, so this runs without a GPU)."""
    from nslsm import _lib
    lib = _lib.load()
    h = C.c_void_p()
    cfg = _lib.LsmBatchConfig()
    cfg.RNitermax, cfg.BigPhi, cfg.use_graph, cfg.autotune = 5, 5.0, 1, 1
    for f in range(6):
        cfg.btype_lsm[f] = 1
    inst = (_lib.LsmBatchInstance * 2)()
    for k in range(2):
        inst[k].ni, inst[k].nj, inst[k].nk = 8, 8, 8
        inst[k].dt, inst[k].dtau, inst[k].eps = 1e-3, 1e-3, 1e-2
    assert lib.lsm_batch_create(C.byref(h), 0, None, 0, inst, C.byref(cfg)) == _lib.LSM_ERR_NULL
    inst[1].nk = 3                                          # below the 4-node minimum
    assert lib.lsm_batch_create(C.byref(h), 0, None, 2, inst, C.byref(cfg)) == _lib.LSM_ERR_BAD_SHAPE
    inst[1].nk = 8
    for field, bad in (("RNitermax", -1), ("precision", 2), ("adjoint_mode", 3)):
        setattr(cfg, field, bad)
        assert lib.lsm_batch_create(C.byref(h), 0, None, 2, inst, C.byref(cfg)) == _lib.LSM_ERR_BAD_PARAM, field
        setattr(cfg, field, 0 if field != "RNitermax" else 5)
    cfg.btype_lsm[3] = 7
    assert lib.lsm_batch_create(C.byref(h), 0, None, 2, inst, C.byref(cfg)) == _lib.LSM_ERR_BAD_PARAM


def test_batch_entry_points_reject_null_handles(lib_built):
    """Every batch entry point answers a null handle or array with its status
    code instead of touching a device (no GPU needed)."""
    from nslsm import _lib
    lib = _lib.load()
    h = C.c_void_p()
    cfg = _lib.LsmBatchConfig()
    cfg.RNitermax, cfg.BigPhi = 5, 5.0
    for f in range(6):
        cfg.btype_lsm[f] = 1
    cfg.mass_correction = 2
    inst = (_lib.LsmBatchInstance * 1)()
    inst[0].ni, inst[0].nj, inst[0].nk = 8, 8, 8
    inst[0].dt, inst[0].dtau, inst[0].eps = 1e-3, 1e-3, 1e-2
    assert lib.lsm_batch_create(C.byref(h), 0, None, 1, inst, C.byref(cfg)) == _lib.LSM_ERR_BAD_PARAM
    ptrs = (C.c_void_p * 1)()
    assert lib.lsm_batch_set_velocities(None, ptrs) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_get_phis(None, ptrs) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_set_velocity(None, 0, None) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_get_phi(None, 0, None) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_water_volume(None, None) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_set_mass_target(None, 0, 1.0) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_mass_state(None, None) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_step(None, 1, None) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_backward(None) == _lib.LSM_ERR_NULL
    assert lib.lsm_batch_stage_kernel(None) == -1
    assert lib.lsm_batch_launches_per_step(None) == 0
