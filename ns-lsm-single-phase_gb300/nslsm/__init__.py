"""GB300-native level-set transport step (NS-LSM-Single-Phase hot path).

    from nslsm import LevelSet, Grid, LsmParams
    ls = LevelSet(device=0)
    vols = ls.levelsetmethod(grid, params, q, csi, eta, zet, aj, phi, phi_n, x, y, z, it)

The compute path is liblsm_gb300.so (hand-written CUDA for sm_103a) behind the
C-ABI of include/lsm_c.h; this package is its Python mirror.
"""
from ._lib import LsmError, load
from .api import Grid, LevelSet, write_total_water_volume
from .build import build as build_library
from .params import LsmParams, read_ind3dmg_lsm

__all__ = ["LevelSet", "Grid", "LsmParams", "LsmError", "read_ind3dmg_lsm", "write_total_water_volume",
           "build_library", "load"]
