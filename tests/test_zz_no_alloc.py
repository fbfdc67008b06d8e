"""The allocation-free water-volume entry point (lsm_total_water_volume_noalloc).

Some callers of this library cannot call cudaMalloc: code that runs under
another framework's memory pool or allocator hooks that forbid raw device
allocations, or a real-time loop where an allocation's latency or failure is
not allowed.  They cannot create a handle, because a handle allocates its
device pool; this entry point takes device arrays and a stream, and keeps its
scratch in one fixed file-scope device array instead.  The test calls it
through the C-ABI twice in a row -- the second call must not be affected by
what the first one left in the shared array -- and compares each result with
the handle-based lsm_total_water_volume within the volume tolerance of the
other GPU tests (1e-12 normwise relative).  This file is collected last so a
failure here never hides the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()


def test_noalloc_volume_matches_handle_entry_point_on_consecutive_calls(ls):
    from nslsm import Grid, _lib
    lib = _lib.load()
    g, x, y, z, phi, _ = cases.curvilinear(40, 28, 22, seed=4)
    grid = Grid(40, 28, 22)
    gc = grid.to_c()
    dx, dy, dz = _dev(x), _dev(y), _dev(z)
    stream = torch.cuda.current_stream().cuda_stream
    fields = [phi, cases.F(-phi + 0.05), phi]
    for k, f in enumerate(fields):
        dphi = _dev(f)
        ref = ls.total_water_volume(grid, dphi, dx, dy, dz)
        got = np.zeros(4)
        st = lib.lsm_total_water_volume_noalloc(C.byref(gc), dphi.data_ptr(), dx.data_ptr(), dy.data_ptr(),
                                                dz.data_ptr(), got.ctypes.data, stream)
        assert st == 0, lib.lsm_last_error(None)
        assert cases.relerr(got, ref) <= TOL, (k, got, ref)
        # the same call straight after, writing the result into device memory
        dres = torch.zeros(4, dtype=torch.float64, device="cuda")
        st = lib.lsm_total_water_volume_noalloc(C.byref(gc), dphi.data_ptr(), dx.data_ptr(), dy.data_ptr(),
                                                dz.data_ptr(), dres.data_ptr(), stream)
        assert st == 0, lib.lsm_last_error(None)
        assert cases.relerr(dres.cpu().numpy(), ref) <= TOL


def test_noalloc_rejects_grids_beyond_its_fixed_scratch(ls):
    from nslsm import Grid, _lib
    lib = _lib.load()
    big = Grid(1024, 1024, 80)           # 83 M cells > LSM_NOALLOC_MAX_CELLS (64 Mi)
    gc = big.to_c()
    dummy = np.zeros(4)
    # the size check returns before any pointer is used or any CUDA call is made
    st = lib.lsm_total_water_volume_noalloc(C.byref(gc), dummy.ctypes.data, dummy.ctypes.data, dummy.ctypes.data,
                                            dummy.ctypes.data, dummy.ctypes.data, None)
    assert st == _lib.LSM_ERR_CAPACITY
    assert b"LSM_NOALLOC_MAX_CELLS" in lib.lsm_last_error(None)


def test_noalloc_leaves_free_device_memory_unchanged(ls):
    """The property the entry point exists for: after one warm-up call (which
    loads the kernels), repeated calls do not change the free device memory
    the driver reports."""
    from nslsm import Grid, _lib
    lib = _lib.load()
    g, x, y, z, phi, _ = cases.curvilinear(36, 24, 20, seed=5)
    grid = Grid(36, 24, 20)
    gc = grid.to_c()
    dx, dy, dz, dphi = _dev(x), _dev(y), _dev(z), _dev(phi)
    dres = torch.zeros(4, dtype=torch.float64, device="cuda")
    got = np.zeros(4)
    stream = torch.cuda.current_stream().cuda_stream
    args = (C.byref(gc), dphi.data_ptr(), dx.data_ptr(), dy.data_ptr(), dz.data_ptr())
    assert lib.lsm_total_water_volume_noalloc(*args, got.ctypes.data, stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for r in range(4):
        out = got.ctypes.data if r % 2 == 0 else dres.data_ptr()
        assert lib.lsm_total_water_volume_noalloc(*args, out, stream) == 0, lib.lsm_last_error(None)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert cases.relerr(dres.cpu().numpy(), got) <= TOL


def test_noalloc_rejects_host_inputs(ls):
    """phi, x, y, z must be device arrays: host arrays are refused before any
    kernel runs."""
    from nslsm import Grid, _lib
    lib = _lib.load()
    g, x, y, z, phi, _ = cases.curvilinear(12, 10, 8, seed=6)
    gc = Grid(12, 10, 8).to_c()
    got = np.zeros(4)
    st = lib.lsm_total_water_volume_noalloc(C.byref(gc), phi.ctypes.data, x.ctypes.data, y.ctypes.data,
                                            z.ctypes.data, got.ctypes.data, None)
    assert st == _lib.LSM_ERR_MIXED_MEMORY
    dphi = _dev(phi)
    st = lib.lsm_total_water_volume_noalloc(C.byref(gc), dphi.data_ptr(), x.ctypes.data, y.ctypes.data,
                                            z.ctypes.data, got.ctypes.data, None)
    assert st == _lib.LSM_ERR_MIXED_MEMORY
