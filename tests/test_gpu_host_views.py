"""The batch's transfer entry points with the three kinds of caller array:
pageable host memory (copied through the staging buffer), page-locked host
memory (read and written in place by the conversion kernels through its
mapped alias) and device memory of the batch's GPU (used in place).  Every
input path must load the same bits and every output path must return the
same bits, for scalar fields and for the strided records q(1:4, .) and
csi/eta/zet(1:3, .) (one pass over all components; q(1) of the velocity
gradient written as zero).  Both precisions."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

NI, NJ, NK = 36, 20, 17


def _case(orc):
    from nslsm.configs import _mesh
    import oracle as O
    XI, ET, ZE = _mesh(NI, NJ, NK)
    X, Y, Z = XI + 0.05 * ET, ET - 0.03 * ZE, ZE + 0.04 * XI
    F = lambda a: np.asfortranarray(a, dtype=np.float64)  # noqa: E731
    x, y, z = F(X), F(Y), F(Z)
    phi = F(Z - 0.5 - 0.04 * np.cos(2 * np.pi * (2 * X + Y)))
    q = np.zeros((4, NI, NJ, NK), order="F")
    q[1] = 0.6 + 0.3 * np.sin(2 * np.pi * Y)
    q[2] = -0.4 * np.cos(2 * np.pi * X)
    q[3] = 0.2 * np.sin(2 * np.pi * X) * np.sin(np.pi * Z)
    csi, eta, zet, _ = orc.mg_metrics(O.make_grid(NI, NJ, NK), x, y, z)
    return dict(x=x, y=y, z=z, csi=csi, eta=eta, zet=zet, q=q, phi=phi)


def _pinned(a):
    """A Fortran-ordered view of page-locked host memory holding a copy of a."""
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    v = t.numpy().reshape(a.shape, order="F")
    v[...] = a
    return v, t


def _device(a):
    """The same bytes as a CUDA tensor of the reversed shape."""
    return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()


def _convert(C, kind):
    keep = []
    out = {}
    for k, a in C.items():
        if kind == "pageable":
            out[k] = a
        elif kind == "pinned":
            v, t = _pinned(a)
            keep.append(t)
            out[k] = v
        else:
            out[k] = _device(a)
    return out, keep


def _empty(shape, kind, keep):
    if kind == "pageable":
        return np.zeros(shape, order="F")
    if kind == "pinned":
        v, t = _pinned(np.zeros(shape, order="F"))
        keep.append(t)
        return v
    return torch.zeros(shape[::-1], dtype=torch.float64, device="cuda")


def _host(a):
    return a.cpu().numpy().T.copy(order="F") if torch.is_tensor(a) else np.array(a, order="F")


def _run(C, kind, precision):
    from nslsm.batch import LevelSetBatch
    A, keep = _convert(C, kind)
    h = 1.0 / (NK - 1)
    b = LevelSetBatch([(NI, NJ, NK, 2e-3, 0.5 * h, 1.5 * h)], RNitermax=3, btype=(1,) * 6, BigPhi=5.0,
                      precision=precision, autotune=False)
    b.set_geometry(0, A["x"], A["y"], A["z"], A["csi"], A["eta"], A["zet"])
    b.set_velocity(0, A["q"])
    b.set_phi(0, A["phi"])
    loaded = _empty((NI, NJ, NK), kind, keep)
    b._chk(b.lib.lsm_batch_get_phi(b.h, 0, _addr(loaded)), "get_phi")
    b.forward_record(4, 2)
    phiT = _empty((NI, NJ, NK), kind, keep)
    b._chk(b.lib.lsm_batch_get_phi(b.h, 0, _addr(phiT)), "get_phi")
    seed = np.asfortranarray(np.random.default_rng(5).standard_normal((NI, NJ, NK)))
    S, keep2 = _convert({"s": seed}, kind)
    keep += keep2
    b.set_grad_phi(0, S["s"])
    b.backward()
    gphi = _empty((NI, NJ, NK), kind, keep)
    gq = _empty((4, NI, NJ, NK), kind, keep)
    b._chk(b.lib.lsm_batch_get_grad_phi0(b.h, 0, _addr(gphi)), "get_grad_phi0")
    b._chk(b.lib.lsm_batch_get_grad_velocity(b.h, 0, _addr(gq)), "get_grad_velocity")
    torch.cuda.synchronize()
    out = [_host(a) for a in (loaded, phiT, gphi, gq)]
    b.close()
    del keep
    return out


def _addr(a):
    return a.data_ptr() if torch.is_tensor(a) else a.ctypes.data


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_pageable_pinned_and_device_arrays_give_the_same_bits(oracle, lib_built, precision):
    C = _case(oracle)
    ref = _run(C, "pageable", precision)
    dt = np.float32 if precision == "fp32" else np.float64
    assert np.array_equal(ref[0], C["phi"].astype(dt).astype(np.float64))   # the loaded field, rounded once
    assert np.all(ref[3][0] == 0.0) and np.any(ref[3][1:] != 0.0)
    for kind in ("pinned", "device"):
        got = _run(C, kind, precision)
        for name, a, r in zip(("phi loaded", "phi_T", "grad phi0", "grad q"), got, ref):
            assert np.array_equal(a, r), (kind, name, float(np.abs(a - r).max()))
