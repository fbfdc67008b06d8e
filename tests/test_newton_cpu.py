"""The global mass-correction Newton solve of the geometric
reinitialisation (NewtonRaphson / newt / fdjac / fmin / lnsrch,
src/NewtonRaphsonSolver.F90): the library's host implementation
(csrc/lsm_geometric.h, compiled here into a small harness) against the
oracle's restatement, on the same function values, bit for bit.

The functions are target - volume(C) shapes that drive the solver's paths:
plain convergence, backtracking line searches (cubic steps), a target out
of reach (20 iterations, C dropped), a zero Jacobian, a solution in the
first evaluation, and a step limited by stpmax."""
import ctypes as C
import math
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
FN = C.CFUNCTYPE(C.c_double, C.c_void_p, C.c_double)
SIG = [FN, C.c_void_p, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if not gxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    out = str(tmp_path_factory.mktemp("newton") / "libnewton_harness.so")
    cmd = [gxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", inc,
           "-I", os.path.join(REPO, "ns-lsm-single-phase_gb300", "csrc"), "-I", os.path.join(REPO, "include"),
           os.path.join(HERE, "newton_harness.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(out)
    lib.product_newton_1d.argtypes = SIG
    lib.product_newton_1d.restype = C.c_int
    return lib


@pytest.fixture(scope="module")
def oracle_lib(oracle):
    lib = oracle.lib
    lib.oracle_newton_1d.argtypes = SIG
    lib.oracle_newton_1d.restype = C.c_int
    return lib


CASES = {
    # name: (f(C), tol)
    "linear": (lambda c: 0.3 - (0.1 + 0.02 * c), 1e-9),
    "cubic": (lambda c: 0.05 - (0.01 * c + 0.004 * c ** 3), 1e-9),
    "backtrack": (lambda c: 0.2 - math.atan(3.0 * c), 1e-9),
    "saturating": (lambda c: 0.02 - (0.05 * math.tanh(0.5 * c) + 1e-4 * c), 1e-11),
    "saturated": (lambda c: 0.5 - (0.1 + 0.01 * math.tanh(c)), 1e-9),
    "unreachable": (lambda c: 0.5 - (0.1 + 0.01 * math.atan(c)), 1e-9),
    "flat": (lambda c: 1e-3 - 1e-13 * c, 1e-9),
    "at_start": (lambda c: 1e-16 - 1e-3 * c, 1e-9),
    "far": (lambda c: 50.0 - (0.1 * c + 1e-6 * c ** 3), 1e-9),
    "oscillating": (lambda c: 0.01 - (0.02 * c + 0.01 * math.sin(7.0 * c)), 1e-10),
}


def _run(fn, lib, name, f, tol):
    calls = []

    def cb(_ud, c):
        calls.append(c)
        return f(c)

    cf = FN(cb)
    its, conv, cc = C.c_int(0), C.c_int(0), C.c_double(0.0)
    assert getattr(lib, fn)(cf, None, tol, C.byref(its), C.byref(conv), C.byref(cc)) == 0
    return its.value, conv.value, cc.value, calls


@pytest.mark.parametrize("name", sorted(CASES))
def test_newton_matches_oracle(harness, oracle_lib, name):
    f, tol = CASES[name]
    r_prod = _run("product_newton_1d", harness, name, f, tol)
    r_orc = _run("oracle_newton_1d", oracle_lib, name, f, tol)
    # same iterations, decision and C, and the same sequence of evaluations
    assert r_prod[:3] == r_orc[:3], (name, r_prod[:3], r_orc[:3])
    assert r_prod[3] == r_orc[3]


def test_newton_paths_are_exercised(oracle_lib):
    res = {n: _run("oracle_newton_1d", oracle_lib, n, *CASES[n]) for n in CASES}
    # the finite-difference Jacobian (step 1.5e-8) leaves C within ~1e-7 of the root
    assert res["linear"][1] == 1 and abs(res["linear"][2] - 10.0) < 1e-6
    # out of reach: the steps are capped by stpmax, MAXITS runs out, C is dropped
    assert res["unreachable"][1] == 0 and res["unreachable"][2] == 0.0 and res["unreachable"][0] == 21
    # kept from the reference: after one step into the saturated region the
    # Jacobian is zero, newt returns with `check` clear and its < MAXITS, and
    # NewtonRaphson keeps that C although the volume is not met
    assert res["saturated"][1] == 1 and res["saturated"][0] == 2 and res["saturated"][2] > 30.0
    assert res["at_start"][0] == 1 and res["at_start"][1] == 1 and res["at_start"][2] == 0.0
    assert res["flat"][1] == 1 and res["flat"][2] == 0.0      # zero Jacobian: C stays at the guess
    # a backtracking line search happened somewhere (more evaluations than 3 per iteration)
    assert any(len(r[3]) > 3 * max(r[0], 1) + 1 for r in res.values())
