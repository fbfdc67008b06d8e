// Test harness (built by tests/test_newton_cpu.py): exposes the library's
// host-side Newton solve of the geometric reinitialisation
// (lsm::geo_newton, csrc/lsm_geometric.h) on a caller's function, so that
// it can be checked against the oracle's restatement on the same values.
#include "lsm_geometric.h"

extern "C" int product_newton_1d(double (*f)(void*, double), void* ud, double tol, int* its, int* conv,
                                 double* C) {
    bool c = false;
    *C = lsm::geo_newton([&](double x) { return f(ud, x); }, tol, its, &c);
    *conv = c ? 1 : 0;
    return 0;
}
