// lsm_geometric.h -- host interface of the geometric reinitialisation
// (lsm_geometric.cu) and its global-volume Newton solve.
#pragma once

#include <cmath>
#include <cuda_runtime.h>

#include "lsm_common.cuh"

namespace lsm {

struct GeoInfo {
    int nnodes, ntetrahedra, nsecond, newton_iterations, newton_converged;
    double C;
};

// device scratch by name (pooled by the caller); sets *e on failure
typedef void* (*GeoAlloc)(void* ctx, const char* name, size_t bytes, cudaError_t* e);

// geometric_reinitialisation (src/geometric_reinitialisation.F90:1-94) on a
// grid without ghost planes: phicorrected `pc` in/out, `tag` receives
// InterfaceNodesID (pnode ids, -1, 0).  d_count: 4 device ints of scratch.
// Returns after `s` has drained.
cudaError_t geo_reinit(const DevGrid& g, const double* phi0, const double* x, const double* y, const double* z,
                       double target, int gmc, double tol, double* pc, int* tag, GeoAlloc alloc, void* actx,
                       unsigned* d_err, int* d_count, GeoInfo* info, cudaStream_t s);

// phicorrected = -9.9 / 9.9 where phi < -epsilon / phi > epsilon
// (src/levelsetmethod.F90:303-304)
void launch_geo_seed(long long n, const double* phi, double* pc, cudaStream_t s);

// NewtonRaphson with newt / fdjac / fmin / lnsrch / ludcmp / lubksb for one
// unknown (src/NewtonRaphsonSolver.F90, Numerical Recipes' globally
// convergent Newton with backtracking), from C = 0.  funcv(C) returns
// target - volume(C).  The PARAMETERs the reference writes as default-real
// literals (1.e-12, 1.e-7, 1.e-4, .1) are single precision promoted to
// REAL(8).  Returns C, or 0 when the reference drops the correction
// (its >= MAXITS or `check` set).
template <class F>
double geo_newton(F funcv, double tol, int* its_out, bool* converged) {
    const int MAXITS = 20;
    const double TOLF = (double)1.e-12f, TOLMIN = (double)1.e-12f, TOLX = (double)1.e-12f, STPMX = 100.0;
    const double ALF = (double)1.e-4f, TOLXL = (double)1.e-7f, P1 = (double)0.1f;
    const double EPSS = 2.220446049250313e-16;
    const double EPS = std::sqrt(EPSS);
    double x = 0.0;
    bool check = false;  // newt leaves it unset on its zero-Jacobian return
    int its = 1;
    auto finish = [&]() {
        *its_out = its;
        *converged = its < MAXITS && !check;
        return *converged ? x : 0.0;
    };
    double fvec = funcv(x);
    double f = 0.5 * (0.0 + fvec * fvec);
    if (std::fabs(fvec) < 0.01 * TOLF && std::fabs(fvec) < tol) return finish();
    const double stpmax = STPMX * std::fmax(std::sqrt(0.0 + x * x), 1.0);
    for (its = 1; its <= MAXITS; ++its) {
        // fdjac
        const double temp = x;
        double h = EPS * std::fabs(temp);
        if (h < EPSS) h = EPS;
        x = temp + h;
        h = x - temp;
        const double fh = funcv(x);
        x = temp;
        double fjac = (fh - fvec) / h;
        if (std::fabs(0.0 + fjac) < tol) return finish();  // zero Jacobian
        fvec = funcv(x);
        const double gr = 0.0 + fjac * fvec;
        const double xold = x, fold = f;
        double p = -fvec;
        if (fjac == 0.0) fjac = 1.0e-20;  // ludcmp's TINY pivot
        p = p / fjac;
        // lnsrch
        check = false;
        const double sum = std::sqrt(0.0 + p * p);
        if (sum > stpmax) p = p * stpmax / sum;
        const double slope = 0.0 + gr * p;
        const double test = std::fabs(p) / std::fmax(std::fabs(xold), 1.0);
        const double alamin = TOLXL / test;
        double alam = 1.0, alam2 = 2.0, f2 = 2.0, tmplam = 0.0;
        for (int guard = 0; guard < 100000; ++guard) {
            x = xold + alam * p;
            fvec = funcv(x);
            f = 0.5 * (0.0 + fvec * fvec);
            if (alam < alamin) { x = xold; check = true; break; }
            if (f <= fold + ALF * alam * slope) break;
            if (alam == 1.0) {
                tmplam = -slope / (2.0 * (f - fold - slope));
            } else {
                const double rhs1 = f - fold - alam * slope, rhs2 = f2 - fold - alam2 * slope;
                const double a = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
                const double b = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) / (alam - alam2);
                if (a == 0.0) {
                    tmplam = -slope / (2.0 * b);
                } else {
                    const double disc = b * b - 3.0 * a * slope;
                    if (disc < 0.0) tmplam = 0.5 * alam;
                    else if (b <= 0.0) tmplam = (-b + std::sqrt(disc)) / (3.0 * a);
                    else tmplam = -slope / (b + std::sqrt(disc));
                }
                if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
            }
            alam2 = alam;
            f2 = f;
            alam = tmplam > P1 * alam ? tmplam : P1 * alam;
        }
        if (std::fabs(fvec) < TOLF && std::fabs(fvec) < tol) { check = false; return finish(); }
        if (check) {
            const double den = std::fmax(f, 0.5 * 1);
            const double t2 = std::fabs(gr) * std::fmax(std::fabs(x), 1.0) / den;
            check = t2 < TOLMIN;  // spurious convergence: check stays set
            return finish();
        }
        const double t3 = std::fabs(x - xold) / std::fmax(std::fabs(x), 1.0);
        if (t3 < TOLX && std::fabs(fvec) < tol) return finish();
    }
    return finish();  // its = MAXITS + 1
}

}  // namespace lsm
