// lsm_fp64.cu -- FP64 kernels of the level-set transport step that keep the
// reference's arithmetic: every expression is evaluated in the Fortran
// source's association order and this translation unit is compiled with
// --fmad=false, so each multiply and add rounds separately as gfortran's
// x86-64 code does.  Division and square root are IEEE-rounded in CUDA FP64;
// sin/cos are CUDA's (a few ulp from glibc's).
//
// Roofline: these kernels are FP64-issue bound on GB300, not HBM bound (the
// WENO3 stage alone spends 24 FP64 divisions per node); they are the
// "plain FP64 GPU path" that the FP32 batched kernels are measured against.
#include <cuda_runtime.h>

#include "lsm_common.cuh"
#include "lsm_kernels.h"

namespace lsm {

namespace {

constexpr int BX = 32, BY = 4, BZ = 2;

inline dim3 box_grid(int ni, int nj, int nk) {
    return dim3((ni + BX - 1) / BX, (nj + BY - 1) / BY, (nk + BZ - 1) / BZ);
}

// GetWENO3Reconstruction, src/AdvectionMethods.F90:195-245
__device__ __forceinline__ double weno3(double f0, double f1, double f2, double f3, double ws) {
    const double d0 = 2.0 / 3.0, d1 = 1.0 / 3.0, epsw = 0.000001;
    double fL, fC, fR;
    if (ws > 0.0) { fL = f0; fC = f1; fR = f2; }
    else          { fL = f3; fC = f2; fR = f1; }
    double b0 = (fC - fR) * (fC - fR);
    double b1 = (fL - fC) * (fL - fC);
    double t0 = b0 + epsw, t1 = b1 + epsw;
    double a0 = d0 / (t0 * t0);
    double a1 = d1 / (t1 * t1);
    double w0 = a0 / (a0 + a1);
    double w1 = a1 / (a0 + a1);
    double u0 = 0.5 * fC + 0.5 * fR;
    double u1 = -0.5 * fL + 1.5 * fC;
    return u0 * w0 + u1 * w1;
}

__device__ __forceinline__ bool in_weno_range(const DevGrid& g, int i, int j, int k) {
    return i >= g.ia + g.pb && i <= g.ib - g.pf && j >= g.ja + g.pl && j <= g.jb - g.pr &&
           k >= g.ka + g.pd && k <= g.kb - g.pu;
}

__device__ __forceinline__ bool non_ghost(const DevGrid& g, int i, int j, int k) {
    return i >= g.ia && i <= g.ib && j >= g.ja && j <= g.jb && k >= g.ka && k <= g.kb;
}

// calc_RH_AD_WENO3 body for one node, src/calc_RH_AD_WENO3.F90:132-399
__device__ double weno3_rhs_node(const DevGrid& g, const double* __restrict__ phi,
                                 const double* __restrict__ ucn, long long l, int i, int j, int k) {
    const int i0 = g.ia + g.pb, i1 = g.ib - g.pf;
    const int j0 = g.ja + g.pl, j1 = g.jb - g.pr;
    const int k0 = g.ka + g.pd, k1 = g.kb - g.pu;
    const bool lo[3] = {g.pb && i == i0, g.pl && j == j0, g.pd && k == k0};
    const bool hi[3] = {g.pf && i == i1, g.pr && j == j1, g.pu && k == k1};
    const long long st[3] = {1, g.sj, g.sk};
    const double dd[3] = {g.dc, g.de, g.dz};
    double L[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long s = st[d];
        const double U = __ldg(ucn + 3 * l + d);
        double ws = U;
        double p0 = __ldg(phi + l - s), p1 = __ldg(phi + l), p2 = __ldg(phi + l + s), p3;
        if (hi[d]) { ws = 1.0; p3 = 0.0; } else p3 = __ldg(phi + l + 2 * s);
        const double fp = weno3(p0, p1, p2, p3, ws);
        ws = U;
        if (lo[d]) { ws = -1.0; p0 = 0.0; } else p0 = __ldg(phi + l - 2 * s);
        p1 = __ldg(phi + l - s); p2 = __ldg(phi + l); p3 = __ldg(phi + l + s);
        const double fm = weno3(p0, p1, p2, p3, ws);
        L[d] = U * (dd[d] * (fp - fm));
    }
    return L[0] + L[1] + L[2];
}

// calc_RH_AD (orderAD == 0) for one non-ghost node, src/calc_RH_AD.F90:1-273
__device__ double upwind_rhs_node(const DevGrid& g, const double* __restrict__ phi,
                                  const double* __restrict__ ucn, long long l, int i, int j, int k) {
    const long long st[3] = {1, g.sj, g.sk};
    const double dd[3] = {g.dc, g.de, g.dz};
    const int c[3] = {i, j, k};
    const int plo[3] = {g.pb, g.pl, g.pd}, phs[3] = {g.pf, g.pr, g.pu};
    const int lo[3] = {g.ia, g.ja, g.ka}, hi[3] = {g.ib, g.jb, g.kb};
    double rh = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long s = st[d];
        const double U = __ldg(ucn + 3 * l + d);
        const double pc = __ldg(phi + l);
        double val;
        if (plo[d] && c[d] == lo[d]) {
            val = dd[d] * U * (__ldg(phi + l + s) - pc);
        } else if (phs[d] && c[d] == hi[d]) {
            val = dd[d] * U * (pc - __ldg(phi + l - s));
        } else {
            const double ucon = 0.5 * U;
            const double up = ucon + fabs(ucon), um = ucon - fabs(ucon);
            val = dd[d] * (up * (pc - __ldg(phi + l - s)) + um * (__ldg(phi + l + s) - pc));
        }
        rh = d == 0 ? val : val + rh;
    }
    return rh;
}

// ---------------------------------------------------------------- A1 ----
// rhs_contra_j, src/rhs_contra_j.F90:2-53; zero outside the loop range
__global__ void contra_kernel(DevGrid g, const double* __restrict__ q, const double* __restrict__ csi,
                              const double* __restrict__ eta, const double* __restrict__ zet,
                              const double* __restrict__ aj, double* __restrict__ ucn) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    const int ista = g.pb ? g.ia : 0, iend = g.pf ? g.ib : g.ni - 1;
    const int jsta = g.pl ? g.ja : 0, jend = g.pr ? g.jb : g.nj - 1;
    const int ksta = g.pd ? g.ka : 0, kend = g.pu ? g.kb : g.nk - 1;
    if (i < ista || i > iend || j < jsta || j > jend || k < ksta || k > kend) {
        ucn[3 * l] = 0.0; ucn[3 * l + 1] = 0.0; ucn[3 * l + 2] = 0.0;
        return;
    }
    const double tmp = 1.0 / aj[l];
    const double u = q[4 * l + 1], v = q[4 * l + 2], w = q[4 * l + 3];
    ucn[3 * l + 0] = tmp * (csi[3 * l] * u + csi[3 * l + 1] * v + csi[3 * l + 2] * w);
    ucn[3 * l + 1] = tmp * (eta[3 * l] * u + eta[3 * l + 1] * v + eta[3 * l + 2] * w);
    ucn[3 * l + 2] = tmp * (zet[3 * l] * u + zet[3 * l + 1] * v + zet[3 * l + 2] * w);
}

// ------------------------------------------------------------ A2 / A7 ----
__global__ void rh_ad_kernel(DevGrid g, int orderAD, const double* __restrict__ phi,
                             const double* __restrict__ ucn, const int* __restrict__ mask,
                             double* __restrict__ rh) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    double r = 0.0;
    if (orderAD == 1) {
        if (in_weno_range(g, i, j, k) && !(mask && mask[l] == 0)) r = weno3_rhs_node(g, phi, ucn, l, i, j, k);
    } else {
        if (non_ghost(g, i, j, k) && !(mask && mask[l] <= 0)) r = upwind_rhs_node(g, phi, ucn, l, i, j, k);
    }
    rh[l] = r;
}

// ---------------------------------------------------------------- A4 ----
// One TVD-RK3 stage, src/ad_RKTVD3.F90:53-81, written to `out` (ping-pong):
// out = c1*phin + c2*phi1 - c3*aj*dt*rh on advected non-ghost nodes, phi1
// elsewhere.  rh is 0 on physical-boundary nodes under WENO3.
__global__ void rk_stage_kernel(DevGrid g, int orderAD, const double* __restrict__ phin,
                                const double* __restrict__ phi1, const double* __restrict__ ucn,
                                const double* __restrict__ aj, const int* __restrict__ mask, double c1,
                                double c2, double c3, double dt, double* __restrict__ out) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    const double p1 = phi1[l];
    if (!non_ghost(g, i, j, k) || (mask && mask[l] <= 0)) { out[l] = p1; return; }
    double rh = 0.0;
    if (orderAD == 1) {
        if (in_weno_range(g, i, j, k)) rh = weno3_rhs_node(g, phi1, ucn, l, i, j, k);
    } else {
        rh = upwind_rhs_node(g, phi1, ucn, l, i, j, k);
    }
    out[l] = c1 * phin[l] + c2 * p1 - c3 * aj[l] * dt * rh;
}

// ---------------------------------------------------------------- A5 ----
// bcond_lsm, src/bcond_lsm.F90:2-287.  The six faces are applied in the
// order i1, im, j1, jm, k1, km, each reading the two nodes inward of it as
// left by the faces before it.  A boundary node's final value is therefore a
// fixed function of the pre-BC field ("P0"): val_k(val_j(val_i(P0))).  Each
// thread evaluates that chain for one boundary node reading P0 only, so the
// kernel never reads a node that another thread writes.
struct BCRule {
    __device__ static double ext(double n1, double n2, double BigPhi) {
        const double a2 = 4.0 / 3.0, b2 = -1.0 / 3.0, a1 = 1.0, b1 = 0.0;
        const double exsign = (1.0 + copysign(1.0, fabs(n2) - BigPhi)) / 2.0;
        const double itpa = a2 + exsign * (a1 - a2);
        const double itpb = b2 + exsign * (b1 - b2);
        return itpa * n1 + itpb * n2;
    }
    __device__ static double apply(int type, int face, double n1, double n2, double BigPhi) {
        if (type == 0) return n1;
        if (type == 1) return ext(n1, n2, BigPhi);
        (void)face;
        return 2.0 * n1 - 1.0 * n2;  // type 2, only on the im face
    }
};

__device__ __forceinline__ bool face_applies(const DevBC& bc, int face, int phys) {
    const int t = bc.type[face];
    return phys && (t == 0 || t == 1 || (t == 2 && face == 1));
}

template <class P0>
__device__ double val_i(const DevGrid& g, const DevBC& bc, const P0& p0, int i, int j, int k) {
    if (i == g.ia && face_applies(bc, 0, g.pb))
        return BCRule::apply(bc.type[0], 0, p0(i + 1, j, k), p0(i + 2, j, k), bc.BigPhi);
    if (i == g.ib && face_applies(bc, 1, g.pf))
        return BCRule::apply(bc.type[1], 1, p0(i - 1, j, k), p0(i - 2, j, k), bc.BigPhi);
    return p0(i, j, k);
}
template <class P0>
__device__ double val_j(const DevGrid& g, const DevBC& bc, const P0& p0, int i, int j, int k) {
    if (j == g.ja && face_applies(bc, 2, g.pl))
        return BCRule::apply(bc.type[2], 2, val_i(g, bc, p0, i, j + 1, k), val_i(g, bc, p0, i, j + 2, k),
                             bc.BigPhi);
    if (j == g.jb && face_applies(bc, 3, g.pr))
        return BCRule::apply(bc.type[3], 3, val_i(g, bc, p0, i, j - 1, k), val_i(g, bc, p0, i, j - 2, k),
                             bc.BigPhi);
    return val_i(g, bc, p0, i, j, k);
}
template <class P0>
__device__ double val_k(const DevGrid& g, const DevBC& bc, const P0& p0, int i, int j, int k) {
    if (k == g.ka && face_applies(bc, 4, g.pd))
        return BCRule::apply(bc.type[4], 4, val_j(g, bc, p0, i, j, k + 1), val_j(g, bc, p0, i, j, k + 2),
                             bc.BigPhi);
    if (k == g.kb && face_applies(bc, 5, g.pu))
        return BCRule::apply(bc.type[5], 5, val_j(g, bc, p0, i, j, k - 1), val_j(g, bc, p0, i, j, k - 2),
                             bc.BigPhi);
    return val_j(g, bc, p0, i, j, k);
}

__device__ __forceinline__ bool on_phys_face(const DevGrid& g, int i, int j, int k) {
    return (g.pb && i == g.ia) || (g.pf && i == g.ib) || (g.pl && j == g.ja) || (g.pr && j == g.jb) ||
           (g.pd && k == g.ka) || (g.pu && k == g.kb);
}

// P0 inside an RK stage: interior nodes from the stage output, physical-
// boundary nodes recomputed pointwise from the stage inputs.
struct P0Stage {
    DevGrid g;
    int orderAD;
    const double *phin, *phi1, *ucn, *aj, *dst;
    const int* mask;
    double c1, c2, c3, dt;
    __device__ double operator()(int i, int j, int k) const {
        const long long l = gid(g, i, j, k);
        if (!on_phys_face(g, i, j, k)) return dst[l];
        const double p1 = phi1[l];
        if (mask && mask[l] <= 0) return p1;
        const double rh = orderAD == 1 ? 0.0 : upwind_rhs_node(g, phi1, ucn, l, i, j, k);
        return c1 * phin[l] + c2 * p1 - c3 * aj[l] * dt * rh;
    }
};

struct P0Field {
    DevGrid g;
    const double* src;
    __device__ double operator()(int i, int j, int k) const { return src[gid(g, i, j, k)]; }
};

// Boundary nodes of the six face planes (edge nodes appear twice and are
// written twice with the same value).
__device__ __forceinline__ bool face_node(const DevGrid& g, long long t, int* pi, int* pj, int* pk) {
    const long long Ni = g.ib - g.ia + 1, Nj = g.jb - g.ja + 1, Nk = g.kb - g.ka + 1;
    const long long nI = Nj * Nk, nJ = Ni * Nk, nK = Ni * Nj;
    const long long off[6] = {0, nI, 2 * nI, 2 * nI + nJ, 2 * nI + 2 * nJ, 2 * nI + 2 * nJ + nK};
    int f = 5;
    for (int q = 1; q < 6; ++q)
        if (t < off[q]) { f = q - 1; break; }
    if (t >= off[5] + nK) return false;
    const long long r = t - off[f];
    const int phys[6] = {g.pb, g.pf, g.pl, g.pr, g.pd, g.pu};
    if (!phys[f]) return false;
    if (f < 2) { *pi = f == 0 ? g.ia : g.ib; *pj = g.ja + (int)(r % Nj); *pk = g.ka + (int)(r / Nj); }
    else if (f < 4) { *pj = f == 2 ? g.ja : g.jb; *pi = g.ia + (int)(r % Ni); *pk = g.ka + (int)(r / Ni); }
    else { *pk = f == 4 ? g.ka : g.kb; *pi = g.ia + (int)(r % Ni); *pj = g.ja + (int)(r / Ni); }
    return true;
}

__global__ void bc_rk_kernel(DevGrid g, DevBC bc, P0Stage p0, double* __restrict__ dst, long long nface) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nface) return;
    int i, j, k;
    if (!face_node(g, t, &i, &j, &k)) return;
    dst[gid(g, i, j, k)] = val_k(g, bc, p0, i, j, k);
}

// dst = bcond_lsm(src) over the full array (ghosts copied); flags non-finite output.
__global__ void bc_full_kernel(DevGrid g, DevBC bc, const double* __restrict__ src, double* __restrict__ dst,
                               unsigned* errflag) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    double v;
    if (non_ghost(g, i, j, k) && on_phys_face(g, i, j, k)) {
        P0Field p0{g, src};
        v = val_k(g, bc, p0, i, j, k);
    } else {
        v = src[l];
    }
    dst[l] = v;
    if (errflag && !isfinite(v)) atomicOr(errflag, (unsigned)kErrNonFinite);
}

// ------------------------------------------------------------ R1 / R2 ----
// One-sided differences of src/calc_sign_ini.F90:42-176 (= calc_RH_RN.F90:36-170)
// and the Godunov norms of calc_sign_ini.F90:204-242, for one node.
__device__ __forceinline__ void godunov_node(const DevGrid& g, const double* __restrict__ f,
                                             const double* __restrict__ csi, const double* __restrict__ eta,
                                             const double* __restrict__ zet, long long l, int i, int j, int k,
                                             double* gplus, double* gminus) {
    const long long st[3] = {1, g.sj, g.sk};
    const double dd[3] = {g.dc, g.de, g.dz};
    const int c[3] = {i, j, k};
    const int plo[3] = {g.pb, g.pl, g.pd}, phs[3] = {g.pf, g.pr, g.pu};
    const int lo[3] = {g.ia, g.ja, g.ka}, hi[3] = {g.ib, g.jb, g.kb};
    double mas[3], men[3];
    const double fc = __ldg(f + l);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long s = st[d];
        if (plo[d] && c[d] == lo[d]) {
            mas[d] = dd[d] * (__ldg(f + l + s) - fc); men[d] = mas[d];
        } else if (phs[d] && c[d] == hi[d]) {
            men[d] = dd[d] * (fc - __ldg(f + l - s)); mas[d] = men[d];
        } else {
            mas[d] = dd[d] * (__ldg(f + l + s) - fc);
            men[d] = dd[d] * (fc - __ldg(f + l - s));
        }
    }
    const double* m[3] = {csi + 3 * l, eta + 3 * l, zet + 3 * l};
    double b[3], fw[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        b[x] = __ldg(m[0] + x) * men[0] + __ldg(m[1] + x) * men[1] + __ldg(m[2] + x) * men[2];
        fw[x] = __ldg(m[0] + x) * mas[0] + __ldg(m[1] + x) * mas[1] + __ldg(m[2] + x) * mas[2];
    }
    double bp[3], bm[3], fp[3], fm[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        double aux = b[x] / 2.0;
        bp[x] = aux + fabs(aux); bm[x] = aux - fabs(aux);
        aux = fw[x] / 2.0;
        fp[x] = aux + fabs(aux); fm[x] = aux - fabs(aux);
    }
    *gplus = sqrt(fmax(bp[0] * bp[0], fm[0] * fm[0]) + fmax(bp[1] * bp[1], fm[1] * fm[1]) +
                  fmax(bp[2] * bp[2], fm[2] * fm[2]));
    *gminus = sqrt(fmax(bm[0] * bm[0], fp[0] * fp[0]) + fmax(bm[1] * bm[1], fp[1] * fp[1]) +
                   fmax(bm[2] * bm[2], fp[2] * fp[2]));
}

// deltaf, src/global_lsm.F90:120-133
__device__ __forceinline__ double deltaf(double v, double e) {
    if (fabs(v) > e) return 0.0;
    return 1.0 / (2.0 * e) * (1.0 + cos(kPi * v / e));
}

// calc_sign_ini, src/calc_sign_ini.F90:199-269 (+ deltaf(phi0) for the reinit steps)
__global__ void sign_ini_kernel(DevGrid g, const double* __restrict__ phi0, const double* __restrict__ csi,
                                const double* __restrict__ eta, const double* __restrict__ zet, double eps,
                                int M_Sphi0, double* __restrict__ sgn, double* __restrict__ ng,
                                double* __restrict__ delta) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    if (!non_ghost(g, i, j, k)) {
        sgn[l] = 0.0; ng[l] = 0.0;
        if (delta) delta[l] = 0.0;
        return;
    }
    double gp, gm;
    godunov_node(g, phi0, csi, eta, zet, l, i, j, k, &gp, &gm);
    const double f = phi0[l];
    const double nrm = f > 0.0 ? gp : (f < 0.0 ? gm : 1.0);
    double s;
    if (M_Sphi0 == 1) {
        if (f >= eps) s = 1.0;
        else if (f <= (-1.0) * eps) s = -1.0;
        else s = f / eps - 1.0 / kPi * sin(kPi * f / eps);
    } else {
        s = f / sqrt(f * f + (nrm * eps) * (nrm * eps));
    }
    sgn[l] = s;
    ng[l] = nrm;
    if (delta) delta[l] = deltaf(f, eps);
}

// calc_RH_RN, src/calc_RH_RN.F90:185-238
__global__ void rh_rn_kernel(DevGrid g, const double* __restrict__ d, const double* __restrict__ sgn,
                             const double* __restrict__ csi, const double* __restrict__ eta,
                             const double* __restrict__ zet, double* __restrict__ rh) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    if (!non_ghost(g, i, j, k)) { rh[l] = 0.0; return; }
    double gp, gm;
    godunov_node(g, d, csi, eta, zet, l, i, j, k, &gp, &gm);
    const double s = sgn[l];
    const double nrm = s > 0.0 ? gp : (s < 0.0 ? gm : 1.0);
    rh[l] = s * (nrm - 1.0);
}

// calc_lambda_RN method 0, src/calc_lambda_RN.F90:42-63
__device__ __forceinline__ double lambda_node(double vc, double del, double dt, double d, double p0,
                                              double ng) {
    const double Lop = del * (1.0 / dt * (d - p0));
    const double num = vc * Lop;
    const double den = vc * (del * del) * ng;
    return den == 0.0 ? 0.0 : -num / den;
}

__global__ void lambda_rn_kernel(DevGrid g, double eps, const double* __restrict__ phi0,
                                 const double* __restrict__ ng, const double* __restrict__ d, double dt,
                                 double* __restrict__ lam) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    if (!non_ghost(g, i, j, k)) { lam[l] = 0.0; return; }
    const double vc = 1.0 / g.dc * (1.0 / g.de) * (1.0 / g.dz);
    lam[l] = lambda_node(vc, deltaf(phi0[l], eps), dt, d[l], phi0[l], ng[l]);
}

// One pseudo-step of `reinitialization`, src/reinitialization.F90:55-99,
// fused: Godunov RHS -> Euler update -> lambda -> correction.
__global__ void reinit_step_kernel(DevGrid g, double dt, const double* __restrict__ din,
                                   const double* __restrict__ sgn, const double* __restrict__ ng,
                                   const double* __restrict__ delta, const double* __restrict__ phi0,
                                   const double* __restrict__ csi, const double* __restrict__ eta,
                                   const double* __restrict__ zet, double* __restrict__ dout) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    const double dc0 = din[l];
    if (!non_ghost(g, i, j, k)) { dout[l] = dc0; return; }
    double gp, gm;
    godunov_node(g, din, csi, eta, zet, l, i, j, k, &gp, &gm);
    const double s = sgn[l];
    const double nrm = s > 0.0 ? gp : (s < 0.0 ? gm : 1.0);
    const double rh = s * (nrm - 1.0);
    const double d1 = dc0 - dt * rh;
    const double vc = 1.0 / g.dc * (1.0 / g.de) * (1.0 / g.dz);
    const double del = delta[l], gn = ng[l];
    const double lam = lambda_node(vc, del, dt, d1, phi0[l], gn);
    dout[l] = d1 + dt * lam * del * gn;
}

// ---------------------------------------------------------------- N1 ----
// narrowband, src/narrowband.F90:9-19 (every node, ghosts included)
__global__ void narrowband_kernel(long long n, double thr, int isnarrow, const double* __restrict__ phin,
                                  int* __restrict__ nb) {
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (l >= n) return;
    nb[l] = isnarrow == 0 ? 1 : (fabs(phin[l]) < thr ? 1 : 0);
}

// ---------------------------------------------------------------- M0 ----
// mg_metrics on one rank's fine grid, src/mg_metrics.F90:44-264
__global__ void metrics_kernel(DevGrid g, const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, double* __restrict__ csi, double* __restrict__ eta,
                               double* __restrict__ zet, double* __restrict__ aj) {
    const int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y,
              k = blockIdx.z * BZ + threadIdx.z;
    if (i >= g.ni || j >= g.nj || k >= g.nk) return;
    const long long l = gid(g, i, j, k);
    const long long st[3] = {1, g.sj, g.sk};
    const double dd[3] = {g.dc, g.de, g.dz};
    const int c[3] = {i, j, k}, hi[3] = {g.ni - 1, g.nj - 1, g.nk - 1};
    double dx[3], dy[3], dzv[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const long long s = st[d];
        const double dum1 = dd[d], dum = 0.5 * dd[d];
        if (c[d] == 0) {
            dx[d] = dum1 * (x[l + s] - x[l]); dy[d] = dum1 * (y[l + s] - y[l]); dzv[d] = dum1 * (z[l + s] - z[l]);
        } else if (c[d] == hi[d]) {
            dx[d] = dum1 * (x[l] - x[l - s]); dy[d] = dum1 * (y[l] - y[l - s]); dzv[d] = dum1 * (z[l] - z[l - s]);
        } else {
            dx[d] = dum * (x[l + s] - x[l - s]); dy[d] = dum * (y[l + s] - y[l - s]);
            dzv[d] = dum * (z[l + s] - z[l - s]);
        }
    }
    const double xc = dx[0], yc = dy[0], zc = dzv[0], xe = dx[1], ye = dy[1], ze = dzv[1];
    const double xz = dx[2], yz = dy[2], zz = dzv[2];
    const double gj = xc * (ye * zz - yz * ze) + xe * (yz * zc - yc * zz) + xz * (yc * ze - ye * zc);
    const double a = 1.0 / gj;
    aj[l] = a;
    csi[3 * l + 0] = a * (ye * zz - yz * ze);
    csi[3 * l + 1] = a * (xz * ze - xe * zz);
    csi[3 * l + 2] = a * (xe * yz - xz * ye);
    eta[3 * l + 0] = a * (yz * zc - yc * zz);
    eta[3 * l + 1] = a * (xc * zz - xz * zc);
    eta[3 * l + 2] = a * (xz * yc - xc * yz);
    zet[3 * l + 0] = a * (yc * ze - ye * zc);
    zet[3 * l + 1] = a * (xe * zc - xc * ze);
    zet[3 * l + 2] = a * (xc * ye - xe * yc);
}

__global__ void copy_kernel(const double* __restrict__ src, double* __restrict__ dst, long long n) {
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n;
         l += (long long)gridDim.x * blockDim.x)
        dst[l] = src[l];
}

}  // namespace

// ---------------------------------------------------------------- launchers
#define LSM_BOX(g) box_grid((g).ni, (g).nj, (g).nk), dim3(BX, BY, BZ), 0, s

void launch_contra(const DevGrid& g, const double* q, const double* csi, const double* eta,
                   const double* zet, const double* aj, double* ucn, cudaStream_t s) {
    ProfScope ps_("contra_kernel", s);
    contra_kernel<<<LSM_BOX(g)>>>(g, q, csi, eta, zet, aj, ucn);
}

void launch_rh_ad(const DevGrid& g, int orderAD, const double* phi, const double* ucn, const int* mask,
                  double* rh, cudaStream_t s) {
    ProfScope ps_("rh_ad_kernel", s);
    rh_ad_kernel<<<LSM_BOX(g)>>>(g, orderAD, phi, ucn, mask, rh);
}

void launch_rk_stage(const DevGrid& g, int orderAD, const double* phin, const double* phi1, const double* ucn,
                     const double* aj, const int* mask, double c1, double c2, double c3, double dt, double* out,
                     cudaStream_t s) {
    ProfScope ps_("rk_stage_kernel", s);
    rk_stage_kernel<<<LSM_BOX(g)>>>(g, orderAD, phin, phi1, ucn, aj, mask, c1, c2, c3, dt, out);
}

void launch_bc_rk(const DevGrid& g, const DevBC& bc, int orderAD, const double* phin, const double* phi1,
                  const double* ucn, const double* aj, const int* mask, double c1, double c2, double c3,
                  double dt, double* dst, cudaStream_t s) {
    const long long Ni = g.ib - g.ia + 1, Nj = g.jb - g.ja + 1, Nk = g.kb - g.ka + 1;
    const long long nface = 2 * (Nj * Nk + Ni * Nk + Ni * Nj);
    P0Stage p0{g, orderAD, phin, phi1, ucn, aj, dst, mask, c1, c2, c3, dt};
    ProfScope ps_("bc_rk_kernel", s);
    bc_rk_kernel<<<(unsigned)((nface + 255) / 256), 256, 0, s>>>(g, bc, p0, dst, nface);
}

void launch_bc_full(const DevGrid& g, const DevBC& bc, const double* src, double* dst, unsigned* errflag,
                    cudaStream_t s) {
    ProfScope ps_("bc_full_kernel", s);
    bc_full_kernel<<<LSM_BOX(g)>>>(g, bc, src, dst, errflag);
}

void launch_sign_ini(const DevGrid& g, const double* phi0, const double* csi, const double* eta,
                     const double* zet, double eps, int M_Sphi0, double* sgn, double* ng, double* delta,
                     cudaStream_t s) {
    ProfScope ps_("sign_ini_kernel", s);
    sign_ini_kernel<<<LSM_BOX(g)>>>(g, phi0, csi, eta, zet, eps, M_Sphi0, sgn, ng, delta);
}

void launch_rh_rn(const DevGrid& g, const double* d, const double* sgn, const double* csi, const double* eta,
                  const double* zet, double* rh, cudaStream_t s) {
    ProfScope ps_("rh_rn_kernel", s);
    rh_rn_kernel<<<LSM_BOX(g)>>>(g, d, sgn, csi, eta, zet, rh);
}

void launch_lambda_rn(const DevGrid& g, double eps, const double* phi0, const double* ng, const double* d,
                      double dt, double* lam, cudaStream_t s) {
    ProfScope ps_("lambda_rn_kernel", s);
    lambda_rn_kernel<<<LSM_BOX(g)>>>(g, eps, phi0, ng, d, dt, lam);
}

void launch_reinit_step(const DevGrid& g, double dt, const double* din, const double* sgn, const double* ng,
                        const double* delta, const double* phi0, const double* csi, const double* eta,
                        const double* zet, double* dout, cudaStream_t s) {
    ProfScope ps_("reinit_step_kernel", s);
    reinit_step_kernel<<<LSM_BOX(g)>>>(g, dt, din, sgn, ng, delta, phi0, csi, eta, zet, dout);
}

void launch_narrowband(const DevGrid& g, double thr, int isnarrow, const double* phin, int* nb, cudaStream_t s) {
    const long long n = (long long)g.ni * g.nj * g.nk;
    ProfScope ps_("narrowband_kernel", s);
    narrowband_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, thr, isnarrow, phin, nb);
}

void launch_metrics(const DevGrid& g, const double* x, const double* y, const double* z, double* csi,
                    double* eta, double* zet, double* aj, cudaStream_t s) {
    ProfScope ps_("metrics_kernel", s);
    metrics_kernel<<<LSM_BOX(g)>>>(g, x, y, z, csi, eta, zet, aj);
}

void launch_copy(const double* src, double* dst, long long n, cudaStream_t s) {
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    ProfScope ps_("copy_kernel", s);
    copy_kernel<<<(unsigned)blocks, 256, 0, s>>>(src, dst, n);
}

}  // namespace lsm
