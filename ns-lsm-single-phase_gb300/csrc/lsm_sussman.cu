// lsm_sussman.cu -- the reference's live reinitialisation,
// reinitialisation_test2 (src/reinitialisation_test2.F90:1-221), and its
// gradient norm calc_NormGrad_d (src/calc_NormGrad_d.F90:1-2448), in FP64
// with the reference's operation order (built with --fmad=false).
//
// calc_NormGrad_d's 27 blocks (interior, 6 faces, 12 edges, 8 corners)
// reduce to one choice per direction and node: a one-sided BiasedDerivative
// (src/AdvectionMethods.F90:248-302, ENO2Boundary :654-707) along a
// direction whose face is physical at the node, GetENO2Reconstruction
// (src/AdvectionMethods.F90:63-191) otherwise, with the stencil clipped on
// the node next to a physical face.  One thread per node; ghost nodes get 0.
// The two i-face blocks never assign phi0, so their ENO2 stencil choice
// uses phizero at the last node of the interior loop (`stale`).
#include <cuda_runtime.h>

#include <algorithm>

#include "lsm_common.cuh"
#include "lsm_kernels.h"

namespace lsm {
namespace {

inline unsigned nblocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// GetENO2Reconstruction, src/AdvectionMethods.F90:63-191
__device__ double eno2(double f0, double fLL, double fL, double fC, double fR, double fRR, bool lo, bool hi) {
    double a, b, Mf, dp, dm;
    if (lo) {
        a = fR - (2.0 * fC) + fL;
        b = fRR - (2.0 * fR) + fC;
        Mf = a;
        if (fabs(b) < fabs(a)) Mf = b;
        dp = fR - fC - 0.5 * Mf;
        Mf = a;
        dm = fC - fL + 0.5 * Mf;
    } else if (hi) {
        a = fR - (2.0 * fC) + fL;
        Mf = a;
        dp = fR - fC - 0.5 * Mf;
        b = fC - (2.0 * fL) + fLL;
        if (fabs(b) < fabs(a)) Mf = b;
        dm = fC - fL + 0.5 * Mf;
    } else {
        a = fR - (2.0 * fC) + fL;
        b = fRR - (2.0 * fR) + fC;
        Mf = a;
        if (fabs(b) < fabs(a)) Mf = b;
        dp = fR - fC - 0.5 * Mf;
        b = fC - (2.0 * fL) + fLL;
        Mf = a;
        if (fabs(b) < fabs(a)) Mf = b;
        dm = fC - fL + 0.5 * Mf;
    }
    const double sg = fabs(f0) > kEpsSims ? (f0 >= 0.0 ? 1.0 : -1.0) : 0.0;
    if (sg * (fR - fC) < 0.0 && sg * (fC - fL) < -sg * (fR - fC)) return dp;
    if (sg * (fC - fL) > 0.0 && sg * (fR - fC) > -sg * (fC - fL)) return dm;
    return 0.5 * (dp + dm);
}

// ENO2Boundary, src/AdvectionMethods.F90:654-707
__device__ double eno2_boundary(double f0, double f1, double f2, int bias) {
    const double as = (double)bias;
    const double D1 = as * (f1 - f0), D2 = as * (f2 - f1), D3 = as * (f2 - f0) / 2.0;
    if (fabs(D1 - D2) < kEpsSims) return D1;
    if (fabs(D1) < fabs(D2)) return (2.0 * D1 + D2) / 3.0;
    if (fabs(D2) < fabs(D1)) return (D1 + 2.0 * D2) / 3.0;
    if (fabs(D1) == fabs(D2)) return (4.0 * D1 + D2) / 5.0;
    if (fabs(D1) < fabs(D3) && fabs(D2) < fabs(D3)) return (3.0 * D1 + 6.0 * D2 - D3) / 7.0;
    if (fabs(D1) >= fabs(D3) && fabs(D2) >= fabs(D3)) return D3;
    return D1;
}

// BiasedDerivative, src/AdvectionMethods.F90:248-302
__device__ double biased(double f0, double f1, double f2, double f3, int order, int bias, bool enobc) {
    const double as = (double)bias;
    if (order == 1) return as * (-1.0 * f0 + 1.0 * f1);
    if (order == 2) {
        if (enobc) return eno2_boundary(f0, f1, f2, bias);
        return as * (-(3.0 * f0) + 4.0 * f1 - 1.0 * f2) / 2.0;
    }
    return as * (-(11.0 * f0) + 18.0 * f1 - 9.0 * f2 + 2.0 * f3) / 6.0;
}

__global__ void sign_phi0_kernel(long long n, const double* __restrict__ phi0, double eps, double* __restrict__ sg) {
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (l >= n) return;
    const double p = phi0[l];
    // GetSignPhi0, src/AdvectionMethods.F90:576-587
    sg[l] = fabs(p) > eps ? (p >= 0.0 ? 1.0 : -1.0) : p / eps - 1.0 / kPi * sin((kPi * p) / eps);
}

__global__ void normgrad_d_kernel(DevGrid g, int order, int enobc, const double* __restrict__ phi,
                                  const double* __restrict__ phizero, long long stale,
                                  const double* __restrict__ csi, const double* __restrict__ eta,
                                  const double* __restrict__ zet, double* __restrict__ out) {
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)g.ni * g.nj * g.nk;
    if (l >= n) return;
    const int i = (int)(l % g.ni), j = (int)((l / g.ni) % g.nj), k = (int)(l / ((long long)g.ni * g.nj));
    if (i < g.ia || i > g.ib || j < g.ja || j > g.jb || k < g.ka || k > g.kb) {
        out[l] = 0.0;   // ghost node (NormGrad_RN = zero)
        return;
    }
    const int c[3] = {i, j, k};
    const int lo[3] = {g.ia, g.ja, g.ka}, hi[3] = {g.ib, g.jb, g.kb};
    const int plo[3] = {g.pb, g.pl, g.pd}, phy[3] = {g.pf, g.pr, g.pu};
    const long long st[3] = {1, g.sj, g.sk};
    const double dd[3] = {g.dc, g.de, g.dz};
    const bool iface = (g.pb && i == g.ia) || (g.pf && i == g.ib);
    const bool jface = (g.pl && j == g.ja) || (g.pr && j == g.jb);
    const bool kface = (g.pd && k == g.ka) || (g.pu && k == g.kb);
    const double phi0 = (iface && !jface && !kface) ? phizero[stale] : phizero[l];
    double d[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const long long s = st[m];
        if (plo[m] && c[m] == lo[m]) {
            d[m] = dd[m] * biased(phi[l], phi[l + s], phi[l + 2 * s], phi[l + 3 * s], order, 1, enobc != 0);
        } else if (phy[m] && c[m] == hi[m]) {
            d[m] = dd[m] * biased(phi[l], phi[l - s], phi[l - 2 * s], phi[l - 3 * s], order, -1, enobc != 0);
        } else {
            // the node next to a physical face clips the stencil (the
            // reference passes a dummy zero instead of the node beyond)
            const bool lob = plo[m] && c[m] == lo[m] + 1, hib = phy[m] && c[m] == hi[m] - 1;
            const double fLL = lob ? 0.0 : phi[l - 2 * s], fRR = hib ? 0.0 : phi[l + 2 * s];
            d[m] = dd[m] * eno2(phi0, fLL, phi[l - s], phi[l], phi[l + s], fRR, lob, hib);
        }
    }
    const double dx = csi[3 * l + 0] * d[0] + eta[3 * l + 0] * d[1] + zet[3 * l + 0] * d[2];
    const double dy = csi[3 * l + 1] * d[0] + eta[3 * l + 1] * d[1] + zet[3 * l + 1] * d[2];
    const double dz = csi[3 * l + 2] * d[0] + eta[3 * l + 2] * d[1] + zet[3 * l + 2] * d[2];
    out[l] = sqrt(dx * dx + dy * dy + dz * dz);
}

// deltaf, src/global_lsm.F90:120-133
__device__ __forceinline__ double deltaf(double v, double e) {
    if (fabs(v) > e) return 0.0;
    return 1.0 / (2.0 * e) * (1.0 + cos(kPi * v / e));
}

// one RK stage of reinitialisation_test2 (src/reinitialisation_test2.F90:140-168)
__global__ void sussman_rk_kernel(DevGrid g, const double* __restrict__ dn, double* __restrict__ dn1,
                                  const double* __restrict__ ng, const double* __restrict__ ngc,
                                  const double* __restrict__ sg, double eps, double epsr, double dt, double c1,
                                  double c2, double c3) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int wi = g.ib - g.ia + 1, wj = g.jb - g.ja + 1, wk = g.kb - g.ka + 1;
    if (t >= (long long)wi * wj * wk) return;
    const int i = g.ia + (int)(t % wi), j = g.ja + (int)((t / wi) % wj), k = g.ka + (int)(t / ((long long)wi * wj));
    const long long l = gid(g, i, j, k);
    if (!(ngc[l] - 1.0 > epsr)) return;
    const double s = sg[l], G = ng[l], d1 = dn1[l];
    double rhs = s * (G - 1.0);
    // GetLambdaMassCorrection, src/global_lsm.F90:200-219
    const double df = deltaf(d1, eps);
    const double num = -df * s * (1.0 - G);
    const double den = (df * df) * G;
    const double lam = fabs(den) < kEpsSims ? 0.0 : num / den;
    const double aux = deltaf(d1, eps) * G;
    rhs = rhs - lam * aux;
    dn1[l] = c1 * dn[l] + c2 * d1 - c3 * dt * rhs;
}

// maximum and minimum of a field (every node, ghosts included, as the
// reference's maxval/minval): per-block partials, then one block; both are
// exact, so the order does not matter
__global__ void minmax_partial_kernel(long long n, const double* __restrict__ a, double* __restrict__ part) {
    __shared__ double smax[256], smin[256];
    double mx = -1.0e308, mn = 1.0e308;
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n; l += (long long)gridDim.x * blockDim.x) {
        const double v = a[l];
        mx = v > mx ? v : mx;
        mn = v < mn ? v : mn;
    }
    smax[threadIdx.x] = mx;
    smin[threadIdx.x] = mn;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + s]);
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = smax[0];
        part[2 * blockIdx.x + 1] = smin[0];
    }
}

__global__ void minmax_final_kernel(int nb, const double* __restrict__ part, double* __restrict__ res) {
    __shared__ double smax[256], smin[256];
    double mx = -1.0e308, mn = 1.0e308;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        mx = fmax(mx, part[2 * b]);
        mn = fmin(mn, part[2 * b + 1]);
    }
    smax[threadIdx.x] = mx;
    smin[threadIdx.x] = mn;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + s]);
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        res[0] = smax[0];
        res[1] = smin[0];
    }
}

}  // namespace

void launch_sign_phi0(long long n, const double* phi0, double eps, double* sg, cudaStream_t s) {
    ProfScope ps("sign_phi0_kernel", s);
    sign_phi0_kernel<<<nblocks(n, 256), 256, 0, s>>>(n, phi0, eps, sg);
}

void launch_normgrad_d(const DevGrid& g, int order, int enobc, const double* phi, const double* phizero,
                       long long stale, const double* csi, const double* eta, const double* zet, double* out,
                       cudaStream_t s) {
    const long long n = (long long)g.ni * g.nj * g.nk;
    ProfScope ps("normgrad_d_kernel", s);
    normgrad_d_kernel<<<nblocks(n, 256), 256, 0, s>>>(g, order, enobc, phi, phizero, stale, csi, eta, zet, out);
}

void launch_sussman_rk(const DevGrid& g, const double* dn, double* dn1, const double* ng, const double* ngc,
                       const double* sg, double eps, double epsr, double dt, double c1, double c2, double c3,
                       cudaStream_t s) {
    const long long w = (long long)(g.ib - g.ia + 1) * (g.jb - g.ja + 1) * (g.kb - g.ka + 1);
    ProfScope ps("sussman_rk_kernel", s);
    sussman_rk_kernel<<<nblocks(w, 256), 256, 0, s>>>(g, dn, dn1, ng, ngc, sg, eps, epsr, dt, c1, c2, c3);
}

int minmax_partials(long long n) { return (int)std::min<long long>(nblocks(n, 256), 1024); }

void launch_minmax(long long n, const double* a, double* part, double* res, cudaStream_t s) {
    const int nb = minmax_partials(n);
    {
        ProfScope ps("minmax_partial_kernel", s);
        minmax_partial_kernel<<<nb, 256, 0, s>>>(n, a, part);
    }
    ProfScope ps("minmax_final_kernel", s);
    minmax_final_kernel<<<1, 256, 0, s>>>(nb, part, res);
}

}  // namespace lsm
