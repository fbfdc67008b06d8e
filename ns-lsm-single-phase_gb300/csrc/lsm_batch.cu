// lsm_batch.cu -- batched FP32 kernels of the level-set transport step.
//
// One launch per pass covers every instance of the batch: the CTAs are
// persistent (grid = SMs x resident CTAs) and walk a brick table in which
// each brick of TX x TY x TZ nodes belongs to one instance.  Every kernel is
// HBM-bound by design; the per-node algorithmic traffic (4-byte words) is
//   contra 15 (u 3, metrics 9; W 3), RK stage 5/6/6 (phi_prev, phi^n, W 3;
//   phi), sign 11 (phi0, metrics 9; s), reinit pseudo-step 12 (d, s,
//   metrics 9; d), volume 7 (phi + FP64 x, y, z).
//
// Arithmetic: FP32 stencils with the reference's formulas rearranged for
// FP32 (one division per WENO3 reconstruction); the volume is FP64 (the
// reference's marching-tetrahedra functions), with per-instance fixed-order
// sums.  The reinitialisation uses the closed form of the reference's
// method-0 lambda correction: with lambda = -(d1 - phi0) / (dtau delta |grad
// phi0|) the correction dtau lambda delta |grad phi0| returns d to phi0
// wherever delta(phi0) |grad phi0| != 0, i.e. |phi0| < eps; those nodes are
// folded into the sign field as s = 0 (no update) and the pseudo-step reads
// only d, s and the metrics.
#include <cuda_runtime.h>

#include "lsm_batch.cuh"
#include "lsm_common.cuh"
#include "lsm_kernels.h"
#include "lsm_volume_dev.cuh"

namespace lsm {
namespace batch {
namespace {

// ------------------------------------------------------------ brick walk
template <int TX, int TY, int TZ>
struct Brick {
    int inst, i, j, k;     // thread's node (may lie outside the instance)
    bool valid;
};

template <int TX, int TY, int TZ>
__device__ __forceinline__ Brick<TX, TY, TZ> brick_node(const Inst* __restrict__ inst,
                                                         const int* __restrict__ brick_inst, int blk) {
    Brick<TX, TY, TZ> b;
    b.inst = __ldg(brick_inst + blk);
    const Inst& I = inst[b.inst];
    const int local = blk - I.brick0;
    const int bx = local % I.nbx, by = (local / I.nbx) % I.nby, bz = local / (I.nbx * I.nby);
    const int t = threadIdx.x;
    b.i = bx * TX + t % TX;
    b.j = by * TY + (t / TX) % TY;
    b.k = bz * TZ + t / (TX * TY);
    b.valid = b.i < I.ni && b.j < I.nj && b.k < I.nk;
    return b;
}

// ------------------------------------------------------------ WENO3 (FP32)
// GetWENO3Reconstruction (src/AdvectionMethods.F90:195-245) on an oriented
// stencil (fL, fC, fR): weights 2/3, 1/3 over (beta + 1e-6)^2, rearranged to
// one division: w0 = 2 t1^2 / (2 t1^2 + t0^2), Phi = u1 + w0 (u0 - u1).
__device__ __forceinline__ float rec3(float fL, float fC, float fR) {
    const float b0 = (fC - fR) * (fC - fR), b1 = (fL - fC) * (fL - fC);
    const float t0 = b0 + 1.0e-6f, t1 = b1 + 1.0e-6f;
    const float a0 = 2.0f * t1 * t1, a1 = t0 * t0;
    const float w0 = __fdividef(a0, a0 + a1);
    const float u1 = 1.5f * fC - 0.5f * fL;
    return fmaf(w0, 0.5f * (fL + fR) - fC, u1);
}

// Phi_{+1/2} - Phi_{-1/2} along one axis for the node with stencil
// (m2, m1, c, p1, p2); lo/hi force the reference's one-sided stencils on
// the first / last interior node (calc_RH_AD_WENO3.F90:201-245).
__device__ __forceinline__ float weno_diff(float m2, float m1, float c, float p1, float p2, float w, bool lo,
                                           bool hi) {
    const bool up = w > 0.0f;
    const float fp = (up || hi) ? rec3(m1, c, p1) : rec3(p2, p1, c);
    const float fm = (up && !lo) ? rec3(m2, m1, c) : rec3(p1, c, m1);
    return fp - fm;
}

// ------------------------------------------------------------ contra
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_contra(const Inst* __restrict__ inst,
        const int* __restrict__ brick_inst, int nbricks, Fields f, float dc, float de, float dz) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const auto b = brick_node<TX, TY, TZ>(inst, brick_inst, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long l = I.off + b.i + (long long)I.ni * (b.j + (long long)I.nj * b.k);
        const float u = f.u[0][l], v = f.u[1][l], w = f.u[2][l];
        const float dd[3] = {dc, de, dz};
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const float c = f.m[3 * m][l] * u + f.m[3 * m + 1][l] * v + f.m[3 * m + 2][l] * w;
            f.W[m][l] = I.dt * dd[m] * c;
        }
    }
}

// ------------------------------------------------------------ RK stage
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_stage(const Inst* __restrict__ inst,
        const int* __restrict__ brick_inst, int nbricks, Fields f, const float* __restrict__ phin,
        const float* __restrict__ phi1, float* __restrict__ out, float c1, float c2, float c3) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const auto b = brick_node<TX, TY, TZ>(inst, brick_inst, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long sj = I.ni, sk = (long long)I.ni * I.nj;
        const long long l = I.off + b.i + sj * b.j + sk * b.k;
        const float p = __ldg(phi1 + l);
        float R = 0.0f;
        const bool interior = b.i > 0 && b.i < I.ni - 1 && b.j > 0 && b.j < I.nj - 1 && b.k > 0 && b.k < I.nk - 1;
        if (interior) {
            {
                const float w = __ldg(f.W[0] + l);
                const float m2 = b.i > 1 ? __ldg(phi1 + l - 2) : 0.0f;
                const float p2 = b.i < I.ni - 2 ? __ldg(phi1 + l + 2) : 0.0f;
                R = w * weno_diff(m2, __ldg(phi1 + l - 1), p, __ldg(phi1 + l + 1), p2, w, b.i == 1,
                                  b.i == I.ni - 2);
            }
            {
                const float w = __ldg(f.W[1] + l);
                const float m2 = b.j > 1 ? __ldg(phi1 + l - 2 * sj) : 0.0f;
                const float p2 = b.j < I.nj - 2 ? __ldg(phi1 + l + 2 * sj) : 0.0f;
                R = fmaf(w, weno_diff(m2, __ldg(phi1 + l - sj), p, __ldg(phi1 + l + sj), p2, w, b.j == 1,
                                      b.j == I.nj - 2), R);
            }
            {
                const float w = __ldg(f.W[2] + l);
                const float m2 = b.k > 1 ? __ldg(phi1 + l - 2 * sk) : 0.0f;
                const float p2 = b.k < I.nk - 2 ? __ldg(phi1 + l + 2 * sk) : 0.0f;
                R = fmaf(w, weno_diff(m2, __ldg(phi1 + l - sk), p, __ldg(phi1 + l + sk), p2, w, b.k == 1,
                                      b.k == I.nk - 2), R);
            }
        }
        out[l] = c1 * __ldg(phin + l) + c2 * p - c3 * R;
    }
}

// ------------------------------------------------------------ bcond_lsm
__device__ __forceinline__ float bc_rule(int type, float n1, float n2, float BigPhi) {
    if (type == 0) return n1;
    if (type == 1) return fabsf(n2) >= BigPhi ? n1 : (4.0f / 3.0f) * n1 - (1.0f / 3.0f) * n2;
    return 2.0f * n1 - n2;  // type 2 on the im face
}
__device__ __forceinline__ bool face_on(const BC& bc, int face) {
    const int t = bc.type[face];
    return t == 0 || t == 1 || (t == 2 && face == 1);
}

template <class P0>
__device__ float bval_i(const BC& bc, const P0& p0, int ni, int i, int j, int k) {
    if (i == 0 && face_on(bc, 0)) return bc_rule(bc.type[0], p0(1, j, k), p0(2, j, k), bc.BigPhi);
    if (i == ni - 1 && face_on(bc, 1)) return bc_rule(bc.type[1], p0(i - 1, j, k), p0(i - 2, j, k), bc.BigPhi);
    return p0(i, j, k);
}
template <class P0>
__device__ float bval_j(const BC& bc, const P0& p0, int ni, int nj, int i, int j, int k) {
    if (j == 0 && face_on(bc, 2))
        return bc_rule(bc.type[2], bval_i(bc, p0, ni, i, 1, k), bval_i(bc, p0, ni, i, 2, k), bc.BigPhi);
    if (j == nj - 1 && face_on(bc, 3))
        return bc_rule(bc.type[3], bval_i(bc, p0, ni, i, j - 1, k), bval_i(bc, p0, ni, i, j - 2, k), bc.BigPhi);
    return bval_i(bc, p0, ni, i, j, k);
}
template <class P0>
__device__ float bval_k(const BC& bc, const P0& p0, int ni, int nj, int nk, int i, int j, int k) {
    if (k == 0 && face_on(bc, 4))
        return bc_rule(bc.type[4], bval_j(bc, p0, ni, nj, i, j, 1), bval_j(bc, p0, ni, nj, i, j, 2), bc.BigPhi);
    if (k == nk - 1 && face_on(bc, 5))
        return bc_rule(bc.type[5], bval_j(bc, p0, ni, nj, i, j, k - 1), bval_j(bc, p0, ni, nj, i, j, k - 2),
                       bc.BigPhi);
    return bval_j(bc, p0, ni, nj, i, j, k);
}

struct P0Stage {
    const float *phin, *phi1, *out;
    long long off, sj, sk;
    int ni, nj, nk;
    float c1, c2;
    __device__ float operator()(int i, int j, int k) const {
        const long long l = off + i + sj * j + sk * k;
        const bool bnd = i == 0 || i == ni - 1 || j == 0 || j == nj - 1 || k == 0 || k == nk - 1;
        return bnd ? c1 * phin[l] + c2 * phi1[l] : out[l];
    }
};
struct P0Src {
    const float* src;
    long long off, sj, sk;
    __device__ float operator()(int i, int j, int k) const { return src[off + i + sj * j + sk * k]; }
};

__global__ void k_bc_stage(const Inst* __restrict__ inst, int ninst, long long nface, BC bc,
                           const float* __restrict__ phin, const float* __restrict__ phi1, float* out, float c1,
                           float c2) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nface) return;
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {  // last instance whose face0 <= t
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].face0 <= t) lo = mid; else hi = mid - 1;
    }
    const Inst& I = inst[lo];
    const long long r0 = t - I.face0;
    const long long nI = (long long)I.nj * I.nk, nJ = (long long)I.ni * I.nk, nK = (long long)I.ni * I.nj;
    int i, j, k;
    long long r = r0;
    if (r < 2 * nI) { i = r < nI ? 0 : I.ni - 1; r %= nI; j = (int)(r % I.nj); k = (int)(r / I.nj); }
    else if ((r -= 2 * nI) < 2 * nJ) { j = r < nJ ? 0 : I.nj - 1; r %= nJ; i = (int)(r % I.ni); k = (int)(r / I.ni); }
    else { r -= 2 * nJ; if (r >= 2 * nK) return; k = r < nK ? 0 : I.nk - 1; r %= nK; i = (int)(r % I.ni); j = (int)(r / I.ni); }
    P0Stage p0{phin, phi1, out, I.off, I.ni, (long long)I.ni * I.nj, I.ni, I.nj, I.nk, c1, c2};
    out[I.off + i + p0.sj * j + p0.sk * k] = bval_k(bc, p0, I.ni, I.nj, I.nk, i, j, k);
}

template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_bc_full(const Inst* __restrict__ inst,
        const int* __restrict__ brick_inst, int nbricks, BC bc, const float* __restrict__ src,
        float* __restrict__ dst, unsigned* err) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const auto b = brick_node<TX, TY, TZ>(inst, brick_inst, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long sj = I.ni, sk = (long long)I.ni * I.nj;
        const long long l = I.off + b.i + sj * b.j + sk * b.k;
        const bool bnd = b.i == 0 || b.i == I.ni - 1 || b.j == 0 || b.j == I.nj - 1 || b.k == 0 || b.k == I.nk - 1;
        float v;
        if (bnd) {
            P0Src p0{src, I.off, sj, sk};
            v = bval_k(bc, p0, I.ni, I.nj, I.nk, b.i, b.j, b.k);
        } else {
            v = src[l];
        }
        dst[l] = v;
        if (err && !isfinite(v)) atomicOr(err, (unsigned)kErrNonFinite);
    }
}

// ------------------------------------------------------------ Godunov |grad|
// One-sided differences (calc_RH_RN.F90:36-170) contracted with the metrics
// and the Godunov norm chosen by the sign (calc_RH_RN.F90:190-236), FP32.
__device__ __forceinline__ float godunov(const Fields& f, const float* __restrict__ d, long long l, long long sj,
                                         long long sk, int i, int j, int k, int ni, int nj, int nk, float s) {
    const float c = __ldg(d + l);
    float mas[3], men[3];
    {
        const float a = i < ni - 1 ? __ldg(d + l + 1) - c : 0.0f, bk = i > 0 ? c - __ldg(d + l - 1) : 0.0f;
        mas[0] = i < ni - 1 ? a : bk; men[0] = i > 0 ? bk : a;
    }
    {
        const float a = j < nj - 1 ? __ldg(d + l + sj) - c : 0.0f, bk = j > 0 ? c - __ldg(d + l - sj) : 0.0f;
        mas[1] = j < nj - 1 ? a : bk; men[1] = j > 0 ? bk : a;
    }
    {
        const float a = k < nk - 1 ? __ldg(d + l + sk) - c : 0.0f, bk = k > 0 ? c - __ldg(d + l - sk) : 0.0f;
        mas[2] = k < nk - 1 ? a : bk; men[2] = k > 0 ? bk : a;
    }
    float acc = 0.0f;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        const float m0 = __ldg(f.m[x] + l), m1 = __ldg(f.m[3 + x] + l), m2 = __ldg(f.m[6 + x] + l);
        const float bb = m0 * men[0] + m1 * men[1] + m2 * men[2];
        const float ff = m0 * mas[0] + m1 * mas[1] + m2 * mas[2];
        const float e = s > 0.0f ? fmaxf(fmaxf(bb, 0.0f) * fmaxf(bb, 0.0f), fminf(ff, 0.0f) * fminf(ff, 0.0f))
                                 : fmaxf(fminf(bb, 0.0f) * fminf(bb, 0.0f), fmaxf(ff, 0.0f) * fmaxf(ff, 0.0f));
        acc += e;
    }
    return sqrtf(acc);
}

// calc_sign_ini (Kang sign) with the frozen band folded in: s = 0 where
// |phi0| < eps and |grad phi0| > 0 (the lambda correction pins d to phi0).
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_sign(const Inst* __restrict__ inst,
        const int* __restrict__ brick_inst, int nbricks, Fields f, const float* __restrict__ phi0) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const auto b = brick_node<TX, TY, TZ>(inst, brick_inst, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long sj = I.ni, sk = (long long)I.ni * I.nj;
        const long long l = I.off + b.i + sj * b.j + sk * b.k;
        const float p = __ldg(phi0 + l);
        const float g = godunov(f, phi0, l, sj, sk, b.i, b.j, b.k, I.ni, I.nj, I.nk, p > 0.0f ? 1.0f : -1.0f);
        float s;
        if (p >= I.eps) s = 1.0f;
        else if (p <= -I.eps) s = -1.0f;
        else if (p != 0.0f && g > 0.0f) s = 0.0f;
        else s = p / I.eps - (float)(1.0 / kPi) * sinf((float)kPi * p / I.eps);
        f.sgn[l] = s;
    }
}

// one reinitialisation pseudo-step: d_out = d - dtau s (|grad d|_G - 1)
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_reinit(const Inst* __restrict__ inst,
        const int* __restrict__ brick_inst, int nbricks, Fields f, const float* __restrict__ din,
        float* __restrict__ dout) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const auto b = brick_node<TX, TY, TZ>(inst, brick_inst, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long sj = I.ni, sk = (long long)I.ni * I.nj;
        const long long l = I.off + b.i + sj * b.j + sk * b.k;
        const float s = __ldg(f.sgn + l);
        const float d = __ldg(din + l);
        float r = d;
        if (s != 0.0f) {
            const float g = godunov(f, din, l, sj, sk, b.i, b.j, b.k, I.ni, I.nj, I.nk, s);
            r = d - I.dtau * s * (g - 1.0f);
        }
        dout[l] = r;
    }
}

// ------------------------------------------------------------ volume (FP64)
template <int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_volume(const Inst* __restrict__ inst,
        const int* __restrict__ brick_inst, int nbricks, Fields f, const float* __restrict__ phi,
        double* __restrict__ partials) {
    constexpr int NT = TX * TY * TZ;
    __shared__ double sh[3][NT / 32];
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const auto b = brick_node<TX, TY, TZ>(inst, brick_inst, blk);
        const Inst& I = inst[b.inst];
        double K = 0.0, S = 0.0, B = 0.0;
        if (b.i < I.ni - 1 && b.j < I.nj - 1 && b.k < I.nk - 1) {
            const long long sj = I.ni, sk = (long long)I.ni * I.nj;
            const long long l = I.off + b.i + sj * b.j + sk * b.k;
            const long long o[8] = {l, l + 1, l + 1 + sj, l + sj, l + sk, l + 1 + sk, l + 1 + sj + sk, l + sj + sk};
            double P[8];
            bool allw = true, alla = true;
#pragma unroll
            for (int v = 0; v < 8; ++v) {
                P[v] = (double)__ldg(phi + o[v]);
                allw &= P[v] > kEpsSims; alla &= P[v] < -kEpsSims;
            }
            if (!alla) {
                double C[8][3];
#pragma unroll
                for (int v = 0; v < 8; ++v) {
                    C[v][0] = __ldg(f.xyz[0] + o[v]); C[v][1] = __ldg(f.xyz[1] + o[v]); C[v][2] = __ldg(f.xyz[2] + o[v]);
                }
                if (allw) B = hex_volume(C);
                else cell_analysis(P, C, &K, &S, nullptr);
            }
        }
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            K += __shfl_down_sync(0xffffffffu, K, o);
            S += __shfl_down_sync(0xffffffffu, S, o);
            B += __shfl_down_sync(0xffffffffu, B, o);
        }
        if (lane == 0) { sh[0][w] = K; sh[1][w] = S; sh[2][w] = B; }
        __syncthreads();
        if (threadIdx.x < 3) {
            double acc = 0.0;
            for (int q = 0; q < NT / 32; ++q) acc += sh[threadIdx.x][q];
            partials[3 * (long long)blk + threadIdx.x] = acc;
        }
        __syncthreads();
    }
}

// one block per instance folds its bricks' partials in brick order
__global__ void __launch_bounds__(256) k_volume_final(const Inst* __restrict__ inst, int ninst, int nbricks,
                                                      const double* __restrict__ partials, double* __restrict__ vols) {
    const int b = blockIdx.x;
    if (b >= ninst) return;
    const int first = inst[b].brick0;
    const int last = b + 1 < ninst ? inst[b + 1].brick0 : nbricks;
    __shared__ double sh[3][8];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int q = first + threadIdx.x; q < last; q += 256)
        for (int c = 0; c < 3; ++c) acc[c] += partials[3 * (long long)q + c];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int c = 0; c < 3; ++c) {
        double v = acc[c];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[c][w] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double v[3];
        for (int c = 0; c < 3; ++c) {
            double a = 0.0;
            for (int q = 0; q < 8; ++q) a += sh[c][q];
            v[c] = a;
        }
        vols[4 * b] = v[0]; vols[4 * b + 1] = v[1]; vols[4 * b + 2] = v[2];
        vols[4 * b + 3] = v[0] + v[1] + v[2];
    }
}

template <template <int, int, int> class Fn, class... A>
void dispatch(int shape, A... a) {
    switch (shape) {
    case 0: Fn<32, 4, 2>::run(a...); break;
    case 1: Fn<32, 8, 1>::run(a...); break;
    case 2: Fn<64, 4, 1>::run(a...); break;
    case 3: Fn<32, 2, 4>::run(a...); break;
    default: Fn<128, 2, 1>::run(a...); break;
    }
}

#define LSM_BATCH_RUNNER(NAME, KERNEL, PARAMS, ARGS)                                     \
    template <int TX, int TY, int TZ>                                                    \
    struct NAME {                                                                         \
        static void run PARAMS {                                                          \
            ProfScope ps_(#KERNEL, s);                                                    \
            KERNEL<TX, TY, TZ><<<grid, TX * TY * TZ, 0, s>>> ARGS;                        \
        }                                                                                 \
    };

LSM_BATCH_RUNNER(RunContra, k_contra,
                 (int grid, const Inst* inst, const int* bi, int nb, Fields f, float a, float b, float c, cudaStream_t s),
                 (inst, bi, nb, f, a, b, c))
LSM_BATCH_RUNNER(RunStage, k_stage,
                 (int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* pn, const float* p1,
                  float* out, float c1, float c2, float c3, cudaStream_t s),
                 (inst, bi, nb, f, pn, p1, out, c1, c2, c3))
LSM_BATCH_RUNNER(RunBcFull, k_bc_full,
                 (int grid, const Inst* inst, const int* bi, int nb, BC bc, const float* src, float* dst, unsigned* err,
                  cudaStream_t s),
                 (inst, bi, nb, bc, src, dst, err))
LSM_BATCH_RUNNER(RunSign, k_sign,
                 (int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* p0, cudaStream_t s),
                 (inst, bi, nb, f, p0))
LSM_BATCH_RUNNER(RunReinit, k_reinit,
                 (int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* din, float* dout,
                  cudaStream_t s),
                 (inst, bi, nb, f, din, dout))
LSM_BATCH_RUNNER(RunVolume, k_volume,
                 (int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* phi, double* part,
                  cudaStream_t s),
                 (inst, bi, nb, f, phi, part))

template <int TX, int TY, int TZ>
struct Occupancy {
    static void run(int kernel, int* out) {
        const int nt = TX * TY * TZ;
        switch (kernel) {
        case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_stage<TX, TY, TZ>, nt, 0); break;
        case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_reinit<TX, TY, TZ>, nt, 0); break;
        default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_volume<TX, TY, TZ>, nt, 0); break;
        }
    }
};

}  // namespace

void contra(int shape, int grid, const Inst* inst, const int* bi, int nb, Fields f, float dcm[3], cudaStream_t s) {
    dispatch<RunContra>(shape, grid, inst, bi, nb, f, dcm[0], dcm[1], dcm[2], s);
}
void stage(int shape, int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* phin,
           const float* phi1, float* out, float c1, float c2, float c3, cudaStream_t s) {
    dispatch<RunStage>(shape, grid, inst, bi, nb, f, phin, phi1, out, c1, c2, c3, s);
}
void bc_stage(const Inst* inst, int ninst, long long nface, Fields f, BC bc, const float* phin, const float* phi1,
              float* out, float c1, float c2, cudaStream_t s) {
    (void)f;
    ProfScope ps_("k_bc_stage", s);
    k_bc_stage<<<(unsigned)((nface + 255) / 256), 256, 0, s>>>(inst, ninst, nface, bc, phin, phi1, out, c1, c2);
}
void bc_full(int shape, int grid, const Inst* inst, const int* bi, int nb, BC bc, const float* src, float* dst,
             unsigned* err, cudaStream_t s) {
    dispatch<RunBcFull>(shape, grid, inst, bi, nb, bc, src, dst, err, s);
}
void sign(int shape, int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* phi0, cudaStream_t s) {
    dispatch<RunSign>(shape, grid, inst, bi, nb, f, phi0, s);
}
void reinit(int shape, int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* din, float* dout,
            cudaStream_t s) {
    dispatch<RunReinit>(shape, grid, inst, bi, nb, f, din, dout, s);
}
void volume(int shape, int grid, const Inst* inst, const int* bi, int nb, Fields f, const float* phi,
            double* partials, cudaStream_t s) {
    dispatch<RunVolume>(shape, grid, inst, bi, nb, f, phi, partials, s);
}
void volume_final(const Inst* inst, int ninst, const int* bi, int nb, const double* partials, double* vols,
                  cudaStream_t s) {
    (void)bi;
    ProfScope ps_("k_volume_final", s);
    k_volume_final<<<ninst, 256, 0, s>>>(inst, ninst, nb, partials, vols);
}
int max_blocks_per_sm(int shape, int kernel) {
    int n = 0;
    dispatch<Occupancy>(shape, kernel, &n);
    return n;
}

}  // namespace batch
}  // namespace lsm
