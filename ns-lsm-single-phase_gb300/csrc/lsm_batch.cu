// lsm_batch.cu -- batched kernels of the level-set transport step, forward
// and adjoint, templated on the scalar type (FP32 for throughput, FP64 for
// gradient checks).
//
// Every launch covers every instance of the batch with persistent CTAs
// (grid = SMs x resident CTAs) walking a table of tiles, each tile inside
// one instance:
//  - brick tables (TX x TY x TZ nodes, one thread per node; the autotuned
//    forward shape): contra, volume, boundary passes, and the brick
//    variants of the pseudo-step;
//  - adjoint-map tiles (adj_shape): the stencil passes that march in k
//    over 32 x 8 columns (RK stage, pseudo-steps, the reverse pseudo-step
//    from stored coefficients), march rows / lines (stage adjoint) or an
//    overlapped 32 x kReinRY tile (reverse pseudo-step recomputing its
//    coefficients).
// Per-node algorithmic traffic (FP32 words): contra 15 (u 3, metrics 9;
// W 3), RK stage 5/6/6 (phi_prev, phi^n, W 3; phi), pseudo-step 12 (d, s,
// metrics 9; d) or 18 recorded (+ six adjoint coefficients), volume 3 (phi
// + 64-bit fixed-point cell volume).
//
// Arithmetic: the reference's formulas rearranged for the GPU (one division
// per WENO3 reconstruction); the water volume sums FP64 hexahedron volumes
// of the bulk water cells and the interface cells' shares (in the stencil
// precision) with exact 64-bit fixed-point sums.  The reinitialisation uses
// the closed form of the reference's method-0 lambda correction: with
// lambda = -(d1 - phi0) / (dtau delta |grad phi0|) the correction dtau
// lambda delta |grad phi0| returns d to phi0 wherever delta(phi0) |grad
// phi0| != 0, i.e. |phi0| < eps; those nodes are folded into the sign field
// as s = 0 (no update) and a pseudo-step reads only d, s and the metrics.
//
// Adjoint: hand-written reverse kernels gathering (no atomics): bcond_lsm
// faces in reverse order; the WENO3 stage with the upwind side of every
// face frozen from the forward pass and the nonlinear weights
// differentiated; the Godunov pseudo-step with its max / clip selections
// and the sign field frozen (a 7-point stencil on lam with coefficients the
// recorded forward step stored, or recomputed from its input); the
// contravariant-velocity chain rule.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "lsm_batch.cuh"
#include "lsm_common.cuh"
#include "lsm_kernels.h"
#include "lsm_volume_dev.cuh"

namespace lsm {
namespace batch {
namespace {

// ------------------------------------------------------------ scalar helpers
template <typename T> __device__ __forceinline__ T vmax(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T vmin(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T vdiv(T a, T b) { return a / b; }
template <> __device__ __forceinline__ float vdiv<float>(float a, float b) { return __fdividef(a, b); }
template <typename T> __device__ __forceinline__ T vfma(T a, T b, T c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float vfma<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <typename T> __device__ __forceinline__ T vsqrt(T a) { return sqrt(a); }
template <> __device__ __forceinline__ float vsqrt<float>(float a) { return sqrtf(a); }
template <typename T> __device__ __forceinline__ T vrsqrt(T a) { return T(1) / sqrt(a); }
template <> __device__ __forceinline__ float vrsqrt<float>(float a) { return rsqrtf(a); }
template <typename T> __device__ __forceinline__ T vsin(T a) { return sin(a); }
template <> __device__ __forceinline__ float vsin<float>(float a) { return sinf(a); }
template <typename T> __device__ __forceinline__ bool vfinite(T a) { return isfinite(a); }
// per-instance parameter in the kernel's precision
template <typename T> __device__ __forceinline__ T ipar(float f, double d);
template <> __device__ __forceinline__ float ipar<float>(float f, double) { return f; }
template <> __device__ __forceinline__ double ipar<double>(float, double d) { return d; }

// ------------------------------------------------------------ node walks
struct Node {
    int inst, i, j, k;
    bool valid;
};

template <int TX, int TY, int TZ>
__device__ __forceinline__ Node brick_node(const Inst* __restrict__ inst, const Brick* __restrict__ bricks, int blk) {
    Node b;
    const int4 bk = __ldg(reinterpret_cast<const int4*>(bricks) + blk);
    b.inst = bk.x;
    const Inst& I = inst[b.inst];
    const int t = threadIdx.x;
    b.i = bk.y * TX + t % TX;
    b.j = bk.z * TY + (t / TX) % TY;
    b.k = bk.w * TZ + t / (TX * TY);
    b.valid = b.i < I.ni && b.j < I.nj && b.k < I.nk;
    return b;
}

// flat walk: node t of the packed arrays -> instance and (i, j, k)
__device__ __forceinline__ bool flat_node(const Flat& fl, long long t, Node* nd) {
    if (t >= fl.n) return false;
    int lo = 0, hi = fl.ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (fl.offs[mid] <= t) lo = mid; else hi = mid - 1;
    }
    const Inst& I = fl.inst[lo];
    const long long r = t - I.off;
    nd->inst = lo;
    nd->i = (int)(r % I.ni);
    nd->j = (int)((r / I.ni) % I.nj);
    nd->k = (int)(r / ((long long)I.ni * I.nj));
    nd->valid = true;
    return true;
}

// Brick `blk` of adjoint map `map`: instance and first node of its tile.
struct ABrick {
    int inst, i0, j0, k0;
};
__device__ __forceinline__ ABrick adj_brick(const Brick* __restrict__ bmap, int map, int blk) {
    const int4 bk = __ldg(reinterpret_cast<const int4*>(bmap) + blk);
    const AdjShape sh = adj_shape(map);
    ABrick b;
    b.inst = bk.x;
    b.i0 = bk.y * sh.ox;
    b.j0 = bk.z * sh.oy;
    b.k0 = bk.w * sh.oz;
    return b;
}

// ------------------------------------------------------------ WENO3
// GetWENO3Reconstruction (src/AdvectionMethods.F90:195-245) on an oriented
// stencil (fL, fC, fR): weights 2/3, 1/3 over (beta + 1e-6)^2, rearranged to
// one division: w0 = 2 t1^2 / (2 t1^2 + t0^2), Phi = u1 + w0 (u0 - u1).
template <typename T>
__device__ __forceinline__ T rec3(T fL, T fC, T fR) {
    const T b0 = (fC - fR) * (fC - fR), b1 = (fL - fC) * (fL - fC);
    const T t0 = b0 + T(1.0e-6), t1 = b1 + T(1.0e-6);
    const T a0 = T(2) * t1 * t1, a1 = t0 * t0;
    const T w0 = vdiv(a0, a0 + a1);
    const T u1 = T(1.5) * fC - T(0.5) * fL;
    return vfma(w0, T(0.5) * (fL + fR) - fC, u1);
}

// Phi_{+1/2} - Phi_{-1/2} along one axis for the node with stencil
// (m2, m1, c, p1, p2); lo/hi force the reference's one-sided stencils on
// the first / last interior node (calc_RH_AD_WENO3.F90:201-245).
template <typename T>
__device__ __forceinline__ T weno_diff(T m2, T m1, T c, T p1, T p2, T w, bool lo, bool hi) {
    // the stencils are selected first so that each face costs one
    // reconstruction (no evaluation of the branch not taken)
    const bool up = w > T(0);
    const bool P = up || hi, M = up && !lo;
    const T fp = rec3(P ? m1 : p2, P ? c : p1, P ? p1 : c);
    const T fm = rec3(M ? m2 : p1, M ? m1 : c, M ? c : m1);
    return fp - fm;
}

// ------------------------------------------------------------ contra
template <typename T, int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_contra(const Inst* __restrict__ inst,
        const Brick* __restrict__ bricks, int nbricks, FieldsT<T> f) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const Node b = brick_node<TX, TY, TZ>(inst, bricks, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long l = I.off + b.i + (long long)I.ni * (b.j + (long long)I.nj * b.k);
        const T u = f.u[0][l], v = f.u[1][l], w = f.u[2][l];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const T c = f.m[3 * m][l] * u + f.m[3 * m + 1][l] * v + f.m[3 * m + 2][l] * w;
            f.W[m][l] = ipar<T>(I.dt, I.dt64) * c;
        }
    }
}

// FP64 contravariant velocity x dt of one instance from the FP64 metrics
// (m64: 9 arrays) and velocity (u64: 3 arrays), the same formula as
// k_contra; packed base arrays, `off` the instance's first node
__global__ void k_w64(long long off, long long n, double dt, const double* const* __restrict__ m64,
                      const double* const* __restrict__ u64, double* const* __restrict__ w64) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long l = off + t;
        const double u = u64[0][l], v = u64[1][l], w = u64[2][l];
#pragma unroll
        for (int m = 0; m < 3; ++m) w64[m][l] = dt * (m64[3 * m][l] * u + m64[3 * m + 1][l] * v + m64[3 * m + 2][l] * w);
    }
}

// ------------------------------------------------------------ RK stage

// The stage output c1 phi^n + c2 phi1 - c3 R at node l.  FP32 batches that
// keep the FP64 contravariant velocity combine the nodes within kBand64 eps
// of the interface in FP64: R = sum_m W64_m D_m over the FP32 differences D.
template <typename T>
__device__ __forceinline__ T stage_out(const FieldsT<T>& f, long long l, bool interior, T c1, T c2, T c3, T pn, T w2,
                                       T R, T D0, T D1, T D2, T eps) {
    if constexpr (sizeof(T) == 4) {
        if (interior && f.W64[0] && fabsf(w2) < kBand64 * eps) {
            const double r = __ldg(f.W64[0] + l) * (double)D0 + __ldg(f.W64[1] + l) * (double)D1 +
                             __ldg(f.W64[2] + l) * (double)D2;
            return (T)((double)c1 * (double)pn + (double)c2 * (double)w2 - (double)c3 * r);
        }
    }
    return c1 * pn + c2 * w2 - c3 * R;
}

// RK stage on the tiles of adjoint map 2 (32 x 8 columns marching 32 planes
// in k).  Each plane of phi1 is staged in shared memory with a two-node
// halo in x and y (double-buffered, one barrier per plane: the x and y
// stencils read it there); the z stencil is a five-plane register window.
// Loads per node: phi1 once (plus the halo share), phi^n and W.  Interior
// nodes: out = c1 phi^n + c2 phi1 - c3 sum_m W_m (Phi+ - Phi-)_m
// (calc_RH_AD_WENO3 x aj dt, the x term first); other nodes get R = 0 and
// their faces from bcond_lsm afterwards.  Halo slots: threads 0..127 hold the y-halo rows
// -2, -1, 8, 9 of the tile, threads 128..159 the x-halo columns -2, -1, 32,
// 33 (the cross stencil needs no corners).
// The z face k-1/2 of a node is the z face k+1/2 of the node below it with
// the same stencil whenever their upwind choices agree (M at k equals P at
// k - 1): that reconstruction is carried from the previous plane, and a
// warp skips the recomputation when all its lanes can reuse it.
constexpr int kStSX = 36, kStSY = 12;
template <typename T>
__global__ void __launch_bounds__(256) k_stage_z(const Inst* __restrict__ inst, const Brick* __restrict__ bmap,
        int nb, FieldsT<T> f, const T* __restrict__ phin, const T* __restrict__ phi1, T* __restrict__ out, T c1, T c2,
        T c3) {
    __shared__ T pl[2][kStSY][kStSX];
    const unsigned FM = 0xffffffffu;
    const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
    int hx = 0, hy = 0;
    if (t < 128) {
        const int r = t >> 5;
        hy = r < 2 ? r - 2 : r + 6;
        hx = tx;
    } else if (t < 160) {
        const int u = t - 128, c = u & 3;
        hy = u >> 2;
        hx = c < 2 ? c - 2 : c + 30;
    }
    const bool has_h = t < 160;
    unsigned ph = 0;   // buffer parity, continuous over the tiles of this CTA
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 2, blk);
        const Inst& I = inst[ab.inst];
        const int ni = I.ni, nj = I.nj, nk = I.nk;
        const long long sk = (long long)ni * nj;
        const int i = ab.i0 + tx, j = ab.j0 + ty;
        const int k0 = ab.k0, k1 = min(k0 + adj_shape(2).oz, nk);
        const bool col = i < ni && j < nj;
        const int gi = ab.i0 + hx, gj = ab.j0 + hy;
        const bool hok = has_h && gi >= 0 && gi < ni && gj >= 0 && gj < nj;
        const long long cb = I.off + i + (long long)ni * j;
        const long long hb = I.off + gi + (long long)ni * gj;
        const bool ij_int = i > 0 && i < ni - 1 && j > 0 && j < nj - 1;
        auto own = [&](int k) { return col && k >= 0 && k < nk ? __ldg(phi1 + cb + sk * k) : T(0); };
        T w0 = own(k0 - 2), w1 = own(k0 - 1), w2 = own(k0), w3 = own(k0 + 1), w4 = own(k0 + 2);
        T hv = hok ? __ldg(phi1 + hb + sk * k0) : T(0);
        T W0 = T(0), W1 = T(0), W2 = T(0), pn = T(0);
        if (col) {
            const long long l = cb + sk * k0;
            W0 = __ldg(f.W[0] + l);
            W1 = __ldg(f.W[1] + l);
            W2 = __ldg(f.W[2] + l);
            pn = __ldg(phin + l);
        }
        // the z face k - 1/2 carried from the previous plane (Pz: its stencil choice)
        T fpz = T(0);
        bool Pz = false, have = false;
        for (int k = k0; k < k1; ++k) {
            // loads of plane k + 1 (window plane k + 3) go out first
            const bool nx = k + 1 < k1;
            const T w5 = nx ? own(k + 3) : T(0);
            T hvn = T(0), W0n = T(0), W1n = T(0), W2n = T(0), pnn = T(0);
            if (hok && nx) hvn = __ldg(phi1 + hb + sk * (k + 1));
            if (col && nx) {
                const long long l = cb + sk * (k + 1);
                W0n = __ldg(f.W[0] + l);
                W1n = __ldg(f.W[1] + l);
                W2n = __ldg(f.W[2] + l);
                pnn = __ldg(phin + l);
            }
            T (*P)[kStSX] = pl[ph & 1u];
            ++ph;
            P[ty + 2][tx + 2] = w2;
            if (has_h) P[hy + 2][hx + 2] = hv;
            __syncthreads();
            const bool interior = col && ij_int && k > 0 && k < nk - 1;
            // z stencil choices (weno_diff's P and M)
            const bool upz = W2 > T(0);
            const bool Pk = upz || k == nk - 2, Mk = upz && k != 1;
            const bool reuse = !interior || (have && Mk == Pz);
            const bool all_reuse = __all_sync(FM, reuse);
            if (col) {
                T R = T(0);
                T D0 = T(0), D1 = T(0), D2 = T(0);
                if (interior) {
                    const int x = tx + 2, y = ty + 2;
                    // the outer stencil values are read unconditionally: every
                    // slot of the cross is written each plane (zero outside the
                    // grid), and weno_diff leaves m2 unused at the first
                    // interior node and p2 at the last
                    D0 = weno_diff(P[y][x - 2], P[y][x - 1], w2, P[y][x + 1], P[y][x + 2], W0, i == 1, i == ni - 2);
                    D1 = weno_diff(P[y - 2][x], P[y - 1][x], w2, P[y + 1][x], P[y + 2][x], W1, j == 1, j == nj - 2);
                    const T p2 = w4;
                    const T fp = rec3(Pk ? w1 : p2, Pk ? w2 : w3, Pk ? w3 : w2);
                    T fm = fpz;
                    if (!all_reuse) {
                        const T g = rec3(Mk ? w0 : w3, Mk ? w1 : w2, Mk ? w2 : w1);
                        if (!reuse) fm = g;
                    }
                    D2 = fp - fm;
                    R = W0 * D0;
                    R = vfma(W1, D1, R);
                    R = vfma(W2, D2, R);
                    fpz = fp;
                    Pz = Pk;
                }
                out[cb + sk * k] = stage_out(f, cb + sk * k, interior, c1, c2, c3, pn, w2, R, D0, D1, D2,
                                             ipar<T>(I.eps, I.eps64));
            }
            have = interior;
            w0 = w1;
            w1 = w2;
            w2 = w3;
            w3 = w4;
            w4 = w5;
            hv = hvn;
            W0 = W0n;
            W1 = W1n;
            W2 = W2n;
            pn = pnn;
        }
    }
}

// ------------------------------------------------------------ TMA staging
// Tensor-memory-accelerator copies of one tile per plane into shared memory
// (cp.async.bulk.tensor), completion tracked by an mbarrier whose phase the
// threads wait on, each wait bounded (kErrTimeout after kTmaSpins polls).
constexpr int kTmaSpins = 1 << 20;
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for phase `parity` of `bar`; false when it gave up
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    for (int it = 0; it < kTmaSpins; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// 4-D tiled load (x, y, z, array) of the map's box into dst, completing on bar
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y, int z, int a,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(a), "r"(smem_addr(bar))
        : "memory");
}

// RK stage (FP32) with the plane tiles staged by TMA: the same arithmetic,
// tiles and z window as k_stage_z, for a batch of one instance whose rows
// are whole 16-byte units (ni a multiple of 4).  The stage input phi1 is
// array `a_in` of the 4-D tensor map `tm` ((ni, nj, nk, arrays), the
// arena's arrays ld apart).  Per plane one thread issues the copy of a 40 x
// 12 box starting at (i0 - 4, j0 - 2): x rounded down to a 16-byte boundary,
// a two-node halo on every side, the out-of-range part zero-filled by the
// copy engine.  Three buffers; the copy of plane k + 2 is issued (after the
// plane barrier that frees its buffer) while plane k is computed.
constexpr int kTmaBX = 40, kTmaBY = 12, kTmaBuf = 3;
__global__ void __launch_bounds__(256) k_stage_tma(const __grid_constant__ CUtensorMap tm, int a_in,
        const Inst* __restrict__ inst, const Brick* __restrict__ bmap, int nb, FieldsT<float> f,
        const float* __restrict__ phin, const float* __restrict__ phi1, float* __restrict__ out, float c1, float c2,
        float c3, unsigned* __restrict__ err) {
    __shared__ __align__(128) float pl[kTmaBuf][kTmaBY][kTmaBX];
    __shared__ __align__(8) unsigned long long bar[kTmaBuf];
    __shared__ int abort_flag;
    const unsigned FM = 0xffffffffu;
    const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
    constexpr unsigned kBytes = kTmaBX * kTmaBY * sizeof(float);
    if (t == 0) {
        for (int b = 0; b < kTmaBuf; ++b) mbar_init(&bar[b], 1);
        abort_flag = 0;
        mbar_fence_init();
    }
    __syncthreads();
    unsigned issued = 0, used = 0;   // copies issued / planes consumed by this CTA (same on every thread)
    const Inst& I = inst[0];
    const int ni = I.ni, nj = I.nj, nk = I.nk;
    const long long sk = (long long)ni * nj;
    auto issue = [&](int i0, int j0, int k) {
        if (t == 0) {
            unsigned long long* b = &bar[issued % kTmaBuf];
            mbar_expect_tx(b, kBytes);
            tma_load_4d(&pl[issued % kTmaBuf][0][0], &tm, i0 - 4, j0 - 2, k, a_in, b);
        }
        ++issued;
    };
    bool aborted = false;
    for (int blk = blockIdx.x; blk < nb && !aborted; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 2, blk);
        const int i = ab.i0 + tx, j = ab.j0 + ty;
        const int k0 = ab.k0, k1 = min(k0 + adj_shape(2).oz, nk);
        const bool col = i < ni && j < nj;
        const long long cb = i + (long long)ni * j;
        const bool ij_int = i > 0 && i < ni - 1 && j > 0 && j < nj - 1;
        // the first two planes of the tile
        issue(ab.i0, ab.j0, k0);
        if (k0 + 1 < k1) issue(ab.i0, ab.j0, k0 + 1);
        auto own = [&](int k) { return col && k >= 0 && k < nk ? __ldg(phi1 + cb + sk * k) : 0.f; };
        float w0 = own(k0 - 2), w1 = own(k0 - 1), w2 = own(k0), w3 = own(k0 + 1), w4 = own(k0 + 2);
        float W0 = 0.f, W1 = 0.f, W2 = 0.f, pn = 0.f;
        if (col) {
            const long long l = cb + sk * k0;
            W0 = __ldg(f.W[0] + l);
            W1 = __ldg(f.W[1] + l);
            W2 = __ldg(f.W[2] + l);
            pn = __ldg(phin + l);
        }
        float fpz = 0.f;
        bool Pz = false, have = false;
        for (int k = k0; k < k1; ++k) {
            const bool nx = k + 1 < k1;
            const float w5 = nx ? own(k + 3) : 0.f;
            float W0n = 0.f, W1n = 0.f, W2n = 0.f, pnn = 0.f;
            if (col && nx) {
                const long long l = cb + sk * (k + 1);
                W0n = __ldg(f.W[0] + l);
                W1n = __ldg(f.W[1] + l);
                W2n = __ldg(f.W[2] + l);
                pnn = __ldg(phin + l);
            }
            const unsigned slot = used % kTmaBuf, par = (used / kTmaBuf) & 1u;
            // a wait that gave up leaves `used` at the copy still owed
            if (mbar_wait(&bar[slot], par)) ++used;
            else abort_flag = 1;
            const float (*P)[kTmaBX] = pl[slot];
            const bool interior = col && ij_int && k > 0 && k < nk - 1;
            const bool upz = W2 > 0.f;
            const bool Pk = upz || k == nk - 2, Mk = upz && k != 1;
            const bool reuse = !interior || (have && Mk == Pz);
            const bool all_reuse = __all_sync(FM, reuse);
            if (col) {
                float R = 0.f;
                float D0 = 0.f, D1 = 0.f, D2 = 0.f;
                if (interior) {
                    const int x = tx + 4, y = ty + 2;
                    // the outer stencil values are read unconditionally: the
                    // tile always holds them (zero-filled outside the grid),
                    // and weno_diff leaves m2 unused at the first interior node
                    // and p2 at the last
                    D0 = weno_diff(P[y][x - 2], P[y][x - 1], w2, P[y][x + 1], P[y][x + 2], W0, i == 1, i == ni - 2);
                    D1 = weno_diff(P[y - 2][x], P[y - 1][x], w2, P[y + 1][x], P[y + 2][x], W1, j == 1, j == nj - 2);
                    const float p2 = w4;
                    const float fp = rec3(Pk ? w1 : p2, Pk ? w2 : w3, Pk ? w3 : w2);
                    float fm = fpz;
                    if (!all_reuse) {
                        const float g = rec3(Mk ? w0 : w3, Mk ? w1 : w2, Mk ? w2 : w1);
                        if (!reuse) fm = g;
                    }
                    D2 = fp - fm;
                    R = W0 * D0;
                    R = vfma(W1, D1, R);
                    R = vfma(W2, D2, R);
                    fpz = fp;
                    Pz = Pk;
                }
                out[cb + sk * k] = stage_out(f, cb + sk * k, interior, c1, c2, c3, pn, w2, R, D0, D1, D2, I.eps);
            }
            have = interior;
            // every thread is done with this plane's buffer: it takes plane k + 2
            __syncthreads();
            if (abort_flag) {
                aborted = true;
                break;
            }
            if (k + 2 < k1) issue(ab.i0, ab.j0, k + 2);
            w0 = w1;
            w1 = w2;
            w2 = w3;
            w3 = w4;
            w4 = w5;
            W0 = W0n;
            W1 = W1n;
            W2 = W2n;
            pn = pnn;
        }
    }
    if (aborted && t == 0) {
        atomicOr(err, (unsigned)kErrTimeout);
        // let the copies still in flight land before the CTA's shared memory
        // goes away (each wait bounded again)
        while (used < issued) {
            mbar_wait(&bar[used % kTmaBuf], (used / kTmaBuf) & 1u);
            ++used;
        }
    }
}

// ------------------------------------------------------------ bcond_lsm
template <typename T>
__device__ __forceinline__ T bc_rule(int type, T n1, T n2, float BigPhi) {
    if (type == 0) return n1;
    if (type == 1) return fabs(n2) >= T(BigPhi) ? n1 : T(4.0 / 3.0) * n1 - T(1.0 / 3.0) * n2;
    return T(2) * n1 - n2;  // type 2 on the im face
}
__device__ __forceinline__ bool face_on(const BC& bc, int face) {
    const int t = bc.type[face];
    return t == 0 || t == 1 || (t == 2 && face == 1);
}

template <typename T, class P0>
__device__ T bval_i(const BC& bc, const P0& p0, int ni, int i, int j, int k) {
    if (i == 0 && face_on(bc, 0)) return bc_rule<T>(bc.type[0], p0(1, j, k), p0(2, j, k), bc.BigPhi);
    if (i == ni - 1 && face_on(bc, 1)) return bc_rule<T>(bc.type[1], p0(i - 1, j, k), p0(i - 2, j, k), bc.BigPhi);
    return p0(i, j, k);
}
template <typename T, class P0>
__device__ T bval_j(const BC& bc, const P0& p0, int ni, int nj, int i, int j, int k) {
    if (j == 0 && face_on(bc, 2))
        return bc_rule<T>(bc.type[2], bval_i<T>(bc, p0, ni, i, 1, k), bval_i<T>(bc, p0, ni, i, 2, k), bc.BigPhi);
    if (j == nj - 1 && face_on(bc, 3))
        return bc_rule<T>(bc.type[3], bval_i<T>(bc, p0, ni, i, j - 1, k), bval_i<T>(bc, p0, ni, i, j - 2, k),
                          bc.BigPhi);
    return bval_i<T>(bc, p0, ni, i, j, k);
}
template <typename T, class P0>
__device__ T bval_k(const BC& bc, const P0& p0, int ni, int nj, int nk, int i, int j, int k) {
    if (k == 0 && face_on(bc, 4))
        return bc_rule<T>(bc.type[4], bval_j<T>(bc, p0, ni, nj, i, j, 1), bval_j<T>(bc, p0, ni, nj, i, j, 2),
                          bc.BigPhi);
    if (k == nk - 1 && face_on(bc, 5))
        return bc_rule<T>(bc.type[5], bval_j<T>(bc, p0, ni, nj, i, j, k - 1), bval_j<T>(bc, p0, ni, nj, i, j, k - 2),
                          bc.BigPhi);
    return bval_j<T>(bc, p0, ni, nj, i, j, k);
}

template <typename T>
struct P0Stage {
    const T *phin, *phi1, *out;
    long long off, sj, sk;
    int ni, nj, nk;
    T c1, c2;
    __device__ T operator()(int i, int j, int k) const {
        const long long l = off + i + sj * j + sk * k;
        const bool bnd = i == 0 || i == ni - 1 || j == 0 || j == nj - 1 || k == 0 || k == nk - 1;
        return bnd ? c1 * phin[l] + c2 * phi1[l] : out[l];
    }
};
template <typename T>
struct P0Src {
    const T* src;
    long long off, sj, sk;
    __device__ T operator()(int i, int j, int k) const { return src[off + i + sj * j + sk * k]; }
};

__device__ __forceinline__ int face_instance(const Inst* __restrict__ inst, int ninst, long long t) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (inst[mid].face0 <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool face_coords(const Inst& I, long long r, int* pi, int* pj, int* pk) {
    const long long nI = (long long)I.nj * I.nk, nJ = (long long)I.ni * I.nk, nK = (long long)I.ni * I.nj;
    if (r < 2 * nI) { *pi = r < nI ? 0 : I.ni - 1; r %= nI; *pj = (int)(r % I.nj); *pk = (int)(r / I.nj); return true; }
    r -= 2 * nI;
    if (r < 2 * nJ) { *pj = r < nJ ? 0 : I.nj - 1; r %= nJ; *pi = (int)(r % I.ni); *pk = (int)(r / I.ni); return true; }
    r -= 2 * nJ;
    if (r >= 2 * nK) return false;
    *pk = r < nK ? 0 : I.nk - 1; r %= nK; *pi = (int)(r % I.ni); *pj = (int)(r / I.ni);
    return true;
}

template <typename T>
__global__ void k_bc_stage(const Inst* __restrict__ inst, int ninst, long long nface, BC bc,
                           const T* __restrict__ phin, const T* __restrict__ phi1, T* out, T c1, T c2) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nface) return;
    const Inst& I = inst[face_instance(inst, ninst, t)];
    int i, j, k;
    if (!face_coords(I, t - I.face0, &i, &j, &k)) return;
    P0Stage<T> p0{phin, phi1, out, I.off, I.ni, (long long)I.ni * I.nj, I.ni, I.nj, I.nk, c1, c2};
    out[I.off + i + p0.sj * j + p0.sk * k] = bval_k<T>(bc, p0, I.ni, I.nj, I.nk, i, j, k);
}

// bcond_lsm on the faces of dst from the pre-BC field src (interior nodes
// of dst already hold src)
template <typename T>
__global__ void k_bc_faces(const Inst* __restrict__ inst, int ninst, long long nface, BC bc, const T* __restrict__ src,
                           T* __restrict__ dst, unsigned* err) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nface) return;
    const Inst& I = inst[face_instance(inst, ninst, t)];
    int i, j, k;
    if (!face_coords(I, t - I.face0, &i, &j, &k)) return;
    const long long sj = I.ni, sk = (long long)I.ni * I.nj;
    P0Src<T> p0{src, I.off, sj, sk};
    const T v = bval_k<T>(bc, p0, I.ni, I.nj, I.nk, i, j, k);
    dst[I.off + i + sj * j + sk * k] = v;
    if (err && !vfinite(v)) atomicOr(err, (unsigned)kErrNonFinite);
}

template <typename T, int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_bc_full(const Inst* __restrict__ inst,
        const Brick* __restrict__ bricks, int nbricks, BC bc, const T* __restrict__ src, T* __restrict__ dst,
        unsigned* err) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const Node b = brick_node<TX, TY, TZ>(inst, bricks, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long sj = I.ni, sk = (long long)I.ni * I.nj;
        const long long l = I.off + b.i + sj * b.j + sk * b.k;
        const bool bnd = b.i == 0 || b.i == I.ni - 1 || b.j == 0 || b.j == I.nj - 1 || b.k == 0 || b.k == I.nk - 1;
        T v;
        if (bnd) {
            P0Src<T> p0{src, I.off, sj, sk};
            v = bval_k<T>(bc, p0, I.ni, I.nj, I.nk, b.i, b.j, b.k);
        } else {
            v = src[l];
        }
        dst[l] = v;
        if (err && !vfinite(v)) atomicOr(err, (unsigned)kErrNonFinite);
    }
}

// ------------------------------------------------------------ Godunov |grad|
// One-sided differences (calc_RH_RN.F90:36-170) along one axis: mas
// (forward) and men (backward); on a physical face both take the one
// available difference.
template <typename T>
__device__ __forceinline__ void one_sided(const T* __restrict__ d, long long l, long long s, int c, int n, T* mas,
                                          T* men) {
    const T x = __ldg(d + l);
    const T a = c < n - 1 ? __ldg(d + l + s) - x : T(0);
    const T b = c > 0 ? x - __ldg(d + l - s) : T(0);
    *mas = c < n - 1 ? a : b;
    *men = c > 0 ? b : a;
}

template <typename T>
__device__ __forceinline__ void godunov_diffs(const T* __restrict__ d, const Inst& I, long long l, int i, int j, int k,
                                              T (&mas)[3], T (&men)[3]) {
    one_sided(d, l, 1, i, I.ni, &mas[0], &men[0]);
    one_sided(d, l, (long long)I.ni, j, I.nj, &mas[1], &men[1]);
    one_sided(d, l, (long long)I.ni * I.nj, k, I.nk, &mas[2], &men[2]);
}

// Godunov norm (calc_RH_RN.F90:190-236) chosen by the sign s
template <typename T>
__device__ __forceinline__ T godunov(const FieldsT<T>& f, const T* __restrict__ d, const Inst& I, long long l, int i,
                                     int j, int k, T s) {
    T mas[3], men[3];
    godunov_diffs(d, I, l, i, j, k, mas, men);
    T acc = T(0);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        const T m0 = __ldg(f.m[x] + l), m1 = __ldg(f.m[3 + x] + l), m2 = __ldg(f.m[6 + x] + l);
        const T bb = m0 * men[0] + m1 * men[1] + m2 * men[2];
        const T ff = m0 * mas[0] + m1 * mas[1] + m2 * mas[2];
        const T P = s > T(0) ? vmax(bb, T(0)) : vmin(bb, T(0));
        const T Q = s > T(0) ? vmin(ff, T(0)) : vmax(ff, T(0));
        acc += vmax(P * P, Q * Q);
    }
    return vsqrt(acc);
}

// calc_sign_ini (Kang sign) with the frozen band folded in: s = 0 where
// |phi0| < eps and |grad phi0| > 0 (the lambda correction pins d to phi0);
// g is the Godunov norm of phi0 chosen by sign(phi0).
template <typename T>
__device__ __forceinline__ T sign_of(T p, T g, T eps) {
    if (p >= eps) return T(1);
    if (p <= -eps) return T(-1);
    if (p != T(0) && g > T(0)) return T(0);
    return p / eps - T(1.0 / kPi) * vsin(T(kPi) * p / eps);
}

// one reinitialisation pseudo-step at a node: d - dtau s (|grad d|_G - 1)
template <typename T>
__device__ __forceinline__ T reinit_node(const FieldsT<T>& f, const T* __restrict__ din, const Inst& I, long long l,
                                         int i, int j, int k) {
    // every load is issued before the frozen-node test (one memory round trip)
    const T s = __ldg(f.sgn + l);
    const T d = __ldg(din + l);
    const T g = godunov(f, din, I, l, i, j, k, s);
    return s == T(0) ? d : d - ipar<T>(I.dtau, I.dtau64) * s * (g - T(1));
}

template <typename T, int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_reinit(const Inst* __restrict__ inst,
        const Brick* __restrict__ bricks, int nbricks, FieldsT<T> f, const T* __restrict__ din,
        T* __restrict__ dout, unsigned* err) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const Node b = brick_node<TX, TY, TZ>(inst, bricks, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long l = I.off + b.i + (long long)I.ni * (b.j + (long long)I.nj * b.k);
        const T r = reinit_node(f, din, I, l, b.i, b.j, b.k);
        dout[l] = r;
        if (err && !vfinite(r)) atomicOr(err, (unsigned)kErrNonFinite);
    }
}

// calc_sign_ini fused with the first pseudo-step: both use the Godunov norm
// of the advected field phi0 chosen by sign(phi0) (a node whose s is not 0
// has the sign of phi0: p / eps - sin(pi p / eps) / pi has the sign of p),
// so one evaluation and one read of phi0 and the metrics give s and
// d1 = phi0 - dtau s (|grad phi0|_G - 1).
template <typename T, int TX, int TY, int TZ>
__global__ void __launch_bounds__(TX * TY * TZ) k_sign_reinit(const Inst* __restrict__ inst,
        const Brick* __restrict__ bricks, int nbricks, FieldsT<T> f, const T* __restrict__ phi0,
        T* __restrict__ dout, unsigned* err) {
    for (int blk = blockIdx.x; blk < nbricks; blk += gridDim.x) {
        const Node b = brick_node<TX, TY, TZ>(inst, bricks, blk);
        if (!b.valid) continue;
        const Inst& I = inst[b.inst];
        const long long l = I.off + b.i + (long long)I.ni * (b.j + (long long)I.nj * b.k);
        const T p = __ldg(phi0 + l);
        const T g = godunov(f, phi0, I, l, b.i, b.j, b.k, p > T(0) ? T(1) : T(-1));
        const T s = sign_of(p, g, ipar<T>(I.eps, I.eps64));
        f.sgn[l] = s;
        const T r = s == T(0) ? p : p - ipar<T>(I.dtau, I.dtau64) * s * (g - T(1));
        dout[l] = r;
        if (err && !vfinite(r)) atomicOr(err, (unsigned)kErrNonFinite);
    }
}

// Recorded pseudo-steps also write the adjoint's coefficients, so that the
// reverse sweep is a 7-point stencil on lam.  With the Godunov selections
// of the step (branch sign sel: P = sel max(sel bb, 0), Q = sel min(sel ff,
// 0), the larger square taken), G^2 = acc, and w = dtau |s| / G:
//   A'_m = w sum_x M[m][x] (P taken ? sel P : 0),  B'_m = the same with Q,
// moved to B' on a low face and to A' on a high face (their one difference
// serves both sides), and the pseudo-step's adjoint is
//   lam_out(j) = lam(j) - sum_m [lam(j) (A'_m - B'_m)(j)
//                - lam(j+e_m) A'_m(j+e_m) + lam(j-e_m) B'_m(j-e_m)].
// acc is accumulated exactly as in godunov() (bit-identical pseudo-step).
template <typename T>
__device__ __forceinline__ T godunov_sel_v(const T (&mas)[3], const T (&men)[3], const T (&M)[9], T sel, T (&e)[3],
                                           T (&g)[3]) {
    const T sg = sel > T(0) ? T(1) : T(-1);
    T acc = T(0);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        const T bb = sg * (M[x] * men[0] + M[3 + x] * men[1] + M[6 + x] * men[2]);
        const T ff = sg * (M[x] * mas[0] + M[3 + x] * mas[1] + M[6 + x] * mas[2]);
        const T p = vmax(bb, T(0)), q = vmin(ff, T(0));
        const bool takeP = p * p >= q * q;
        acc += takeP ? p * p : q * q;
        e[x] = takeP ? p : T(0);
        g[x] = takeP ? T(0) : q;
    }
    return acc;
}

// One reinitialisation pseudo-step on the tiles of adjoint map 2 (32 x 8
// columns marching 32 planes in k): each node loads d (and s) and its
// metrics once, a plane ahead; the z neighbours of d stay in a register
// window, the x neighbours come by warp shuffles (the tile's edge lanes load
// the one outside) and the y neighbours are loaded (L1/L2).
//   SIGN: the first pseudo-step fused with calc_sign_ini: din is phi0, the
//         Godunov branch is chosen by sign(phi0) (a node whose s is not 0
//         has the sign of phi0), s is computed and stored;
//   REC:  the pseudo-step's adjoint coefficients are stored as well.
// dout2 (nullable) receives a second copy of d'.  d' equals reinit_node's
// arithmetic (one_sided, godunov) bit for bit.
template <typename T, bool SIGN, bool REC>
__global__ void __launch_bounds__(256) k_reinit_z(const Inst* __restrict__ inst, const Brick* __restrict__ bmap,
        int nb, FieldsT<T> f, const T* __restrict__ din, T* __restrict__ dout, T* __restrict__ dout2,
        T* __restrict__ cf, long long ld, unsigned* err) {
    const unsigned FM = 0xffffffffu;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 2, blk);
        const Inst& I = inst[ab.inst];
        const int ni = I.ni, nj = I.nj, nk = I.nk;
        const long long sj = ni, sk = (long long)ni * nj;
        const int i = ab.i0 + tx, j = ab.j0 + ty;
        const int k0 = ab.k0, k1 = min(k0 + adj_shape(2).oz, nk);
        const bool col = i < ni && j < nj;
        const long long cb = I.off + i + sj * j;
        const bool xm = i > 0, xp = i < ni - 1, ym = j > 0, yp = j < nj - 1;
        const bool ex = col && ((tx == 0 && xm) || (tx == 31 && xp));
        const int eo = tx == 0 ? -1 : 1;
        const T dtau = ipar<T>(I.dtau, I.dtau64), eps = ipar<T>(I.eps, I.eps64);
        struct Plane {
            T s, M[9], dxe, dym, dyp;
        };
        auto ld_plane = [&](int k, Plane& p) {
            p.s = p.dxe = p.dym = p.dyp = T(0);
#pragma unroll
            for (int c = 0; c < 9; ++c) p.M[c] = T(0);
            if (!col || k < 0 || k >= nk) return;
            const long long l = cb + sk * k;
            if (!SIGN) p.s = __ldg(f.sgn + l);
#pragma unroll
            for (int c = 0; c < 9; ++c) p.M[c] = __ldg(f.m[c] + l);
            if (ex) p.dxe = __ldg(din + l + eo);
            if (ym) p.dym = __ldg(din + l - sj);
            if (yp) p.dyp = __ldg(din + l + sj);
        };
        auto ldd = [&](int k) { return col && k >= 0 && k < nk ? __ldg(din + cb + sk * k) : T(0); };
        T dm = ldd(k0 - 1), dc = ldd(k0), dp = ldd(k0 + 1);
        Plane pc, pn;
        ld_plane(k0, pc);
        for (int k = k0; k < k1; ++k) {
            const T dn = ldd(k + 2);
            if (k + 1 < k1) ld_plane(k + 1, pn);
            const T xl = __shfl_up_sync(FM, dc, 1), xr = __shfl_down_sync(FM, dc, 1);
            if (col) {
                // one-sided differences (calc_RH_RN.F90:36-170), as one_sided()
                const T dxm = tx == 0 ? pc.dxe : xl, dxp = tx == 31 ? pc.dxe : xr;
                const T nbm[3] = {dxm, pc.dym, dm}, nbp[3] = {dxp, pc.dyp, dp};
                const bool lo[3] = {!xm, !ym, k == 0}, hi[3] = {!xp, !yp, k == nk - 1};
                T mas[3], men[3];
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    const T a = hi[m] ? T(0) : nbp[m] - dc;
                    const T b = lo[m] ? T(0) : dc - nbm[m];
                    mas[m] = hi[m] ? b : a;
                    men[m] = lo[m] ? a : b;
                }
                T e[3], g[3];
                const long long l = cb + sk * k;
                const T acc = godunov_sel_v(mas, men, pc.M, SIGN ? (dc > T(0) ? T(1) : T(-1)) : pc.s, e, g);
                T s = pc.s;
                if (SIGN) {
                    s = sign_of(dc, vsqrt(acc), eps);
                    f.sgn[l] = s;
                }
                const T r = s == T(0) ? dc : dc - dtau * s * (vsqrt(acc) - T(1));
                dout[l] = r;
                if (dout2) dout2[l] = r;
                if (REC) {
                    const T w = s != T(0) && acc > T(0) ? dtau * fabs(s) * vrsqrt(acc) : T(0);
#pragma unroll
                    for (int m = 0; m < 3; ++m) {
                        const T gmen = pc.M[3 * m] * e[0] + pc.M[3 * m + 1] * e[1] + pc.M[3 * m + 2] * e[2];
                        const T gmas = pc.M[3 * m] * g[0] + pc.M[3 * m + 1] * g[1] + pc.M[3 * m + 2] * g[2];
                        cf[m * ld + l] = lo[m] ? T(0) : w * (hi[m] ? gmen + gmas : gmen);
                        cf[(3 + m) * ld + l] = hi[m] ? T(0) : w * (lo[m] ? gmen + gmas : gmas);
                    }
                }
                if (err && !vfinite(r)) atomicOr(err, (unsigned)kErrNonFinite);
            }
            dm = dc;
            dc = dp;
            dp = dn;
            pc = pn;
        }
    }
}

// Reverse of one recorded pseudo-step from its stored coefficients (cf:
// A'_0..2, B'_0..2, ld apart), on the tiles of adjoint map 2 (32 x 8
// columns marching 32 planes in k).  Each node loads its own lam and six
// coefficients once (one plane ahead); the z neighbours (lam, A'_2 above,
// B'_2 below) stay in registers, the x neighbours come by warp shuffles
// (the tile's edge lanes load the one outside), the y neighbours are
// loaded (L1/L2).
template <typename T>
__global__ void __launch_bounds__(256) k_adj_reinit_c(const Inst* __restrict__ inst, const Brick* __restrict__ bmap,
        int nb, const T* __restrict__ cf, long long ld, const T* __restrict__ lam, T* __restrict__ lam_out) {
    const unsigned FM = 0xffffffffu;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 2, blk);
        const Inst& I = inst[ab.inst];
        const int ni = I.ni, nj = I.nj, nk = I.nk;
        const long long sj = ni, sk = (long long)ni * nj;
        const int i = ab.i0 + tx, j = ab.j0 + ty;
        const int k0 = ab.k0, k1 = min(k0 + adj_shape(2).oz, nk);
        const bool col = i < ni && j < nj;
        const long long cb = I.off + i + sj * j;
        const bool xm = i > 0, xp = i < ni - 1, ym = j > 0, yp = j < nj - 1;
        const bool exm = col && xm && tx == 0, exp_ = col && xp && tx == 31;
        // own values of a plane: lam, A'_0..2, B'_0..2; the x-edge lanes' outside
        // neighbour (lam, and A'_0 above / B'_0 below); the y neighbours
        struct Plane {
            T L, A[3], B[3], Le, Ce, Lym, Bym, Lyp, Ayp;
        };
        auto ld_plane = [&](int k, Plane& p) {
            p.L = p.Le = p.Ce = p.Lym = p.Bym = p.Lyp = p.Ayp = T(0);
#pragma unroll
            for (int m = 0; m < 3; ++m) p.A[m] = p.B[m] = T(0);
            if (!col || k < 0 || k >= nk) return;
            const long long l = cb + sk * k;
            p.L = __ldg(lam + l);
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                p.A[m] = __ldg(cf + m * ld + l);
                p.B[m] = __ldg(cf + (3 + m) * ld + l);
            }
            if (exm) {
                p.Le = __ldg(lam + l - 1);
                p.Ce = __ldg(cf + 3 * ld + l - 1);
            }
            if (exp_) {
                p.Le = __ldg(lam + l + 1);
                p.Ce = __ldg(cf + l + 1);
            }
            if (ym) {
                p.Lym = __ldg(lam + l - sj);
                p.Bym = __ldg(cf + 4 * ld + l - sj);
            }
            if (yp) {
                p.Lyp = __ldg(lam + l + sj);
                p.Ayp = __ldg(cf + ld + l + sj);
            }
        };
        Plane pm, pc, pn;          // planes k-1, k, k+1
        ld_plane(k0 - 1, pm);
        ld_plane(k0, pc);
        for (int k = k0; k < k1; ++k) {
            ld_plane(k + 1, pn);
            // x neighbours: lam and A'_0 of i+1, lam and B'_0 of i-1
            const T Lxp = __shfl_down_sync(FM, pc.L, 1), Axp = __shfl_down_sync(FM, pc.A[0], 1);
            const T Lxm = __shfl_up_sync(FM, pc.L, 1), Bxm = __shfl_up_sync(FM, pc.B[0], 1);
            if (col) {
                const T L = pc.L;
                const T lxp = xp ? (tx == 31 ? pc.Le : Lxp) : T(0), axp = xp ? (tx == 31 ? pc.Ce : Axp) : T(0);
                const T lxm = xm ? (tx == 0 ? pc.Le : Lxm) : T(0), bxm = xm ? (tx == 0 ? pc.Ce : Bxm) : T(0);
                const bool zm = k > 0, zp = k < nk - 1;
                const T t0 = L * pc.A[0] - L * pc.B[0] - lxp * axp + lxm * bxm;
                const T t1 = L * pc.A[1] - L * pc.B[1] - pc.Lyp * pc.Ayp + pc.Lym * pc.Bym;
                const T t2 = L * pc.A[2] - L * pc.B[2] - (zp ? pn.L * pn.A[2] : T(0)) + (zm ? pm.L * pm.B[2] : T(0));
                lam_out[cb + sk * k] = L - t0 - t1 - t2;
            }
            pm = pc;
            pc = pn;
        }
    }
}

// P0 after the last pseudo-step: interior from its output, boundary nodes
// recomputed from its input (their output slots are being overwritten).
template <typename T>
struct P0Reinit {
    FieldsT<T> f;
    const T *din, *dout;
    const Inst* I;
    __device__ T operator()(int i, int j, int k) const {
        const long long l = I->off + i + (long long)I->ni * (j + (long long)I->nj * k);
        const bool bnd = i == 0 || i == I->ni - 1 || j == 0 || j == I->nj - 1 || k == 0 || k == I->nk - 1;
        return bnd ? reinit_node(f, din, *I, l, i, j, k) : dout[l];
    }
};

template <typename T>
__global__ void k_bc_reinit(const Inst* __restrict__ inst, int ninst, long long nface, BC bc, FieldsT<T> f,
                            const T* __restrict__ din, T* dout) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= nface) return;
    const Inst& I = inst[face_instance(inst, ninst, t)];
    int i, j, k;
    if (!face_coords(I, t - I.face0, &i, &j, &k)) return;
    P0Reinit<T> p0{f, din, dout, &I};
    dout[I.off + i + (long long)I.ni * (j + (long long)I.nj * k)] = bval_k<T>(bc, p0, I.ni, I.nj, I.nk, i, j, k);
}

// ------------------------------------------------------------ volume
// Water volume of one tetrahedron of an interface cell: the same regions as
// MarchingTetrahedron + GetWaterVolume (src/TetrahedronMethods.F90:26-954),
// each sub-tetrahedron's share of the tetrahedron evaluated in barycentric
// closed form: one determinant per tetrahedron instead of up to four
// (equal in exact arithmetic, rounding differs).  G is the geometry type:
// FP64 for the FP64 stencils, FP32 for the FP32 ones (vertices relative to
// the cell's first vertex, see k_vol_iface).
template <typename G>
__device__ __forceinline__ G tetvol_g(const G (&a)[3], const G (&b)[3], const G (&c)[3], const G (&d)[3]) {
    const G u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
    const G v0 = c[0] - a[0], v1 = c[1] - a[1], v2 = c[2] - a[2];
    const G w0 = d[0] - a[0], w1 = d[1] - a[1], w2 = d[2] - a[2];
    const G t = w0 * (u1 * v2 - u2 * v1) + w1 * (u2 * v0 - u0 * v2) + w2 * (u0 * v1 - u1 * v0);
    return fabs(t) * G(1.0 / 6.0);
}

// 4-way selection without indexing (keeps the tetrahedron in registers)
template <typename X>
__device__ __forceinline__ X sel4(const X (&a)[4], int i) {
    return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

// ------------------------------------------------------------ dual numbers
// Forward-mode derivatives of the tetrahedron water volume with respect to
// its vertex values (the mass correction and its adjoint): a value and K
// partials; S is a scalar or itself a Dual (second derivatives).
template <typename S, int K>
struct Dual {
    S v;
    S d[K];
};
template <typename X> struct DualTraits { using Base = X; };
template <typename S, int K> struct DualTraits<Dual<S, K>> { using Base = typename DualTraits<S>::Base; };
template <typename X> __device__ __forceinline__ typename DualTraits<X>::Base dval(const X& x) { return x; }
template <typename S, int K> __device__ __forceinline__ typename DualTraits<S>::Base dval(const Dual<S, K>& x) {
    return dval(x.v);
}
// constant (all partials zero)
template <typename X> struct Lift { __device__ static X of(typename DualTraits<X>::Base c) { return X(c); } };
template <typename S, int K> struct Lift<Dual<S, K>> {
    __device__ static Dual<S, K> of(typename DualTraits<S>::Base c) {
        Dual<S, K> r;
        r.v = Lift<S>::of(c);
#pragma unroll
        for (int k = 0; k < K; ++k) r.d[k] = Lift<S>::of(typename DualTraits<S>::Base(0));
        return r;
    }
};
template <typename S, int K>
__device__ __forceinline__ Dual<S, K> operator+(const Dual<S, K>& a, const Dual<S, K>& b) {
    Dual<S, K> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <typename S, int K>
__device__ __forceinline__ Dual<S, K> operator-(const Dual<S, K>& a, const Dual<S, K>& b) {
    Dual<S, K> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <typename S, int K>
__device__ __forceinline__ Dual<S, K> operator-(const Dual<S, K>& a) {
    Dual<S, K> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <typename S, int K>
__device__ __forceinline__ Dual<S, K> operator*(const Dual<S, K>& a, const Dual<S, K>& b) {
    Dual<S, K> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <typename S, int K>
__device__ __forceinline__ Dual<S, K> operator/(const Dual<S, K>& a, const Dual<S, K>& b) {
    Dual<S, K> r;
    r.v = a.v / b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
    return r;
}
// scalar (geometry) factor times a dual
template <typename S, int K>
__device__ __forceinline__ Dual<S, K> operator*(typename DualTraits<S>::Base c, const Dual<S, K>& a) {
    Dual<S, K> r;
    r.v = c * a.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = c * a.d[k];
    return r;
}
template <typename S, int K>
__device__ __forceinline__ Dual<S, K> operator-(typename DualTraits<S>::Base c, const Dual<S, K>& a) {
    return Lift<Dual<S, K>>::of(c) - a;
}

// Water (phi > 0) volume of one tetrahedron with vertices V and vertex
// values ph (the reference's MarchingTetrahedron + GetWaterVolume cases,
// src/TetrahedronMethods.F90:586-954, in closed form).  X is the vertex
// value type: the geometry type G, or a Dual of it for the derivatives with
// respect to the vertex values (the case chosen by the values themselves).
template <typename G, typename X>
__device__ __forceinline__ X tet_water_x(const G (&V)[4][3], const X (&ph)[4]) {
    const G TV = tetvol_g(V[0], V[1], V[2], V[3]);
    const G tiny = G(sizeof(G) == 8 ? kTinyD : 0.0);   // tiny(1d0); in FP32 every nonzero value exceeds it
    const X zero = Lift<X>::of(G(0)), one = Lift<X>::of(G(1)), full = Lift<X>::of(TV);
    int s[4], nz = 0, fi = 0;
    bool allp = true, alln = true, allge = true, allle = true;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const G pv = dval(ph[v]);
        s[v] = pv > tiny ? 1 : (pv < -tiny ? -1 : 0);
        allp &= s[v] == 1; alln &= s[v] == -1; nz += s[v] == 0;
        allge &= s[v] >= 0; allle &= s[v] <= 0;
        if (s[v] == -1) fi |= 1 << v;
    }
    if (allp) return full;
    if (alln) return zero;
    if (nz > 0 && (allge || allle)) {
        // the reference's zero-vertex cases: full or empty tetrahedron
        int water = -1;
        if (nz == 1) {
            if (s[0] == 0) water = s[1] == 1; else if (s[1] == 0) water = s[0] == 1;
            else if (s[2] == 0) water = s[0] == 1; else water = s[0] == 1;
        } else if (nz == 2) {
            if (s[0] == 0 && s[1] == 0) water = s[2] == 1;
            else if (s[1] == 0 && s[2] == 0) water = s[0] == 1;
            else if (s[2] == 0 && s[0] == 0) water = s[1] == 1;
            else if (s[0] == 0 && s[3] == 0) water = s[1] == 1;
            else if (s[1] == 0 && s[3] == 0) water = s[0] == 1;
            else water = s[0] == 1;
        } else if (nz == 3) {
#pragma unroll
            for (int v = 0; v < 4; ++v)
                if (water < 0 && s[v] != 0) water = s[v] == 1;   // the non-zero vertex
        }
        return water == 0 ? zero : full;   // four zero vertices: full (FlagIndex 0)
    }
    // one vertex isolated from the other three (cases 2/15, 3/14, 5/12, 9/8)
    int iso = -1;
    if (fi == 1 || fi == 14) iso = 0; else if (fi == 2 || fi == 13) iso = 1;
    else if (fi == 4 || fi == 11) iso = 2; else if (fi == 8 || fi == 7) iso = 3;
    if (iso >= 0) {
        // prod_k p_iso / (p_iso - p_k) over one division (the differences
        // all carry the sign of p_iso: no cancellation); the factor of k =
        // iso is an exact 1
        const X pI = sel4(ph, iso);
        X num = one, den = one;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            num = num * (k != iso ? pI : one);
            den = den * (k != iso ? pI - ph[k] : one);
        }
        const X AV = TV * (num / den);
        return (sel4(s, iso) == -1) ? TV - AV : AV;   // isolated vertex negative: the rest is water
    }
    // two against two (cases 4/13, 6/11, 7/10): pair (A, B) as listed by the
    // reference's sub-tetrahedra, C, D the other pair:
    //   fi 3/12: A 0, B 1, C 2;  fi 5/10: A 0, B 2, C 1;  else A 1, B 2, C 0;  D 3
    const int cs = (fi == 3 || fi == 12) ? 0 : ((fi == 5 || fi == 10) ? 1 : 2);
    // with the edge fractions aX = pA / (pA - pX), bX = pB / (pB - pX) the
    // share is aC aD (1 - bD) + aC bD (1 - bC) + bC bD; over the common
    // denominator (pA - pC)(pA - pD)(pB - pC)(pB - pD), using 1 - bX =
    // -pX / (pB - pX), it needs one division, and its three numerator terms
    // share one sign (A, B on one side of the interface, C, D on the other)
    const X pA = cs == 2 ? ph[1] : ph[0];
    const X pB = cs == 0 ? ph[1] : ph[2];
    const X pC = cs == 0 ? ph[2] : (cs == 1 ? ph[1] : ph[0]);
    const X pD = ph[3];
    const X dAC = pA - pC, dAD = pA - pD, dBC = pB - pC, dBD = pB - pD;
    const X num = pB * pB * dAC * dAD - pA * pA * pD * dBC - pA * pB * pC * dAD;
    const X AV = TV * (num / (dAC * dAD * dBC * dBD));
    return ((cs == 2 ? s[1] : s[0]) == -1) ? TV - AV : AV;
}

template <typename G>
__device__ __forceinline__ G tet_water(const G (&V)[4][3], const G (&ph)[4]) {
    return tet_water_x<G, G>(V, ph);
}

// vertex v of tetrahedron t of CellAnalysis's split (the c_tets table
// {0,5,1,6}, {0,1,2,6}, {0,2,3,6}, {0,3,7,6}, {0,7,4,6}, {0,4,5,6}) as a
// constant expression, so that unrolled loops index registers
__host__ __device__ constexpr int cell_tet(int t, int v) {
    return v == 0 ? 0
                  : v == 3 ? 6
                           : v == 1 ? (t == 0 ? 5 : t == 1 ? 1 : t == 2 ? 2 : t == 3 ? 3 : t == 4 ? 7 : 4)
                                    : (t == 0 ? 1 : t == 1 ? 2 : t == 2 ? 3 : t == 3 ? 7 : t == 4 ? 4 : 5);
}

// CellAnalysis's tetrahedron classes: pct (phase change, a K tetrahedron)
// or second (all water); the phi-type compares equal the FP64 ones.
template <typename P>
__device__ __forceinline__ void tet_class(const P (&ph8)[8], int t, bool* pct_out, bool* second_out) {
    const P es = P(kEpsSims);
    bool pct = false, second = true;
    const P pa = ph8[cell_tet(t, 0)];
    if (pa <= es) second = false;
    if (fabs(pa) < es) pct = true;
    const P sg = signbit(pa) ? P(-1) : P(1);
#pragma unroll
    for (int v = 1; v < 4; ++v) {
        const P pb = ph8[cell_tet(t, v)];
        if (sg * pb < P(0) || fabs(pb) < es) {
            if (pb <= es) second = false;
            pct = true;
        }
    }
    *pct_out = pct;
    *second_out = second;
}

// whether CellAnalysis splits the cell (a vertex within eps_sims of zero or
// a sign change)
template <typename P>
__device__ __forceinline__ bool cell_is_interface(const P (&ph8)[8]) {
    const P es = P(kEpsSims);
    bool pcc = false;
#pragma unroll
    for (int v = 0; v < 8; ++v) pcc |= fabs(ph8[v]) < es;
    if (!pcc) {
        const P sg = signbit(ph8[0]) ? P(-1) : P(1);   // copysign(1, phi)
#pragma unroll
        for (int v = 1; v < 8; ++v) pcc |= sg * ph8[v] < P(0);
    }
    return pcc;
}

// CellAnalysis's split of an interface cell (src/TetrahedronMethods.F90:
// 1823-2121): phase-change tetrahedra -> K, all-water tetrahedra -> S.
// The classification runs in the phi type P (eps_sims = 2^-52 and +-1 are
// exact in FP32, so its compares equal the FP64 ones on the same values),
// the geometry in P as well, on vertex coordinates relative to the cell's
// first vertex (C, formed in FP64 by the caller).  Fully unrolled: every
// array index is a constant (no local memory).  With SLOPE, *A also gets
// dK/dC, the derivative of the K volume under a uniform shift phi + C
// (forward-mode dual numbers through the same case formulas).
template <typename P, bool SLOPE = false>
__device__ void cell_water_fast(const P (&ph8)[8], const P (&C)[8][3], double* K, double* S, double* A = nullptr) {
    P k = P(0), s2 = P(0), a = P(0);
    if (cell_is_interface(ph8)) {
#pragma unroll
        for (int t = 0; t < 6; ++t) {
            bool pct, second;
            tet_class(ph8, t, &pct, &second);
            if (pct || second) {
                P V[4][3], ph[4];
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    V[v][0] = C[cell_tet(t, v)][0];
                    V[v][1] = C[cell_tet(t, v)][1];
                    V[v][2] = C[cell_tet(t, v)][2];
                    ph[v] = ph8[cell_tet(t, v)];
                }
                if (pct) {
                    if constexpr (SLOPE) {
                        Dual<P, 1> pd[4];
#pragma unroll
                        for (int v = 0; v < 4; ++v) {
                            pd[v].v = ph[v];
                            pd[v].d[0] = P(1);
                        }
                        const Dual<P, 1> w = tet_water_x<P, Dual<P, 1>>(V, pd);
                        k += w.v;
                        a += w.d[0];
                    } else {
                        k += tet_water(V, ph);
                    }
                } else {
                    s2 += tetvol_g(V[0], V[1], V[2], V[3]);
                }
            }
        }
    }
    *K = (double)k; *S = (double)s2;
    if (A) *A = (double)a;
}

// Mass-correction adjoint weights of one interface cell: for each vertex v
// the derivative of the cell's K volume g_v = dK/dphi_v plus Cs h_v with
// h_v = d(dK/dC)/dphi_v (second-order dual numbers), so that the shift
// C = (target - V) / A has dC/dphi_v = -(g_v + C h_v) / A summed over the
// cells around the node.
template <typename P>
__device__ void cell_mass_weights(const P (&ph8)[8], const P (&C)[8][3], P Cs, P (&w8)[8]) {
#pragma unroll
    for (int v = 0; v < 8; ++v) w8[v] = P(0);
    if (!cell_is_interface(ph8)) return;
    using D1 = Dual<P, 1>;
    using D2 = Dual<D1, 4>;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
        bool pct, second;
        tet_class(ph8, t, &pct, &second);
        if (!pct) continue;
        P V[4][3];
        D2 pd[4];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            V[v][0] = C[cell_tet(t, v)][0];
            V[v][1] = C[cell_tet(t, v)][1];
            V[v][2] = C[cell_tet(t, v)][2];
            pd[v].v.v = ph8[cell_tet(t, v)];
            pd[v].v.d[0] = P(1);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                pd[v].d[u].v = u == v ? P(1) : P(0);
                pd[v].d[u].d[0] = P(0);
            }
        }
        const D2 r = tet_water_x<P, D2>(V, pd);
#pragma unroll
        for (int u = 0; u < 4; ++u) w8[cell_tet(t, u)] += r.d[u].v + Cs * r.d[u].d[0];
    }
}

// The volume pass runs in two kernels.  k_vol_scan_z streams every cell of
// every instance (a k march over the tiles of adjoint map 2): cells whose
// eight vertices are water (phi > eps_sims, in the phi type) add their
// precomputed FP64 hexahedron volume in 64-bit fixed point; interface cells
// (any other mix) are appended to a list, each warp reserving its slots with
// one atomic (list order is not fixed; every sum below is an integer sum, so
// the result does not depend on it).  k_vol_iface then runs the reference's
// six-tetrahedra split on the listed cells with every lane busy, in the
// stencil precision on coordinates relative to each cell's first vertex
// (differences formed in FP64; an FP32 batch keeps them per cell, formed
// once per geometry), optionally with the mass correction's slope
// dK/dC.  Each cell's shares are rounded to multiples of 2^-48 and added to
// the instance's accumulators with integer atomics after a warp sum: exact
// and order-independent.
// exact warp sum of 64-bit integers (two's complement, modulo 2^64): three
// limbs of 22, 22 and 20 bits, each summed by the warp's integer reduction
// (32 x 2^22 < 2^32), recombined; every lane gets the sum
__device__ __forceinline__ long long warp_sum_nn(long long v) {
    const unsigned long long u = (unsigned long long)v;
    const unsigned m = (1u << 22) - 1u;
    const unsigned long long s0 = __reduce_add_sync(0xffffffffu, (unsigned)(u & m));
    const unsigned long long s1 = __reduce_add_sync(0xffffffffu, (unsigned)((u >> 22) & m));
    const unsigned long long s2 = __reduce_add_sync(0xffffffffu, (unsigned)(u >> 44));
    return (long long)(s0 + (s1 << 22) + (s2 << 44));
}

// Bulk water volumes of the cells and the interface-cell list (SUMS: also
// add the bulk cells' fixed-point volumes to acc[4 inst + 2]), on the tiles
// of adjoint map 2: thread (lane, row) owns the cell column (i0 + lane, j0 +
// row) and marches the tile's planes in k.  A cell's eight vertices are the
// 2 x 2 quads of planes k and k + 1; a quad is the thread's own node and
// the one at j + 1 (loaded), with the i + 1 pair from the next lane by a
// shuffle (the tile's last lane loads it).  Each plane is loaded once, a
// plane ahead of its use; a quad is reduced to two flags (all water, all
// air) and a cell is water / air when both of its quads are.
template <typename T, bool SUMS>
__global__ void __launch_bounds__(256) k_vol_scan_z(const Inst* __restrict__ inst, const Brick* __restrict__ bmap,
        int nb, FieldsT<T> f, const T* __restrict__ phi, unsigned long long* __restrict__ acc,
        unsigned* __restrict__ list, unsigned* __restrict__ count) {
    const T eps = T(kEpsSims);
    const unsigned FM = 0xffffffffu;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    long long Bq = 0;
    int cur = -1;
    auto flush = [&]() {
        const long long v = warp_sum_nn(Bq);
        if (tx == 0 && v != 0) atomicAdd(acc + 4 * (long long)cur + 2, (unsigned long long)v);
        Bq = 0;
    };
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 2, blk);
        if (SUMS && ab.inst != cur) {
            if (cur >= 0) flush();
            cur = ab.inst;
        }
        const Inst& I = inst[ab.inst];
        const int ni = I.ni, nj = I.nj, nk = I.nk;
        const long long sj = ni, sk = (long long)ni * nj;
        const int i = ab.i0 + tx, j = ab.j0 + ty;
        // cells k0 .. kc1 - 1 (a cell's top plane k + 1 stays inside the grid)
        const int k0 = ab.k0, kc1 = min(k0 + adj_shape(2).oz, nk - 1);
        const bool cell = i < ni - 1 && j < nj - 1;
        const bool own = i < ni && j < nj - 1, edge = tx == 31 && i + 1 < ni && j < nj - 1;
        const long long cb = I.off + i + sj * j;
        struct Quad {
            T a, c, ae, ce;   // (i, j), (i, j + 1); the last lane's (i + 1, j), (i + 1, j + 1)
        };
        auto ld = [&](int k, Quad& q) {
            q.a = q.c = q.ae = q.ce = T(0);
            const long long l = cb + sk * k;
            if (own) {
                q.a = __ldg(phi + l);
                q.c = __ldg(phi + l + sj);
            }
            if (edge) {
                q.ae = __ldg(phi + l + 1);
                q.ce = __ldg(phi + l + 1 + sj);
            }
        };
        auto flags = [&](const Quad& q, bool& qw, bool& qa) {
            const T b = __shfl_down_sync(FM, q.a, 1), d = __shfl_down_sync(FM, q.c, 1);
            const T bb = tx == 31 ? q.ae : b, dd = tx == 31 ? q.ce : d;
            qw = q.a > eps && bb > eps && q.c > eps && dd > eps;
            qa = q.a < -eps && bb < -eps && q.c < -eps && dd < -eps;
        };
        bool qw0 = false, qa0 = false;
        Quad qn;
        long long cv = 0;
        if (k0 < kc1) {
            Quad q0;
            ld(k0, q0);
            ld(k0 + 1, qn);
            if (SUMS && cell) cv = __ldg(f.cellfix + cb + sk * k0);
            flags(q0, qw0, qa0);
        }
        for (int k = k0; k < kc1; ++k) {
            Quad qq;
            long long cvn = 0;
            if (k + 1 < kc1) {
                ld(k + 2, qq);
                if (SUMS && cell) cvn = __ldg(f.cellfix + cb + sk * (k + 1));
            }
            bool qw1, qa1;
            flags(qn, qw1, qa1);
            const bool allw = qw0 && qw1, alla = qa0 && qa1;
            if (SUMS && cell && allw) Bq += cv;
            const bool mix = cell && !allw && !alla;
            const unsigned m = __ballot_sync(FM, mix);
            if (m) {
                unsigned base = 0;
                if (tx == 0) base = atomicAdd(count, (unsigned)__popc(m));
                base = __shfl_sync(FM, base, 0);
                if (mix) list[base + __popc(m & ((1u << tx) - 1u))] = (unsigned)(cb + sk * k);
            }
            qw0 = qw1;
            qa0 = qa1;
            qn = qq;
            cv = cvn;
        }
    }
    if (SUMS && cur >= 0) flush();
}

// the eight vertex values and the coordinates relative to vertex 0 of the
// listed cell whose first node is l (instance I)
template <typename T>
__device__ __forceinline__ void cell_gather(const Inst& I, const FieldsT<T>& f, const T* __restrict__ phi,
                                            long long l, long long (&o)[8], T (&P8)[8], T (&C)[8][3]) {
    const long long sj = I.ni, sk = (long long)I.ni * I.nj;
    o[0] = l; o[1] = l + 1; o[2] = l + 1 + sj; o[3] = l + sj;
    o[4] = l + sk; o[5] = l + 1 + sk; o[6] = l + 1 + sj + sk; o[7] = l + sj + sk;
#pragma unroll
    for (int v = 0; v < 8; ++v) P8[v] = __ldg(phi + o[v]);
    if constexpr (sizeof(T) == 4) {
        if (f.cellrel) {
            // the same values, formed once per geometry (k_cell_rel)
            const float4* r = reinterpret_cast<const float4*>(f.cellrel + 24 * l);
            float q[24];
#pragma unroll
            for (int u = 0; u < 6; ++u) {
                const float4 w = __ldg(r + u);
                q[4 * u] = w.x; q[4 * u + 1] = w.y; q[4 * u + 2] = w.z; q[4 * u + 3] = w.w;
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) C[0][a] = T(0);
#pragma unroll
            for (int v = 1; v < 8; ++v)
#pragma unroll
                for (int a = 0; a < 3; ++a) C[v][a] = q[3 * (v - 1) + a];
            return;
        }
    }
    double X0[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) X0[a] = __ldg(f.xyz[a] + l);
#pragma unroll
    for (int v = 0; v < 8; ++v)
#pragma unroll
        for (int a = 0; a < 3; ++a) C[v][a] = (T)(__ldg(f.xyz[a] + o[v]) - X0[a]);
}

// instance of packed node t (binary search over the node offsets)
__device__ __forceinline__ int node_instance(const Flat& fl, long long t) {
    int lo = 0, hi = fl.ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (fl.offs[mid] <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// K and S volumes (and with SLOPE dK/dC) of the listed interface cells into
// acc[4 inst + 0, 1, 3]: lanes of a warp that all hold one instance add a
// warp sum, otherwise each lane adds its own
template <typename T, bool SLOPE>
__global__ void __launch_bounds__(128) k_vol_iface(Flat fl, FieldsT<T> f, const T* __restrict__ phi,
                                                   const unsigned* __restrict__ list, const unsigned* __restrict__ count,
                                                   unsigned long long* __restrict__ acc) {
    const unsigned FM = 0xffffffffu;
    const unsigned n = *count;
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); e0 < n; e0 += stride) {
        const long long e = e0 + lane;
        const bool valid = e < n;
        long long Kq = 0, Sq = 0, Aq = 0;
        int q = -1;
        if (valid) {
            const long long l = list[e];
            q = node_instance(fl, l);
            long long o[8];
            T P8[8], C[8][3];
            cell_gather(fl.inst[q], f, phi, l, o, P8, C);
            double K = 0.0, S = 0.0, A = 0.0;
            cell_water_fast<T, SLOPE>(P8, C, &K, &S, &A);
            Kq = __double2ll_rn(K * kVolScale);
            Sq = __double2ll_rn(S * kVolScale);
            if (SLOPE) Aq = __double2ll_rn(A * kVolScale);
        }
        const int q0 = __shfl_sync(FM, q, 0);
        if (__all_sync(FM, q == q0)) {
            const long long v[3] = {warp_sum_nn(Kq), warp_sum_nn(Sq), SLOPE ? warp_sum_nn(Aq) : 0};
            if (lane == 0 && q0 >= 0) {
                if (v[0]) atomicAdd(acc + 4 * (long long)q0, (unsigned long long)v[0]);
                if (v[1]) atomicAdd(acc + 4 * (long long)q0 + 1, (unsigned long long)v[1]);
                if (v[2]) atomicAdd(acc + 4 * (long long)q0 + 3, (unsigned long long)v[2]);
            }
        } else if (valid) {
            if (Kq) atomicAdd(acc + 4 * (long long)q, (unsigned long long)Kq);
            if (Sq) atomicAdd(acc + 4 * (long long)q + 1, (unsigned long long)Sq);
            if (SLOPE && Aq) atomicAdd(acc + 4 * (long long)q + 3, (unsigned long long)Aq);
        }
    }
}

// converts each instance's accumulators (K, S, bulk, slope) to volumes and
// clears them for the next volume pass; with `mass` it also forms the
// mass correction C = (target - V) / A of the total V (C = 0 without a
// finite target or without interface), into mass[q] and, when recording,
// mrec[q]
__global__ void k_volume_final(int ninst, unsigned long long* __restrict__ acc, double* __restrict__ vols,
                               const double* __restrict__ target, Mass* __restrict__ mass, Mass* __restrict__ mrec) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ninst) return;
    long long v[4];
    for (int c = 0; c < 4; ++c) {
        v[c] = (long long)acc[4 * q + c];
        acc[4 * q + c] = 0ull;
    }
    const double tot = (double)(v[0] + v[1] + v[2]) * kVolUnit;
    vols[4 * q] = (double)v[0] * kVolUnit;
    vols[4 * q + 1] = (double)v[1] * kVolUnit;
    vols[4 * q + 2] = (double)v[2] * kVolUnit;
    vols[4 * q + 3] = tot;
    if (mass) {
        Mass m;
        m.V = tot;
        m.A = (double)v[3] * kVolUnit;
        m.target = target[q];
        const double c = (target[q] - tot) / m.A;
        m.C = mass_on(m) ? c : 0.0;
        mass[q] = m;
        if (mrec) mrec[q] = m;
    }
}

// dst = src + C of the node's instance (the mass correction's uniform shift)
template <typename T>
__global__ void k_mass_shift(Flat fl, const Mass* __restrict__ mass, const T* __restrict__ src, T* __restrict__ dst) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < fl.n;
         t += (long long)gridDim.x * blockDim.x) {
        Node nd;
        flat_node(fl, t, &nd);
        dst[t] = src[t] + (T)mass[nd.inst].C;
    }
}

// Adjoint of the shift, part 1: every listed interface cell of the step's
// pre-correction field adds its vertices' weights g_v + C h_v
// (cell_mass_weights) to wfix in fixed point (integer atomics: exact and
// order-independent).
template <typename T>
__global__ void __launch_bounds__(128) k_mass_weights(Flat fl, FieldsT<T> f, const T* __restrict__ phi,
                                                      const unsigned* __restrict__ list,
                                                      const unsigned* __restrict__ count, const Mass* __restrict__ mass,
                                                      unsigned long long* __restrict__ wfix) {
    const unsigned n = *count;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const long long l = list[e];
        const int q = node_instance(fl, l);
        const Mass M = mass[q];
        if (!mass_on(M)) continue;
        long long o[8];
        T P8[8], C[8][3], W8[8];
        cell_gather(fl.inst[q], f, phi, l, o, P8, C);
        cell_mass_weights<T>(P8, C, (T)M.C, W8);
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const long long w = __double2ll_rn((double)W8[v] * kVolScale);
            if (w != 0) atomicAdd(wfix + o[v], (unsigned long long)w);
        }
    }
}

// Adjoint of the shift, part 2: per tile of adjoint map 2 (32 x 8 columns
// x 32 planes, inside one instance) the sum of lam over the tile, in a
// fixed order (each thread its column, then a fixed tree), accumulated in
// FP64.  FP32 lam is first summed in FP32 over runs of 8 planes (the FP64
// pipe would otherwise take a conversion and an add per node).
template <typename T>
__global__ void __launch_bounds__(256) k_tile_sum(const Inst* __restrict__ inst, const Brick* __restrict__ bmap,
                                                   int nb, const T* __restrict__ lam, double* __restrict__ part) {
    __shared__ double red[8];
    const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 2, blk);
        const Inst& I = inst[ab.inst];
        const int i = ab.i0 + tx, j = ab.j0 + ty, k1 = min(ab.k0 + adj_shape(2).oz, I.nk);
        double sacc = 0.0;
        if (i < I.ni && j < I.nj) {
            const long long sk = (long long)I.ni * I.nj;
            const T* p = lam + I.off + i + (long long)I.ni * j;
            if constexpr (sizeof(T) == 4) {
                for (int k = ab.k0; k < k1; k += 8) {
                    float r = 0.f;
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        if (k + u < k1) r += __ldg(p + sk * (k + u));
                    sacc += (double)r;
                }
            } else {
                for (int k = ab.k0; k < k1; ++k) sacc += (double)__ldg(p + sk * k);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
        if (tx == 0) red[ty] = sacc;
        __syncthreads();
        if (t == 0) {
            double r = 0.0;
            for (int u = 0; u < 8; ++u) r += red[u];
            part[blk] = r;
        }
        __syncthreads();
    }
}

// part 3: one block per instance sums its tiles' partials in a fixed order
__global__ void __launch_bounds__(256) k_inst_sum(const Inst* __restrict__ inst, const double* __restrict__ part,
                                                  double* __restrict__ out) {
    __shared__ double red[8];
    const Inst& I = inst[blockIdx.x];
    const int t0 = I.am[2][0];
    const int nt = I.am[2][1] * I.am[2][2] * ((I.nk + adj_shape(2).oz - 1) / adj_shape(2).oz);
    double s = 0.0;
    for (int u = threadIdx.x; u < nt; u += blockDim.x) s += part[t0 + u];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int u = 0; u < 8; ++u) r += red[u];
        out[blockIdx.x] = r;
    }
}

// part 4: lam_pre = lam - (S / A) w with S = sum(lam) of the instance and
// w = wfix in fixed point, on the vertices of the listed interface cells
// (the only nodes with a weight).  Each vertex's weight is taken and cleared
// for the next step by one atomic exchange, so exactly one thread applies
// it, whatever the list order.
template <typename T>
__global__ void __launch_bounds__(128) k_mass_apply(Flat fl, const Mass* __restrict__ mass,
                                                    const double* __restrict__ ssum, const unsigned* __restrict__ list,
                                                    const unsigned* __restrict__ count, T* __restrict__ lam,
                                                    unsigned long long* __restrict__ wfix) {
    const unsigned n = *count;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const long long l = list[e];
        const int q = node_instance(fl, l);
        const Mass M = mass[q];
        if (!mass_on(M)) continue;
        const Inst& I = fl.inst[q];
        const long long sj = I.ni, sk = (long long)I.ni * I.nj;
        const long long o[8] = {l, l + 1, l + 1 + sj, l + sj, l + sk, l + 1 + sk, l + 1 + sj + sk, l + sj + sk};
        const double r = ssum[q] / M.A;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const long long w = (long long)atomicExch(wfix + o[v], 0ull);
            if (w != 0) lam[o[v]] = (T)((double)lam[o[v]] - r * ((double)w * kVolUnit));
        }
    }
}

// fixed-point Davies-Salmond volume of every cell of one instance
__global__ void k_cell_hex(long long off, int ni, int nj, int nk, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z, long long* __restrict__ cellfix) {
    const long long ncell = (long long)(ni - 1) * (nj - 1) * (nk - 1);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % (ni - 1)), j = (int)((c / (ni - 1)) % (nj - 1));
        const int k = (int)(c / ((long long)(ni - 1) * (nj - 1)));
        const long long sj = ni, sk = (long long)ni * nj;
        const long long l = off + i + sj * j + sk * k;
        const long long o[8] = {l, l + 1, l + 1 + sj, l + sj, l + sk, l + 1 + sk, l + 1 + sj + sk, l + sj + sk};
        double C[8][3];
#pragma unroll
        for (int v = 0; v < 8; ++v) { C[v][0] = x[o[v]]; C[v][1] = y[o[v]]; C[v][2] = z[o[v]]; }
        cellfix[l] = __double2ll_rn(hex_volume(C) * kVolScale);
    }
}

// FP32 coordinates of the vertices 1..7 of every cell relative to its vertex
// 0, the differences formed in FP64 (cell_gather's values), 24 floats per
// cell by base node
__global__ void k_cell_rel(long long off, int ni, int nj, int nk, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z, float* __restrict__ rel) {
    const long long ncell = (long long)(ni - 1) * (nj - 1) * (nk - 1);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % (ni - 1)), j = (int)((c / (ni - 1)) % (nj - 1));
        const int k = (int)(c / ((long long)(ni - 1) * (nj - 1)));
        const long long sj = ni, sk = (long long)ni * nj;
        const long long l = off + i + sj * j + sk * k;
        const long long o[8] = {l, l + 1, l + 1 + sj, l + sj, l + sk, l + 1 + sk, l + 1 + sj + sk, l + sj + sk};
        const double X0[3] = {x[l], y[l], z[l]};
        float q[24];
#pragma unroll
        for (int v = 1; v < 8; ++v) {
            q[3 * (v - 1)] = (float)(x[o[v]] - X0[0]);
            q[3 * (v - 1) + 1] = (float)(y[o[v]] - X0[1]);
            q[3 * (v - 1) + 2] = (float)(z[o[v]] - X0[2]);
        }
        q[21] = q[22] = q[23] = 0.f;
        float4* r = reinterpret_cast<float4*>(rel + 24 * l);
#pragma unroll
        for (int u = 0; u < 6; ++u) r[u] = make_float4(q[4 * u], q[4 * u + 1], q[4 * u + 2], q[4 * u + 3]);
    }
}

// ================================================================ adjoint
// Reverse of face `face` of bcond_lsm: for every node b of that face plane,
// lam(n1) += a lam(b), lam(n2) += c lam(b), lam(b) = 0, with (a, c) the
// face rule's weights (the BigPhi switch evaluated on the forward value of
// n2 at that point of the face sequence).  Distinct nodes of one plane have
// distinct targets, so the kernel needs no atomics.
template <typename T, class P0>
__device__ __forceinline__ T prev_value(const BC& bc, const P0& p0, int face, int ni, int nj, int i, int j, int k) {
    if (face < 2) return p0(i, j, k);
    if (face < 4) return bval_i<T>(bc, p0, ni, i, j, k);
    return bval_j<T>(bc, p0, ni, nj, i, j, k);
}

template <typename T>
__global__ void k_adj_face(Flat fl, int face0, long long nplane, int nface, BC bc, int kind,
                           const T* __restrict__ phin, const T* __restrict__ in, const T* __restrict__ out, T c1, T c2,
                           T* lam) {
    // nface 2: face0 (odd) and the opposite face face0 - 1 of the same axis in
    // one launch (no shared nodes, no shared targets when the axis has at
    // least 6 nodes in every instance)
    const long long tt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tt >= nplane * nface) return;
    const bool second = tt >= nplane;
    const int face = second ? face0 - 1 : face0;
    const long long t = second ? tt - nplane : tt;
    if (!face_on(bc, face)) return;
    const int ax = face >> 1;
    int lo = 0, hi = fl.ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (fl.inst[mid].fpre[ax] <= t) lo = mid; else hi = mid - 1;
    }
    const Inst& I = fl.inst[lo];
    const long long r = t - I.fpre[ax];
    int i, j, k;
    if (ax == 0) { i = (face == 0) ? 0 : I.ni - 1; j = (int)(r % I.nj); k = (int)(r / I.nj); }
    else if (ax == 1) { j = (face == 2) ? 0 : I.nj - 1; i = (int)(r % I.ni); k = (int)(r / I.ni); }
    else { k = (face == 4) ? 0 : I.nk - 1; i = (int)(r % I.ni); j = (int)(r / I.ni); }
    const int dir = (face & 1) ? -1 : 1;     // inward direction
    const long long sj = I.ni, sk = (long long)I.ni * I.nj;
    const long long st = ax == 0 ? 1 : (ax == 1 ? sj : sk);
    const long long l = I.off + i + sj * j + sk * k;
    const T g = lam[l];
    T a, c;
    const int type = bc.type[face];
    if (type == 0) { a = T(1); c = T(0); }
    else if (type == 2) { a = T(2); c = T(-1); }
    else {
        const int i2 = ax == 0 ? i + 2 * dir : i, j2 = ax == 1 ? j + 2 * dir : j, k2 = ax == 2 ? k + 2 * dir : k;
        T v2;
        if (kind == 0) {
            P0Stage<T> p0{phin, in, out, I.off, sj, sk, I.ni, I.nj, I.nk, c1, c2};
            v2 = prev_value<T>(bc, p0, face, I.ni, I.nj, i2, j2, k2);
        } else {
            P0Src<T> p0{out, I.off, sj, sk};
            v2 = prev_value<T>(bc, p0, face, I.ni, I.nj, i2, j2, k2);
        }
        if (fabs(v2) >= T(bc.BigPhi)) { a = T(1); c = T(0); }
        else { a = T(4.0 / 3.0); c = T(-1.0 / 3.0); }
    }
    lam[l + dir * st] += a * g;
    lam[l + 2 * dir * st] += c * g;
    lam[l] = T(0);
}

// value and gradient of rec3 (one reciprocal)
template <typename T>
__device__ __forceinline__ T rec3_vg(T fL, T fC, T fR, T* dL, T* dC, T* dR) {
    const T eL = fL - fC, eR = fC - fR;
    const T t0 = eR * eR + T(1.0e-6), t1 = eL * eL + T(1.0e-6);
    const T a0 = T(2) * t1 * t1, a1 = t0 * t0;
    const T r = vdiv(T(1), a0 + a1);
    const T w0 = a0 * r;
    const T g = T(0.5) * (fL + fR) - fC;
    // d w0 / d t1 = 4 t1 a1 r^2, d w0 / d t0 = -2 t0 a0 r^2
    const T q1 = T(4) * t1 * a1 * r * r * g, q0 = T(-2) * t0 * a0 * r * r * g;
    *dL = T(-0.5) + T(0.5) * w0 + q1 * (T(2) * eL);
    *dC = T(1.5) - w0 - q1 * (T(2) * eL) + q0 * (T(2) * eR);
    *dR = T(0.5) * w0 - q0 * (T(2) * eR);
    return vfma(w0, g, T(1.5) * fC - T(0.5) * fL);
}

// D = Phi+ - Phi- of a node (stencil s, orientation frozen by w) and the
// gradient G = lp w dD/ds of lp w D, branch-free
template <typename T>
__device__ __forceinline__ T stage_node_grad(const T (&s)[5], T w, T lp, bool lo, bool hi, T (&G)[5]) {
    const bool up = w > T(0);
    const bool P = up || hi, M = up && !lo;
    T a, b, c, a2, b2, c2;
    const T vp = rec3_vg(P ? s[1] : s[4], P ? s[2] : s[3], P ? s[3] : s[2], &a, &b, &c);
    const T vm = rec3_vg(M ? s[0] : s[3], M ? s[1] : s[2], M ? s[2] : s[1], &a2, &b2, &c2);
    const T k = lp * w;
    G[0] = -k * (M ? a2 : T(0));
    G[1] = k * ((P ? a : T(0)) - (M ? b2 : c2));
    G[2] = k * ((P ? b : c) - (M ? c2 : b2));
    G[3] = k * ((P ? c : b) - (M ? T(0) : a2));
    G[4] = k * (P ? T(0) : a);
    return vp - vm;
}

// Stage adjoint, x part (adjoint map 0: bricks of 8 whole rows of one
// plane, one warp per row) plus the pointwise terms.  The warp marches its
// row in aligned chunks of 32 nodes: it evaluates G_x of chunk c + 1, then
// writes chunk c, gathering the five contributions of each node by warp
// shuffles from chunks c - 1, c, c + 1 held in registers.  Each warp starts
// at its own chunk (rows hashed over the row length) and wraps around, so
// that the warps of the GPU do not all stream the same columns at once.
// Writes lam_in = c2 lamP0 - c3 acc_x (+ lamPhin + c1 lamP0 when last),
// updates lamPhin and lamW_x.
template <typename T>
__global__ void __launch_bounds__(256) k_adj_stage_x(const Inst* __restrict__ inst, const Brick* __restrict__ bmap,
        int nb, FieldsT<T> f, const T* __restrict__ in, const T* __restrict__ lamP0, T* __restrict__ lam_in,
        T* __restrict__ lamPhin, T* __restrict__ lamW0, T c1, T c2, T c3, int last) {
    const int lane = threadIdx.x & 31, row = threadIdx.x >> 5;
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 0, blk);
        const Inst& I = inst[ab.inst];
        const int ni = I.ni, nj = I.nj, nk = I.nk;
        const int j = ab.j0 + row, k = ab.k0;
        if (j >= nj) continue;   // whole warp
        const bool jk_int = j >= 1 && j <= nj - 2 && k >= 1 && k <= nk - 2;
        const long long rowbase = I.off + (long long)ni * (j + (long long)nj * k);
        const int nc = (ni + 31) >> 5;
        // G_x of chunk c (zero outside the row and at non-interior nodes)
        auto eval = [&](int c, T (&G)[5], T& D, T& lp) {
#pragma unroll
            for (int p = 0; p < 5; ++p) G[p] = T(0);
            D = lp = T(0);
            const int ii = (c << 5) + lane;
            if (c >= 0 && c < nc && ii < ni) {
                const long long l = rowbase + ii;
                lp = __ldg(lamP0 + l);
                if (jk_int && ii >= 1 && ii <= ni - 2) {
                    const T sv[5] = {ii >= 2 ? __ldg(in + l - 2) : T(0), __ldg(in + l - 1), __ldg(in + l),
                                     __ldg(in + l + 1), ii <= ni - 3 ? __ldg(in + l + 2) : T(0)};
                    D = stage_node_grad(sv, __ldg(f.W[0] + l), lp, ii == 1, ii == ni - 2, G);
                }
            }
        };
        // march chunks a .. b-1 (outputs), with chunk a-1 primed
        auto segment = [&](int a, int b) {
            T Gp[5], Gc[5], Gn[5], Dc, Dn, lpc, lpn;
            eval(a - 1, Gc, Dc, lpc);
#pragma unroll
            for (int p = 0; p < 5; ++p) Gp[p] = T(0);
            for (int c = a; c <= b; ++c) {
                // read-modify-write values of the output chunk c - 1 first, so
                // that their loads are in flight together with chunk c's
                const int io = ((c - 1) << 5) + lane;
                const bool wo = c > a && io < ni;
                const long long lo = rowbase + io;
                T phin_old = T(0), w_old = T(0);
                if (wo) {
                    phin_old = lamPhin[lo];
                    w_old = lamW0[lo];
                }
                eval(c, Gn, Dn, lpn);
                if (c > a) {
                    // node lane + o of chunk c - 1 contributes component 2 - o;
                    // across the chunk edges it lies in chunk c - 2 (Gp) or c (Gn)
                    const unsigned FM = 0xffffffffu;
                    const T m2c = __shfl_sync(FM, Gc[4], (lane - 2) & 31), m2p = __shfl_sync(FM, Gp[4], (lane - 2) & 31);
                    const T m1c = __shfl_sync(FM, Gc[3], (lane - 1) & 31), m1p = __shfl_sync(FM, Gp[3], (lane - 1) & 31);
                    const T p1c = __shfl_sync(FM, Gc[1], (lane + 1) & 31), p1n = __shfl_sync(FM, Gn[1], (lane + 1) & 31);
                    const T p2c = __shfl_sync(FM, Gc[0], (lane + 2) & 31), p2n = __shfl_sync(FM, Gn[0], (lane + 2) & 31);
                    const T acc = (lane >= 2 ? m2c : m2p) + (lane >= 1 ? m1c : m1p) + Gc[2] +
                                  (lane <= 30 ? p1c : p1n) + (lane <= 29 ? p2c : p2n);
                    if (wo) {
                        lamW0[lo] = w_old - c3 * lpc * Dc;
                        T r = c2 * lpc - c3 * acc;
                        if (last) {
                            r += phin_old + c1 * lpc;
                            lamPhin[lo] = T(0);
                        } else {
                            lamPhin[lo] = phin_old + c1 * lpc;
                        }
                        lam_in[lo] = r;
                    }
                }
#pragma unroll
                for (int p = 0; p < 5; ++p) {
                    Gp[p] = Gc[p];
                    Gc[p] = Gn[p];
                }
                Dc = Dn;
                lpc = lpn;
            }
        };
        const int s0 = (int)(((unsigned)(j + 7 * k) * 2654435761u >> 16) % (unsigned)nc);
        segment(s0, nc);
        if (s0 > 0) segment(0, s0);
    }
}

// Stage adjoint, y (AX = 1, adjoint map 1) or z (AX = 2, map 2) part: each
// thread marches one line along AX over adj_shape(map) outputs, keeping
// windows of five G, lamP0 and D values in registers; lam_in -= c3 acc,
// lamW_AX -= c3 lamP0 D.
template <typename T, int AX>
__global__ void __launch_bounds__(256) k_adj_stage_m(const Inst* __restrict__ inst, const Brick* __restrict__ bmap,
        int nb, FieldsT<T> f, const T* __restrict__ in, const T* __restrict__ lamP0, T* __restrict__ lam_in,
        T* __restrict__ lamW, T c3) {
    constexpr int MAP = AX;
    const int tx = threadIdx.x & 31, tq = threadIdx.x >> 5;
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, MAP, blk);
        const Inst& I = inst[ab.inst];
        const int ni = I.ni, nj = I.nj, nk = I.nk;
        const long long sj = ni, sk = (long long)ni * nj;
        const int i = ab.i0 + tx;
        // the other coordinate (k for AX = 1, j for AX = 2) and the march range
        const int c2 = AX == 1 ? ab.k0 + tq : ab.j0 + tq;
        const int n2 = AX == 1 ? nk : nj, nm = AX == 1 ? nj : nk;
        const int m0 = AX == 1 ? ab.j0 : ab.k0;
        const int m1 = min(m0 + (AX == 1 ? adj_shape(1).oy : adj_shape(2).oz), nm);
        const bool col = i < ni && c2 < n2;
        const bool line = col && i >= 1 && i <= ni - 2 && c2 >= 1 && c2 <= n2 - 2;
        const long long st = AX == 1 ? sj : sk;
        const long long base = I.off + i + (AX == 1 ? sk * c2 : sj * c2);
        // windows over march positions q-4 .. q (index 0..4)
        T g[5][5], lpw[5], dw[5];
#pragma unroll
        for (int a = 0; a < 5; ++a) {
            lpw[a] = dw[a] = T(0);
#pragma unroll
            for (int p = 0; p < 5; ++p) g[a][p] = T(0);
        }
        for (int q = m0 - 2; q < m1 + 2; ++q) {
            const int jo = q - 2;   // output position: window index 2 after the shift
            const bool wo = col && jo >= m0 && jo < m1;
            const long long lo = base + st * jo;
            T lin_old = T(0), w_old = T(0);
            if (wo) {
                lin_old = lam_in[lo];
                w_old = lamW[lo];
            }
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                lpw[a] = lpw[a + 1];
                dw[a] = dw[a + 1];
#pragma unroll
                for (int p = 0; p < 5; ++p) g[a][p] = g[a + 1][p];
            }
            T G[5] = {T(0), T(0), T(0), T(0), T(0)};
            T D = T(0), lp = T(0);
            if (col && q >= 0 && q < nm) {
                const long long l = base + st * q;
                lp = __ldg(lamP0 + l);
                if (line && q >= 1 && q <= nm - 2) {
                    const T sv[5] = {q >= 2 ? __ldg(in + l - 2 * st) : T(0), __ldg(in + l - st), __ldg(in + l),
                                     __ldg(in + l + st), q <= nm - 3 ? __ldg(in + l + 2 * st) : T(0)};
                    D = stage_node_grad(sv, __ldg(f.W[AX] + l), lp, q == 1, q == nm - 2, G);
                }
            }
            lpw[4] = lp;
            dw[4] = D;
#pragma unroll
            for (int p = 0; p < 5; ++p) g[4][p] = G[p];
            if (wo) {
                T acc = T(0);
#pragma unroll
                for (int o = -2; o <= 2; ++o) acc += g[2 + o][2 - o];
                lam_in[lo] = lin_old - c3 * acc;
                lamW[lo] = w_old - c3 * lpw[2] * dw[2];
            }
        }
    }
}

// Reinitialisation adjoint coefficients of one node from its inputs:
// with w = dtau s lam / (2 G) and the Godunov selections of the forward
// pass, A_m = w dG^2/dmen_m, B_m = w dG^2/dmas_m (a physical face's single
// difference goes to B on the low face, to A on the high face; lo / hi flag
// the node's faces).  Branch-free: with sigma = sign(s) both Godunov
// branches are one, P = sigma max(sigma bb, 0), Q = sigma min(sigma ff, 0),
// and w dG^2/dmen_m = dtau |s| lam / G sum_x M[m][x] (P chosen ? sigma P : 0).
template <typename T>
struct CoefIn {
    T d[7];     // d at the node, -x, +x, -y, +y, -z, +z (any finite value where outside)
    T s, lam;
    T M[9];
};

template <typename T>
__device__ __forceinline__ void coef_eval(const CoefIn<T>& c, T dtau, const bool (&lo)[3], const bool (&hi)[3],
                                          T (&A)[3], T (&B)[3]) {
    const T sg = c.s > T(0) ? T(1) : T(-1);
    T mas[3], men[3];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const T fwd = c.d[2 + 2 * m] - c.d[0], bwd = c.d[0] - c.d[1 + 2 * m];
        mas[m] = sg * (hi[m] ? bwd : fwd);
        men[m] = sg * (lo[m] ? fwd : bwd);
    }
    T e[3], g[3], acc = T(0);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        const T bb = c.M[x] * men[0] + c.M[3 + x] * men[1] + c.M[6 + x] * men[2];   // sigma bb
        const T ff = c.M[x] * mas[0] + c.M[3 + x] * mas[1] + c.M[6 + x] * mas[2];   // sigma ff
        const T p = vmax(bb, T(0)), q = vmin(ff, T(0));
        const bool takeP = p * p >= q * q;
        acc += takeP ? p * p : q * q;
        e[x] = takeP ? p : T(0);
        g[x] = takeP ? T(0) : q;
    }
    const T wgt = (c.s != T(0) && acc > T(0)) ? dtau * fabs(c.s) * c.lam * vrsqrt(acc) : T(0);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const T gmen = c.M[3 * m] * e[0] + c.M[3 * m + 1] * e[1] + c.M[3 * m + 2] * e[2];
        const T gmas = c.M[3 * m] * g[0] + c.M[3 * m + 1] * g[1] + c.M[3 * m + 2] * g[2];
        A[m] = lo[m] ? T(0) : wgt * (hi[m] ? gmen + gmas : gmen);
        B[m] = hi[m] ? T(0) : wgt * (lo[m] ? gmen + gmas : gmas);
    }
}

// Reverse of one reinitialisation pseudo-step d' = d - dtau s (G(d) - 1):
//   lam_out(j) = lam(j) - sum_m [A_m(j) - B_m(j) - A_m(j+e_m) + B_m(j-e_m)]
// (adjoint map 3).  A block of 32 x kReinRY threads covers nodes i0-1 ..
// i0+30, j0-1 .. j0+kReinRY-2 and writes the inner 30 x (kReinRY-2); it
// marches in k.  Iteration k evaluates the coefficients of plane k and
// writes plane k-1.  Each node loads its own d, s, lam and metrics only:
// the x neighbours of d come by warp shuffles (the tile's edge lanes load
// the one outside), the y neighbours from the plane in shared memory (the
// edge rows load the one outside), the z neighbours from a register window
// (d is fetched two planes ahead, the rest one plane ahead).  The
// coefficients travel the same way: A_x / B_x by shuffles, A_y / B_y
// through shared memory, A_z / B_z in registers.  One barrier per plane,
// shared planes double-buffered (a buffer is rewritten two iterations
// later, after every thread has passed the barrier between).
template <typename T>
__global__ void __launch_bounds__(32 * kReinRY, sizeof(T) == 4 ? 2 : 1) k_adj_reinit(const Inst* __restrict__ inst,
        const Brick* __restrict__ bmap, int nb, FieldsT<T> f, const T* __restrict__ d, const T* __restrict__ lam,
        T* __restrict__ lam_out) {
    constexpr int RY = kReinRY;
    __shared__ T sD[2][RY + 2][32];   // row ty + 1 holds row ty (rows 0, RY + 1: padding)
    __shared__ T sA1[2][RY][32], sB1[2][RY][32];
    const unsigned FM = 0xffffffffu;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int blk = blockIdx.x; blk < nb; blk += gridDim.x) {
        const ABrick ab = adj_brick(bmap, 3, blk);
        const Inst& I = inst[ab.inst];
        const int ni = I.ni, nj = I.nj, nk = I.nk;
        const long long sj = ni, sk = (long long)ni * nj;
        const int i = ab.i0 - 1 + tx, j = ab.j0 - 1 + ty;
        const int k0 = ab.k0, k1 = min(k0 + adj_shape(3).oz, nk);
        const bool node = i >= 0 && i < ni && j >= 0 && j < nj;
        const bool out = node && tx >= 1 && tx <= 30 && ty >= 1 && ty <= RY - 2;
        const T dtau = ipar<T>(I.dtau, I.dtau64);
        const long long cb = I.off + i + sj * j;   // this column at k = 0
        // the neighbour outside the tile that edge lanes / rows load
        const int ox = tx == 0 ? -1 : (tx == 31 ? 1 : 0), oy = ty == 0 ? -1 : (ty == RY - 1 ? 1 : 0);
        const bool ldx = node && ox != 0 && i + ox >= 0 && i + ox < ni;
        const bool ldy = node && oy != 0 && j + oy >= 0 && j + oy < nj;
        auto ldd = [&](int k) { return node && k >= 0 && k < nk ? __ldg(d + cb + sk * k) : T(0); };
        // plane-k inputs other than d (plane k evaluated iff 0 <= k < nk, k <= k1)
        struct PlaneIn {
            T s, lam, ex, ey, M[9];
        };
        auto ldp = [&](int k, PlaneIn& q) {
            q.s = q.lam = q.ex = q.ey = T(0);
            if (node && k >= 0 && k < nk && k <= k1) {
                const long long l = cb + sk * k;
                q.s = __ldg(f.sgn + l);
                q.lam = __ldg(lam + l);
                if (ldx) q.ex = __ldg(d + l + ox);
                if (ldy) q.ey = __ldg(d + l + oy * sj);
#pragma unroll
                for (int c = 0; c < 9; ++c) q.M[c] = __ldg(f.m[c] + l);
            }
        };
        __syncthreads();   // the previous tile's readers of sD / sA1 / sB1 are done
        T dm = ldd(k0 - 2), dc = ldd(k0 - 1), dp = ldd(k0);   // d at k-1, k, k+1 for k = k0-1
        PlaneIn cur, nxt;
        ldp(k0 - 1, nxt);
        T Ap[3] = {T(0), T(0), T(0)}, Bp[3] = {T(0), T(0), T(0)}, Bz2 = T(0), lamp = T(0);
        int it = 0;
#pragma unroll 2
        for (int k = k0 - 1; k <= k1; ++k, ++it) {
            cur = nxt;
            const T dnn = ldd(k + 2);   // two planes ahead
            ldp(k + 1, nxt);
            sD[it & 1][ty + 1][tx] = dc;
            if (it > 0) {
                sA1[(it - 1) & 1][ty][tx] = Ap[1];
                sB1[(it - 1) & 1][ty][tx] = Bp[1];
            }
            __syncthreads();
            // neighbours of d at plane k (one-sided copies on physical faces)
            CoefIn<T> c;
            c.s = cur.s;
            c.lam = cur.lam;
#pragma unroll
            for (int q = 0; q < 9; ++q) c.M[q] = cur.M[q];
            c.d[0] = dc;
            const T xl = __shfl_up_sync(FM, dc, 1), xr = __shfl_down_sync(FM, dc, 1);
            c.d[1] = tx == 0 ? cur.ex : xl;
            c.d[2] = tx == 31 ? cur.ex : xr;
            c.d[3] = ty == 0 ? cur.ey : sD[it & 1][ty][tx];
            c.d[4] = ty == RY - 1 ? cur.ey : sD[it & 1][ty + 2][tx];
            c.d[5] = dm;
            c.d[6] = dp;
            const bool lo[3] = {i == 0, j == 0, k == 0}, hi[3] = {i == ni - 1, j == nj - 1, k == nk - 1};
            T A[3], B[3];
            coef_eval(c, dtau, lo, hi, A, B);
            // plane k-1: x neighbours by shuffles, y from shared memory
            const T ax = __shfl_down_sync(FM, Ap[0], 1);
            const T bx = __shfl_up_sync(FM, Bp[0], 1);
            const int ko = k - 1;
            if (out && ko >= k0 && ko < k1) {
                const int q = (it - 1) & 1;
                T t0 = Ap[0] - Bp[0];
                if (i < ni - 1) t0 -= ax;
                if (i > 0) t0 += bx;
                T t1 = Ap[1] - Bp[1];
                if (j < nj - 1) t1 -= sA1[q][ty + 1][tx];
                if (j > 0) t1 += sB1[q][ty - 1][tx];
                T t2 = Ap[2] - Bp[2];
                if (ko < nk - 1) t2 -= A[2];
                if (ko > 0) t2 += Bz2;
                lam_out[cb + sk * ko] = lamp - t0 - t1 - t2;
            }
            Bz2 = Bp[2];
#pragma unroll
            for (int m = 0; m < 3; ++m) {
                Ap[m] = A[m];
                Bp[m] = B[m];
            }
            lamp = cur.lam;
            dm = dc;
            dc = dp;
            dp = dnn;
        }
    }
}

template <typename T>
__global__ void k_adj_contra(Flat fl, FieldsT<T> f, const T* __restrict__ w0, const T* __restrict__ w1,
                             const T* __restrict__ w2, T* __restrict__ u0, T* __restrict__ u1, T* __restrict__ u2) {
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    Node nd;
    if (!flat_node(fl, l, &nd)) return;
    const T dt = ipar<T>(fl.inst[nd.inst].dt, fl.inst[nd.inst].dt64);
    const T lw[3] = {w0[l], w1[l], w2[l]};
    T* out[3] = {u0, u1, u2};
#pragma unroll
    for (int c = 0; c < 3; ++c)
        out[c][l] += dt * (f.m[c][l] * lw[0] + f.m[3 + c][l] * lw[1] + f.m[6 + c][l] * lw[2]);
}

// ------------------------------------------------------------ dispatch
template <template <typename, int, int, int> class Fn, typename T, class... A>
void dispatch(int shape, A... a) {
    if constexpr (sizeof(T) == 8) {
        (void)shape;
        Fn<T, 32, 4, 2>::run(a...);   // FP64 (gradient checks): one tile shape
    } else {
        switch (shape) {
        case 0: Fn<T, 32, 4, 2>::run(a...); break;
        case 1: Fn<T, 32, 8, 1>::run(a...); break;
        case 2: Fn<T, 64, 4, 1>::run(a...); break;
        case 3: Fn<T, 32, 2, 4>::run(a...); break;
        default: Fn<T, 128, 2, 1>::run(a...); break;
        }
    }
}

#define LSM_BATCH_RUNNER(NAME, KERNEL, PARAMS, ARGS)                                   \
    template <typename T, int TX, int TY, int TZ>                                      \
    struct NAME {                                                                       \
        static void run PARAMS {                                                        \
            ProfScope ps_(#KERNEL, s);                                                  \
            KERNEL<T, TX, TY, TZ><<<grid, TX * TY * TZ, 0, s>>> ARGS;                   \
        }                                                                               \
    };

LSM_BATCH_RUNNER(RunContra, k_contra,
                 (int grid, const Inst* inst, const Brick* bi, int nb, FieldsT<T> f, cudaStream_t s),
                 (inst, bi, nb, f))
LSM_BATCH_RUNNER(RunBcFull, k_bc_full,
                 (int grid, const Inst* inst, const Brick* bi, int nb, BC bc, const T* src, T* dst, unsigned* err,
                  cudaStream_t s),
                 (inst, bi, nb, bc, src, dst, err))
LSM_BATCH_RUNNER(RunReinit, k_reinit,
                 (int grid, const Inst* inst, const Brick* bi, int nb, FieldsT<T> f, const T* din, T* dout,
                  unsigned* err, cudaStream_t s),
                 (inst, bi, nb, f, din, dout, err))
LSM_BATCH_RUNNER(RunSignReinit, k_sign_reinit,
                 (int grid, const Inst* inst, const Brick* bi, int nb, FieldsT<T> f, const T* p0, T* dout,
                  unsigned* err, cudaStream_t s),
                 (inst, bi, nb, f, p0, dout, err))

template <typename T, int TX, int TY, int TZ>
struct Occupancy {
    static void run(int kernel, int* out) {
        const int nt = TX * TY * TZ;
        (void)kernel;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, k_contra<T, TX, TY, TZ>, nt, 0);
    }
};

inline unsigned flat_blocks(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

// ------------------------------------------------------------ launchers
template <typename T>
void contra(int shape, int grid, const Inst* inst, const Brick* bi, int nb, FieldsT<T> f, cudaStream_t s) {
    dispatch<RunContra, T>(shape, grid, inst, bi, nb, f, s);
}
template <typename T>
void stage(int grid, const Inst* inst, const Brick* bmap2, int nb, FieldsT<T> f, const T* phin, const T* phi1, T* out,
           double c1, double c2, double c3, cudaStream_t s) {
    ProfScope ps_("k_stage_z", s);
    k_stage_z<T><<<grid, 256, 0, s>>>(inst, bmap2, nb, f, phin, phi1, out, T(c1), T(c2), T(c3));
}
void stage_tma(int grid, const CUtensorMap* tm, int a_in, const Inst* inst, const Brick* bmap2, int nb,
               FieldsT<float> f, const float* phin, const float* phi1, float* out, double c1, double c2, double c3,
               unsigned* err, cudaStream_t s) {
    ProfScope ps_("k_stage_tma", s);
    k_stage_tma<<<grid, 256, 0, s>>>(*tm, a_in, inst, bmap2, nb, f, phin, phi1, out, (float)c1, (float)c2, (float)c3,
                                     err);
}
int stage_tma_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_stage_tma, 256, 0);
    return n;
}
template <typename T>
int stage_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_stage_z<T>, 256, 0);
    return n;
}
template <typename T>
void bc_stage(const Inst* inst, int ninst, long long nface, BC bc, const T* phin, const T* phi1, T* out, double c1,
              double c2, cudaStream_t s) {
    ProfScope ps_("k_bc_stage", s);
    k_bc_stage<T><<<flat_blocks(nface), 256, 0, s>>>(inst, ninst, nface, bc, phin, phi1, out, T(c1), T(c2));
}
template <typename T>
void bc_full(int shape, int grid, const Inst* inst, const Brick* bi, int nb, BC bc, const T* src, T* dst, unsigned* err,
             cudaStream_t s) {
    dispatch<RunBcFull, T>(shape, grid, inst, bi, nb, bc, src, dst, err, s);
}
template <typename T>
void bc_faces(const Inst* inst, int ninst, long long nface, BC bc, const T* src, T* dst, unsigned* err,
              cudaStream_t s) {
    ProfScope ps_("k_bc_faces", s);
    k_bc_faces<T><<<flat_blocks(nface), 256, 0, s>>>(inst, ninst, nface, bc, src, dst, err);
}
template <typename T>
void reinit(int shape, int grid, const Inst* inst, const Brick* bi, int nb, FieldsT<T> f, const T* din, T* dout,
            unsigned* err, cudaStream_t s) {
    dispatch<RunReinit, T>(shape, grid, inst, bi, nb, f, din, dout, err, s);
}
template <typename T>
void sign_reinit(int shape, int grid, const Inst* inst, const Brick* bi, int nb, FieldsT<T> f, const T* phi0,
                 T* dout, unsigned* err, cudaStream_t s) {
    dispatch<RunSignReinit, T>(shape, grid, inst, bi, nb, f, phi0, dout, err, s);
}
template <typename T>
void reinit_z(int kind, int grid, const Inst* inst, const Brick* bmap2, int nb, FieldsT<T> f, const T* din, T* dout,
              T* dout2, T* cf, long long ld, unsigned* err, cudaStream_t s) {
    switch (kind) {
    case 0: {
        ProfScope ps_("k_reinit_z", s);
        k_reinit_z<T, false, false><<<grid, 256, 0, s>>>(inst, bmap2, nb, f, din, dout, dout2, cf, ld, err);
        break;
    }
    case 1: {
        ProfScope ps_("k_reinit_rec_z", s);
        k_reinit_z<T, false, true><<<grid, 256, 0, s>>>(inst, bmap2, nb, f, din, dout, dout2, cf, ld, err);
        break;
    }
    case 2: {
        ProfScope ps_("k_sign_reinit_z", s);
        k_reinit_z<T, true, false><<<grid, 256, 0, s>>>(inst, bmap2, nb, f, din, dout, dout2, cf, ld, err);
        break;
    }
    default: {
        ProfScope ps_("k_sign_reinit_rec_z", s);
        k_reinit_z<T, true, true><<<grid, 256, 0, s>>>(inst, bmap2, nb, f, din, dout, dout2, cf, ld, err);
        break;
    }
    }
}
template <typename T>
int reinit_z_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_reinit_z<T, true, true>, 256, 0);
    return n;
}
template <typename T>
void adj_reinit_c(int grid, const Inst* inst, const Brick* bmap2, int nb, const T* cf, long long ld, const T* lam,
                  T* lam_out, cudaStream_t s) {
    ProfScope ps_("k_adj_reinit_c", s);
    k_adj_reinit_c<T><<<grid, 256, 0, s>>>(inst, bmap2, nb, cf, ld, lam, lam_out);
}
template <typename T>
int adj_reinit_c_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adj_reinit_c<T>, 256, 0);
    return n;
}
template <typename T>
void bc_reinit(const Inst* inst, int ninst, long long nface, FieldsT<T> f, BC bc, const T* din, T* dout,
               cudaStream_t s) {
    ProfScope ps_("k_bc_reinit", s);
    k_bc_reinit<T><<<flat_blocks(nface), 256, 0, s>>>(inst, ninst, nface, bc, f, din, dout);
}
inline unsigned list_blocks() { return 152 * 8; }
template <typename T>
void volume(int grid2, const Inst* inst, const Brick* bmap2, int nb2, const Flat& fl, FieldsT<T> f, const T* phi,
            unsigned long long* acc, bool slope, unsigned* list, unsigned* count, cudaStream_t s) {
    cudaMemsetAsync(count, 0, sizeof(unsigned), s);
    {
        ProfScope ps_("k_vol_scan_z", s);
        k_vol_scan_z<T, true><<<grid2, 256, 0, s>>>(inst, bmap2, nb2, f, phi, acc, list, count);
    }
    if (slope) {
        ProfScope ps_("k_vol_iface_slope", s);
        k_vol_iface<T, true><<<list_blocks(), 128, 0, s>>>(fl, f, phi, list, count, acc);
    } else {
        ProfScope ps_("k_vol_iface", s);
        k_vol_iface<T, false><<<list_blocks(), 128, 0, s>>>(fl, f, phi, list, count, acc);
    }
}
void volume_final(int ninst, unsigned long long* acc, double* vols, const double* target, Mass* mass, Mass* mrec,
                  cudaStream_t s) {
    ProfScope ps_("k_volume_final", s);
    k_volume_final<<<(ninst + 127) / 128, 128, 0, s>>>(ninst, acc, vols, target, mass, mrec);
}
template <typename T>
void mass_shift(const Flat& fl, const Mass* mass, const T* src, T* dst, cudaStream_t s) {
    ProfScope ps_("k_mass_shift", s);
    k_mass_shift<T><<<(unsigned)std::min<long long>((fl.n + 255) / 256, 152 * 16), 256, 0, s>>>(fl, mass, src, dst);
}
template <typename T>
void mass_adjoint(const Inst* inst, const Brick* bmap2, int nb2, const Flat& fl, FieldsT<T> f, const T* phi_pre,
                  const Mass* mass, T* lam, unsigned long long* wfix, double* part, double* ssum, const unsigned* list,
                  const unsigned* count, cudaStream_t s) {
    {
        ProfScope ps_("k_mass_weights", s);
        k_mass_weights<T><<<list_blocks(), 128, 0, s>>>(fl, f, phi_pre, list, count, mass, wfix);
    }
    {
        ProfScope ps_("k_tile_sum", s);
        k_tile_sum<T><<<std::min(nb2, 152 * 8), 256, 0, s>>>(inst, bmap2, nb2, lam, part);
    }
    {
        ProfScope ps_("k_inst_sum", s);
        k_inst_sum<<<fl.ninst, 256, 0, s>>>(inst, part, ssum);
    }
    ProfScope ps_("k_mass_apply", s);
    k_mass_apply<T><<<list_blocks(), 128, 0, s>>>(fl, mass, ssum, list, count, lam, wfix);
}
void w64(long long off, long long n, double dt, const double* const* m64, const double* const* u64,
         double* const* w, cudaStream_t s) {
    ProfScope ps_("k_w64", s);
    k_w64<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 16), 256, 0, s>>>(off, n, dt, m64, u64, w);
}
void cell_hex(long long off, int ni, int nj, int nk, const double* x, const double* y, const double* z,
              long long* cellfix, cudaStream_t s) {
    const long long ncell = (long long)(ni - 1) * (nj - 1) * (nk - 1);
    ProfScope ps_("k_cell_hex", s);
    k_cell_hex<<<(unsigned)std::min<long long>((ncell + 255) / 256, 152 * 16), 256, 0, s>>>(off, ni, nj, nk, x, y, z,
                                                                                             cellfix);
}
void cell_rel(long long off, int ni, int nj, int nk, const double* x, const double* y, const double* z, float* rel,
              cudaStream_t s) {
    const long long ncell = (long long)(ni - 1) * (nj - 1) * (nk - 1);
    ProfScope ps_("k_cell_rel", s);
    k_cell_rel<<<(unsigned)std::min<long long>((ncell + 255) / 256, 152 * 16), 256, 0, s>>>(off, ni, nj, nk, x, y, z,
                                                                                             rel);
}
int max_blocks_per_sm(int shape, int kernel) {
    int n = 0;
    dispatch<Occupancy, float>(shape, kernel, &n);
    return n;
}
template <typename T>
int vol_scan_blocks_per_sm() {
    int n = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_vol_scan_z<T, true>, 256, 0);
    return n;
}

template <typename T>
void adj_face(const Flat& fl, int face, long long nplane, int nface, BC bc, int kind, const T* phin, const T* in,
              const T* out, double c1, double c2, T* lam, cudaStream_t s) {
    ProfScope ps_("k_adj_face", s);
    k_adj_face<T><<<flat_blocks(nplane * nface), 256, 0, s>>>(fl, face, nplane, nface, bc, kind, phin, in, out, T(c1),
                                                              T(c2), lam);
}
template <typename T>
void adj_stage(const int* grid, const Inst* inst, const Brick* const* bmap, const int* nb, FieldsT<T> f, const T* in,
               const T* lamP0, T* lam_in, T* lamPhin, T* lamW0, T* lamW1, T* lamW2, double c1, double c2, double c3,
               bool last, cudaStream_t s) {
    {
        ProfScope ps_("k_adj_stage_x", s);
        k_adj_stage_x<T><<<grid[0], 256, 0, s>>>(inst, bmap[0], nb[0], f, in, lamP0, lam_in, lamPhin, lamW0, T(c1),
                                                 T(c2), T(c3), last ? 1 : 0);
    }
    {
        ProfScope ps_("k_adj_stage_y", s);
        k_adj_stage_m<T, 1><<<grid[1], 256, 0, s>>>(inst, bmap[1], nb[1], f, in, lamP0, lam_in, lamW1, T(c3));
    }
    ProfScope ps_("k_adj_stage_z", s);
    k_adj_stage_m<T, 2><<<grid[2], 256, 0, s>>>(inst, bmap[2], nb[2], f, in, lamP0, lam_in, lamW2, T(c3));
}
template <typename T>
void adj_reinit(int grid, const Inst* inst, const Brick* bmap, int nb, FieldsT<T> f, const T* d, const T* lam,
                T* lam_out, cudaStream_t s) {
    ProfScope ps_("k_adj_reinit", s);
    k_adj_reinit<T><<<grid, 32 * kReinRY, 0, s>>>(inst, bmap, nb, f, d, lam, lam_out);
}
template <typename T>
int adj_blocks_per_sm(int map) {
    int n = 0;
    switch (map) {
    case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adj_stage_x<T>, 256, 0); break;
    case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adj_stage_m<T, 1>, 256, 0); break;
    case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adj_stage_m<T, 2>, 256, 0); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_adj_reinit<T>, 32 * kReinRY, 0); break;
    }
    return n;
}
template <typename T>
void adj_contra(const Flat& fl, FieldsT<T> f, const T* w0, const T* w1, const T* w2, T* u0, T* u1, T* u2,
                cudaStream_t s) {
    ProfScope ps_("k_adj_contra", s);
    k_adj_contra<T><<<flat_blocks(fl.n), 256, 0, s>>>(fl, f, w0, w1, w2, u0, u1, u2);
}

#define LSM_BATCH_INSTANTIATE(T)                                                                                      \
    template void contra<T>(int, int, const Inst*, const Brick*, int, FieldsT<T>, cudaStream_t);                       \
    template int stage_blocks_per_sm<T>();                                                                      \
    template void stage<T>(int, const Inst*, const Brick*, int, FieldsT<T>, const T*, const T*, T*, double,            \
                           double, double, cudaStream_t);                                                                     \
    template void bc_stage<T>(const Inst*, int, long long, BC, const T*, const T*, T*, double, double, cudaStream_t);   \
    template void bc_full<T>(int, int, const Inst*, const Brick*, int, BC, const T*, T*, unsigned*, cudaStream_t);      \
    template void bc_faces<T>(const Inst*, int, long long, BC, const T*, T*, unsigned*, cudaStream_t);                 \
    template void bc_reinit<T>(const Inst*, int, long long, FieldsT<T>, BC, const T*, T*, cudaStream_t);              \
    template void reinit<T>(int, int, const Inst*, const Brick*, int, FieldsT<T>, const T*, T*, unsigned*,             \
                            cudaStream_t);                                                                            \
    template void sign_reinit<T>(int, int, const Inst*, const Brick*, int, FieldsT<T>, const T*, T*, unsigned*,      \
                                 cudaStream_t);                                                                   \
    template void reinit_z<T>(int, int, const Inst*, const Brick*, int, FieldsT<T>, const T*, T*, T*, T*, long long, \
                              unsigned*, cudaStream_t);                                                         \
    template int reinit_z_blocks_per_sm<T>();                                                                   \
    template void adj_reinit_c<T>(int, const Inst*, const Brick*, int, const T*, long long, const T*, T*,           \
                                  cudaStream_t);                                                                \
    template int adj_reinit_c_blocks_per_sm<T>();                                                               \
    template void volume<T>(int, const Inst*, const Brick*, int, const Flat&, FieldsT<T>, const T*,                \
                            unsigned long long*, bool, unsigned*, unsigned*, cudaStream_t);                          \
    template int vol_scan_blocks_per_sm<T>();                                                                   \
    template void mass_shift<T>(const Flat&, const Mass*, const T*, T*, cudaStream_t);                                 \
    template void mass_adjoint<T>(const Inst*, const Brick*, int, const Flat&, FieldsT<T>, const T*, const Mass*,  \
                                  T*, unsigned long long*, double*, double*, const unsigned*, const unsigned*,          \
                                  cudaStream_t);                                                                     \
    template void adj_face<T>(const Flat&, int, long long, int, BC, int, const T*, const T*, const T*, double, double, \
                              T*, cudaStream_t);                                                                     \
    template void adj_stage<T>(const int*, const Inst*, const Brick* const*, const int*, FieldsT<T>, const T*,      \
                               const T*, T*, T*, T*, T*, T*, double, double, double, bool, cudaStream_t);      \
    template void adj_reinit<T>(int, const Inst*, const Brick*, int, FieldsT<T>, const T*, const T*, T*,            \
                                cudaStream_t);                                                                \
    template int adj_blocks_per_sm<T>(int);                                                                     \
    template void adj_contra<T>(const Flat&, FieldsT<T>, const T*, const T*, const T*, T*, T*, T*, cudaStream_t);

LSM_BATCH_INSTANTIATE(float)
LSM_BATCH_INSTANTIATE(double)

}  // namespace batch
}  // namespace lsm
