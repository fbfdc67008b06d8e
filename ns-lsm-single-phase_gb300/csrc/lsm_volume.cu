// lsm_volume.cu -- total water volume (FP64), the AdvectionNodes band and
// the ghost-fluid node list.  Compiled with --fmad=false: per-cell volumes
// and band membership are bit-identical to the reference's arithmetic; the
// three volume sums are deterministic fixed-order trees (block tree, then
// one block over the block partials) instead of the reference's sequential
// k-j-i accumulation.
//
// Roofline: one cell reads 8 phi + 24 coordinates, but 7 of every 8 come
// from neighbouring cells through L1/L2, so the algorithmic HBM traffic is
// 4 words per cell (phi, x, y, z); interface cells cost ~100x the flops of
// bulk cells and are rare.
#include <cuda_runtime.h>

#include "lsm_common.cuh"
#include "lsm_kernels.h"
#include "lsm_volume_dev.cuh"

namespace lsm {
namespace {

constexpr int VOL_THREADS = 256;

struct CellBox {
    int i0, j0, k0, Ni, Nj, Nk;       // base cells
    int ista, iend, jsta, jend, ksta, kend;  // clamp range of the band search
};

__host__ __device__ inline CellBox cell_box(const DevGrid& g) {
    CellBox b;
    b.i0 = g.ia; b.j0 = g.ja; b.k0 = g.ka;
    b.Ni = (g.ib - (g.pf ? 1 : 0)) - g.ia + 1;
    b.Nj = (g.jb - (g.pr ? 1 : 0)) - g.ja + 1;
    b.Nk = (g.kb - (g.pu ? 1 : 0)) - g.ka + 1;
    b.ista = g.pb ? g.ia : 0; b.iend = g.pf ? g.ib : g.ni - 1;
    b.jsta = g.pl ? g.ja : 0; b.jend = g.pr ? g.jb : g.nj - 1;
    b.ksta = g.pd ? g.ka : 0; b.kend = g.pu ? g.kb : g.nk - 1;
    return b;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// One thread per base cell (TotalWaterVolume.F90:136-294); block partials
// written in a fixed tree order.
__global__ void __launch_bounds__(VOL_THREADS) volume_kernel(DevGrid g, CellBox cb,
        const double* __restrict__ phi, const double* __restrict__ x, const double* __restrict__ y,
        const double* __restrict__ z, double* __restrict__ partials, unsigned char* __restrict__ pcflag,
        double* __restrict__ cellvol, unsigned* err) {
    const long long ncell = (long long)cb.Ni * cb.Nj * cb.Nk;
    const long long t = blockIdx.x * (long long)VOL_THREADS + threadIdx.x;
    double K = 0.0, S = 0.0, B = 0.0;
    if (t < ncell) {
        const int i = cb.i0 + (int)(t % cb.Ni);
        const int j = cb.j0 + (int)((t / cb.Ni) % cb.Nj);
        const int k = cb.k0 + (int)(t / ((long long)cb.Ni * cb.Nj));
        const long long l = gid(g, i, j, k);
        if (pcflag) {
            // phase-change node test, TotalWaterVolume.F90:169-224
            const double f = phi[l];
            const double sg = copysign(1.0, f);
            bool pc = fabs(f) < kEpsSims;
            const int km = max(k - 1, cb.ksta), kp = min(k + 1, cb.kend);
            const int jm = max(j - 1, cb.jsta), jp = min(j + 1, cb.jend);
            const int im = max(i - 1, cb.ista), ip = min(i + 1, cb.iend);
            for (int ks = km; ks <= kp && !pc; ++ks)
                for (int js = jm; js <= jp && !pc; ++js)
                    for (int is = im; is <= ip && !pc; ++is) {
                        const double h = phi[gid(g, is, js, ks)];
                        if (sg * h < 0.0 || fabs(h) < kEpsSims) pc = true;
                    }
            pcflag[l] = pc ? 1 : 0;
        }
        const long long o[8] = {l, l + 1, l + 1 + g.sj, l + g.sj,
                                l + g.sk, l + 1 + g.sk, l + 1 + g.sj + g.sk, l + g.sj + g.sk};
        double P[8];
        bool allw = true, alla = true;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            P[v] = __ldg(phi + o[v]);
            allw &= P[v] > kEpsSims; alla &= P[v] < -kEpsSims;
        }
        if (!alla) {
            double C[8][3];
#pragma unroll
            for (int v = 0; v < 8; ++v) {
                C[v][0] = __ldg(x + o[v]); C[v][1] = __ldg(y + o[v]); C[v][2] = __ldg(z + o[v]);
            }
            if (allw) B = hex_volume(C);
            else cell_analysis<true>(P, C, &K, &S, err);
        }
        if (cellvol) cellvol[l] = K + S + B;
    }
    // fixed-order block reduction of (K, S, B)
    __shared__ double sh[3][VOL_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    K = warp_sum(K); S = warp_sum(S); B = warp_sum(B);
    if (lane == 0) { sh[0][w] = K; sh[1][w] = S; sh[2][w] = B; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double acc = 0.0;
        for (int q = 0; q < VOL_THREADS / 32; ++q) acc = acc + sh[threadIdx.x][q];
        partials[3 * (long long)blockIdx.x + threadIdx.x] = acc;
    }
}

// One block folds the block partials in a fixed order; result = (VK, V2, VB, total).
__global__ void __launch_bounds__(1024) volume_final_kernel(const double* __restrict__ partials, int nblk,
                                                            double* __restrict__ result) {
    __shared__ double sh[3][32];
    double acc[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nblk; b += 1024) {
        acc[0] = acc[0] + partials[3 * (long long)b];
        acc[1] = acc[1] + partials[3 * (long long)b + 1];
        acc[2] = acc[2] + partials[3 * (long long)b + 2];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double v = warp_sum(acc[c]);
        if (lane == 0) sh[c][w] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double v[3];
        for (int c = 0; c < 3; ++c) {
            double a = 0.0;
            for (int q = 0; q < 32; ++q) a = a + sh[c][q];
            v[c] = a;
        }
        result[0] = v[0]; result[1] = v[1]; result[2] = v[2];
        result[3] = v[0] + v[1] + v[2];
    }
}

// AdvectionNodes: the clamped 3x3x3 box of every phase-change base node is
// marked (TotalWaterVolume.F90:227-235), evaluated as a gather per node.
__global__ void adv_nodes_kernel(DevGrid g, CellBox cb, const unsigned char* __restrict__ pcflag,
                                 int* __restrict__ adv) {
    const long long n = (long long)g.ni * g.nj * g.nk;
    const long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (l >= n) return;
    const int i = (int)(l % g.ni), j = (int)((l / g.ni) % g.nj), k = (int)(l / ((long long)g.ni * g.nj));
    int a = 0;
    if (i >= cb.ista && i <= cb.iend && j >= cb.jsta && j <= cb.jend && k >= cb.ksta && k <= cb.kend) {
        const int bi0 = max(i - 1, cb.i0), bi1 = min(i + 1, cb.i0 + cb.Ni - 1);
        const int bj0 = max(j - 1, cb.j0), bj1 = min(j + 1, cb.j0 + cb.Nj - 1);
        const int bk0 = max(k - 1, cb.k0), bk1 = min(k + 1, cb.k0 + cb.Nk - 1);
        for (int bk = bk0; bk <= bk1 && !a; ++bk)
            for (int bj = bj0; bj <= bj1 && !a; ++bj)
                for (int bi = bi0; bi <= bi1 && !a; ++bi)
                    if (pcflag[gid(g, bi, bj, bk)]) a = 1;
    }
    adv[l] = a;
}

// ---------------------------------------------------------------- N3 ----
// get_gfm_list, src/get_gfm_list.F90:1-143: flag -> block counts -> scan ->
// ordered scatter.  The box is walked in Fortran (k, j, i) order, i.e. in
// increasing linear index, so the list order is the reference's.
constexpr int GFM_THREADS = 256;

struct GfmBox { int i0, j0, k0, Ni, Nj, Nk; };

__host__ __device__ inline GfmBox gfm_box(const DevGrid& g) {
    GfmBox b;
    b.i0 = g.ia + g.pb; b.j0 = g.ja + g.pl; b.k0 = g.ka + g.pd;
    b.Ni = (g.ib - g.pf) - b.i0 + 1; b.Nj = (g.jb - g.pr) - b.j0 + 1; b.Nk = (g.kb - g.pu) - b.k0 + 1;
    return b;
}

__device__ __forceinline__ bool gfm_flag(const DevGrid& g, const GfmBox& b, double BigPhi,
                                         const double* __restrict__ phi, long long t, int* pi, int* pj, int* pk) {
    const long long T = (long long)b.Ni * b.Nj * b.Nk;
    if (t >= T) return false;
    const int i = b.i0 + (int)(t % b.Ni), j = b.j0 + (int)((t / b.Ni) % b.Nj),
              k = b.k0 + (int)(t / ((long long)b.Ni * b.Nj));
    *pi = i; *pj = j; *pk = k;
    const double f = phi[gid(g, i, j, k)];
    if (f > kEpsSims || fabs(f) > BigPhi) return false;
    for (int kk = k - 1; kk <= k + 1; ++kk)
        for (int jj = j - 1; jj <= j + 1; ++jj)
            for (int ii = i - 1; ii <= i + 1; ++ii)
                if (phi[gid(g, ii, jj, kk)] > kEpsSims) return true;
    return false;
}

__global__ void __launch_bounds__(GFM_THREADS) gfm_count_kernel(DevGrid g, GfmBox b, double BigPhi,
                                                                const double* __restrict__ phi, int* counts) {
    const long long t = blockIdx.x * (long long)GFM_THREADS + threadIdx.x;
    int i, j, k;
    const int f = gfm_flag(g, b, BigPhi, phi, t, &i, &j, &k) ? 1 : 0;
    const int c = __syncthreads_count(f);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

// exclusive scan of the block counts (one block, sequential chunks per thread)
__global__ void __launch_bounds__(1024) gfm_scan_kernel(int* counts, int nblk, int* total) {
    __shared__ int sh[1024];
    const int per = (nblk + 1023) / 1024;
    const int b0 = threadIdx.x * per, b1 = min(b0 + per, nblk);
    int sum = 0;
    for (int b = b0; b < b1; ++b) sum += counts[b];
    sh[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    int run = sh[threadIdx.x] - sum;
    for (int b = b0; b < b1; ++b) {
        const int c = counts[b];
        counts[b] = run;
        run += c;
    }
    if (threadIdx.x == 1023) *total = sh[1023];
}

__global__ void __launch_bounds__(GFM_THREADS) gfm_scatter_kernel(DevGrid g, GfmBox b, double BigPhi,
        const double* __restrict__ phi, const int* __restrict__ offsets, int il, int jl, int kl,
        int* __restrict__ list, int ld) {
    const long long t = blockIdx.x * (long long)GFM_THREADS + threadIdx.x;
    int i = 0, j = 0, k = 0;
    const bool f = gfm_flag(g, b, BigPhi, phi, t, &i, &j, &k);
    const unsigned m = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __shared__ int wsum[GFM_THREADS / 32];
    if (lane == 0) wsum[w] = __popc(m);
    __syncthreads();
    int base = offsets[blockIdx.x];
    for (int q = 0; q < w; ++q) base += wsum[q];
    if (f) {
        const int pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < ld) {
            list[pos] = i + il;
            list[pos + (long long)ld] = j + jl;
            list[pos + 2 * (long long)ld] = k + kl;
        }
    }
}

}  // namespace

int volume_partial_blocks(const DevGrid& g) {
    const CellBox cb = cell_box(g);
    const long long ncell = (long long)cb.Ni * cb.Nj * cb.Nk;
    return (int)((ncell + VOL_THREADS - 1) / VOL_THREADS);
}

void launch_volume(const DevGrid& g, const double* phi, const double* x, const double* y, const double* z,
                   double* partials, double* result, unsigned char* pcflag, double* cellvol, unsigned* err,
                   cudaStream_t s) {
    const CellBox cb = cell_box(g);
    const int nblk = volume_partial_blocks(g);
    {
        ProfScope ps_("volume_kernel", s);
        volume_kernel<<<nblk, VOL_THREADS, 0, s>>>(g, cb, phi, x, y, z, partials, pcflag, cellvol, err);
    }
    ProfScope ps_("volume_final_kernel", s);
    volume_final_kernel<<<1, 1024, 0, s>>>(partials, nblk, result);
}

void launch_adv_nodes(const DevGrid& g, const unsigned char* pcflag, int* adv, cudaStream_t s) {
    const long long n = (long long)g.ni * g.nj * g.nk;
    ProfScope ps_("adv_nodes_kernel", s);
    adv_nodes_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, cell_box(g), pcflag, adv);
}

long long gfm_scratch_ints(const DevGrid& g) {
    const GfmBox b = gfm_box(g);
    const long long T = (long long)b.Ni * b.Nj * b.Nk;
    return (T + GFM_THREADS - 1) / GFM_THREADS;
}

// Passes 1-2 when list == nullptr (count only), pass 3 otherwise (the caller
// has already run passes 1-2 on the same scratch and checked the capacity).
void launch_gfm_list(const DevGrid& g, double BigPhi, const double* phi, int* scratch, int* count_out, int* list,
                     int ld, int il, int jl, int kl, cudaStream_t s) {
    const GfmBox b = gfm_box(g);
    const int nblk = (int)gfm_scratch_ints(g);
    if (!list) {
        {
            ProfScope ps_("gfm_count_kernel", s);
            gfm_count_kernel<<<nblk, GFM_THREADS, 0, s>>>(g, b, BigPhi, phi, scratch);
        }
        ProfScope ps_("gfm_scan_kernel", s);
        gfm_scan_kernel<<<1, 1024, 0, s>>>(scratch, nblk, count_out);
    } else {
        ProfScope ps_("gfm_scatter_kernel", s);
        gfm_scatter_kernel<<<nblk, GFM_THREADS, 0, s>>>(g, b, BigPhi, phi, scratch, il, jl, kl, list, ld);
    }
}

}  // namespace lsm
