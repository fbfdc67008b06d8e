// lsm_common.cuh -- device-side grid descriptor and helpers shared by the
// level-set kernels.
//
// Layout in HBM: every scalar field is one contiguous FP64 (or FP32) array in
// the reference's Fortran order (i fastest, then j, then k) over the full
// bounds (il:iu, jl:ju, kl:ku), ghost planes included; vector fields keep the
// reference's (1:3, i, j, k) order with the component fastest, so a warp that
// walks 32 consecutive i reads 96 contiguous words of a metric row.  Indices
// inside kernels are 0-based offsets from (il, jl, kl).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace lsm {

struct DevGrid {
    int ni, nj, nk;          // full extents (ghosts included)
    long long sj, sk;        // strides of j and k
    int ia, ib, ja, jb, ka, kb;  // non-ghost range (0-based, inclusive)
    int pb, pf, pl, pr, pd, pu;  // physical faces i1, im, j1, jm, k1, km
    double dc, de, dz;       // 1/dxi, 1/deta, 1/dzeta
};

__host__ __device__ inline long long gid(const DevGrid& g, int i, int j, int k) {
    return (long long)i + g.sj * j + g.sk * k;
}

// Boundary-condition description handed to the bcond kernels.
struct DevBC {
    int type[6];     // btype_lsm per face (i1, im, j1, jm, k1, km)
    double BigPhi;
};

// Device error flags (bit mask) written by kernels, read by the host.
enum : unsigned {
    kErrNegativeVolume = 1u,
    kErrNonFinite = 2u,
    kErrTimeout = 4u,   // a bounded wait on an asynchronous copy gave up
};

constexpr double kPi = 3.141592653589793;     // src/precision.F90:51
constexpr double kEpsSims = 2.220446049250313e-16;  // epsilon(1d0), src/precision.F90:62
constexpr double kTinyD = 2.2250738585072014e-308;  // tiny(1d0)

}  // namespace lsm
