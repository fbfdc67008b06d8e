// lsm_batch.cuh -- device descriptors and host launchers of the batched FP32
// level-set path (many independent instances of uneven sizes per launch).
//
// Layout in HBM: every field of every instance is packed into one array per
// field (instance after instance, each in the reference's i-fastest order);
// vector fields are split into components (SoA), so each component of a
// warp's 32 consecutive i is one 128-byte line.  Instance b occupies nodes
// [off_b, off_b + ni*nj*nk) of every packed array.  All faces of an
// instance are physical boundaries (one rank per instance, no ghosts).
#pragma once

#include <cuda_runtime.h>

namespace lsm {
namespace batch {

struct Inst {
    long long off;     // first node of the instance in the packed arrays
    int ni, nj, nk;
    int brick0;        // first brick of the instance in the current brick map
    int nbx, nby;      // bricks per row / per plane of the instance
    float dt;          // advection time step (already multiplied into W)
    float dtau;        // reinitialisation pseudo time step
    float eps;         // smoothing half-width epslsm
    float pad;
    long long face0;   // first boundary-face node of the instance (bc kernels)
    long long cell0;   // unused slot kept for alignment
};

// Packed fields of one batch (device pointers).
struct Fields {
    float* phi;        // level set (state; start and end of every step)
    float* stage[2];   // RK stage ping-pong
    float* d[2];       // reinitialisation ping-pong
    float* W[3];       // dt * d_m * (grad xi_m . u): contravariant velocity x dt
    float* m[9];       // metrics: csi_x, csi_y, csi_z, eta_x, ..., zet_z
    float* u[3];       // Cartesian velocity
    float* sgn;        // sign field of the reinitialisation (0 where the lambda correction freezes d)
    const double* xyz[3];  // FP64 coordinates (volume)
};

struct BC {
    int type[6];
    float BigPhi;
};

// tile shapes the autotuner chooses from (threads per brick = TX*TY*TZ)
constexpr int kNumShapes = 5;
struct Shape { int tx, ty, tz; };
constexpr Shape kShapes[kNumShapes] = {{32, 4, 2}, {32, 8, 1}, {64, 4, 1}, {32, 2, 4}, {128, 2, 1}};

// launchers (shape = index into kShapes); grid = persistent CTA count
void contra(int shape, int grid, const Inst* inst, const int* brick_inst, int nbricks, Fields f, float dcm[3],
            cudaStream_t s);
void stage(int shape, int grid, const Inst* inst, const int* brick_inst, int nbricks, Fields f, const float* phin,
           const float* phi1, float* out, float c1, float c2, float c3, cudaStream_t s);
void bc_stage(const Inst* inst, int ninst, long long nface, Fields f, BC bc, const float* phin, const float* phi1,
              float* out, float c1, float c2, cudaStream_t s);
void bc_full(int shape, int grid, const Inst* inst, const int* brick_inst, int nbricks, BC bc, const float* src,
             float* dst, unsigned* err, cudaStream_t s);
void sign(int shape, int grid, const Inst* inst, const int* brick_inst, int nbricks, Fields f, const float* phi0,
          cudaStream_t s);
void reinit(int shape, int grid, const Inst* inst, const int* brick_inst, int nbricks, Fields f, const float* din,
            float* dout, cudaStream_t s);
void volume(int shape, int grid, const Inst* inst, const int* brick_inst, int nbricks, Fields f, const float* phi,
            double* partials, cudaStream_t s);
void volume_final(const Inst* inst, int ninst, const int* brick_inst, int nbricks, const double* partials,
                  double* vols, cudaStream_t s);
int max_blocks_per_sm(int shape, int kernel);

}  // namespace batch
}  // namespace lsm
