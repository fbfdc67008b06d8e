// lsm_batch.cuh -- device descriptors and host launchers of the batched
// level-set path (many independent instances of uneven sizes per launch),
// forward and adjoint, in FP32 (throughput) or FP64 (gradient checks).
//
// Layout in HBM: every field of every instance is packed into one array per
// field (instance after instance, each in the reference's i-fastest order);
// vector fields are split into components (SoA), so each component of a
// warp's 32 consecutive i is one 128-byte line.  Instance b occupies nodes
// [off_b, off_b + ni*nj*nk) of every packed array.  All faces of an
// instance are physical boundaries (one rank per instance, no ghosts).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace lsm {
namespace batch {

struct Inst {
    long long off;     // first node of the instance in the packed arrays
    int ni, nj, nk;
    int brick0;        // first brick of the instance in the current brick map
    int nbx, nby;      // bricks per row / per plane of the instance
    float dt;          // advection time step (multiplied into W)
    float dtau;        // reinitialisation pseudo time step
    float eps;         // smoothing half-width epslsm
    float pad;
    long long face0;   // first boundary-face node of the instance (forward bc kernels)
    long long fpre[3]; // first node of the instance's i-, j-, k-face planes (adjoint face kernels)
    double dt64, dtau64, eps64;  // the same three parameters for the FP64 kernels
    int am[4][3];                // adjoint brick maps (adj_shape): first brick, bricks per row, per plane
};

// Packed fields of one batch (device pointers), scalar type T.
template <typename T>
struct FieldsT {
    T* phi;            // level set (state; start and end of every step)
    T* stage[2];       // RK stage ping-pong
    T* d[2];           // reinitialisation ping-pong
    T* W[3];           // dt * d_m * (grad xi_m . u): contravariant velocity x dt
    T* m[9];           // metrics: csi_x, csi_y, csi_z, eta_x, ..., zet_z
    T* u[3];           // Cartesian velocity
    T* sgn;            // sign field of the reinitialisation (0 where the lambda correction freezes d)
    const double* xyz[3];  // FP64 coordinates (volume)
    const double* W64[3];  // FP32 batches: W in FP64 (from the FP64 metrics and velocity) for the
                           // stage nodes within kBand64 eps of the interface; nullptr: not kept
    long long* cellfix;    // hexahedron volume of cell (i..i+1, j..j+1, k..k+1) in fixed point, by base node
    // FP32 batches: per cell (by base node, 24 floats apart) the FP32
    // coordinates of its vertices 1..7 relative to vertex 0 (differences
    // formed in FP64), 21 values and 3 of padding; nullptr: formed per use
    const float* cellrel;
};
using Fields = FieldsT<float>;

// Stage nodes whose input |phi| is below kBand64 * eps combine the RK stage
// with the FP64 contravariant velocity and in FP64 (FP32 batches).
constexpr float kBand64 = 1.0f;

// Batched water volumes are accumulated as 64-bit fixed point: each cell's
// FP64 volume is rounded to a multiple of 2^-48 (coordinate units^3) and the
// integers are summed, which is exact and independent of the summation
// order.  Valid while an instance's volume stays below 2^15 units^3.
constexpr double kVolScale = 281474976710656.0;       // 2^48
constexpr double kVolUnit = 1.0 / 281474976710656.0;  // 2^-48

// Mass correction of one instance for one step (FP64): the water volume V
// of the step's result before the correction, A = dK/dC, the derivative of
// that volume under a uniform shift phi + C (only the interface cells'
// K tetrahedra depend on it), the shift C = (target - V) / A that was
// applied, and the instance's target volume (NaN: no correction).
struct Mass {
    double V, A, C, target;
};
__host__ __device__ inline bool mass_on(const Mass& m) {
    const double c = (m.target - m.V) / m.A;
    return m.target == m.target && m.A > 0.0 && c - c == 0.0;   // finite target, slope and shift
}

struct BC {
    int type[6];
    float BigPhi;
};

// One brick of a brick table: its instance and brick coordinates.
struct __align__(16) Brick {
    int inst, bx, by, bz;
};

// A flat walk of the packed nodes (one thread per node, the instance found
// by binary search over the node offsets).
struct Flat {
    const Inst* inst;
    const long long* offs;  // ninst + 1 node offsets
    int ninst;
    long long n;            // total nodes
};

// tile shapes the autotuner chooses from (threads per brick = TX*TY*TZ)
constexpr int kNumShapes = 5;
struct Shape { int tx, ty, tz; };
constexpr Shape kShapes[kNumShapes] = {{32, 4, 2}, {32, 8, 1}, {64, 4, 1}, {32, 2, 4}, {128, 2, 1}};

// ------------------------------------------------------------ forward
// (shape = index into kShapes; FP64 instantiations exist for shape 0 only)
template <typename T>
void contra(int shape, int grid, const Inst* inst, const Brick* bricks, int nbricks, FieldsT<T> f,
            cudaStream_t s);
// RK stage out = c1 phin + c2 phi1 - c3 dt aj RH(phi1) on the tiles of
// adjoint map 2 (z march, shared-memory planes); grid from
// stage_blocks_per_sm
template <typename T>
void stage(int grid, const Inst* inst, const Brick* bmap2, int nb, FieldsT<T> f, const T* phin, const T* phi1,
           T* out, double c1, double c2, double c3, cudaStream_t s);
template <typename T>
int stage_blocks_per_sm();
// The same stage (FP32) with each plane's tile + two-node halo staged in
// shared memory by TMA copies: a batch of one instance with ni a multiple
// of 4; phi1 is array a_in of the 4-D tensor map tm (ni, nj, nk, arrays);
// err gets kErrTimeout if a copy's completion never arrived
void stage_tma(int grid, const CUtensorMap* tm, int a_in, const Inst* inst, const Brick* bmap2, int nb,
               FieldsT<float> f, const float* phin, const float* phi1, float* out, double c1, double c2, double c3,
               unsigned* err, cudaStream_t s);
int stage_tma_blocks_per_sm();
template <typename T>
void bc_stage(const Inst* inst, int ninst, long long nface, BC bc, const T* phin, const T* phi1, T* out, double c1,
              double c2, cudaStream_t s);
template <typename T>
void bc_full(int shape, int grid, const Inst* inst, const Brick* bricks, int nbricks, BC bc, const T* src, T* dst,
             unsigned* err, cudaStream_t s);
// bcond_lsm on the face nodes of dst only, from the pre-BC field src (the
// interior of dst already equals src)
template <typename T>
void bc_faces(const Inst* inst, int ninst, long long nface, BC bc, const T* src, T* dst, unsigned* err, cudaStream_t s);
// one reinitialisation pseudo-step on the brick table (the sign field
// fused with the first one in sign_reinit)
template <typename T>
void reinit(int shape, int grid, const Inst* inst, const Brick* bricks, int nbricks, FieldsT<T> f, const T* din,
            T* dout, unsigned* err, cudaStream_t s);
template <typename T>
void sign_reinit(int shape, int grid, const Inst* inst, const Brick* bricks, int nbricks, FieldsT<T> f,
                 const T* phi0, T* dout, unsigned* err, cudaStream_t s);
// bcond_lsm on the output of the last reinitialisation pseudo-step (dout):
// boundary values are recomputed pointwise from that step's input din.
template <typename T>
void bc_reinit(const Inst* inst, int ninst, long long nface, FieldsT<T> f, BC bc, const T* din, T* dout,
               cudaStream_t s);
// One reinitialisation pseudo-step on the tiles of adjoint map 2 (z march;
// grid from reinit_z_blocks_per_sm): kind 0 plain, 1 recorded (the
// pseudo-step's adjoint coefficients A'_0..2, B'_0..2 also written to cf,
// arrays ld apart), 2 the sign field of phi0 (din) fused with the first
// pseudo-step, 3 the same recorded; dout2 (nullable) gets a second copy of
// the output
template <typename T>
void reinit_z(int kind, int grid, const Inst* inst, const Brick* bmap2, int nb, FieldsT<T> f, const T* din, T* dout,
              T* dout2, T* cf, long long ld, unsigned* err, cudaStream_t s);
template <typename T>
int reinit_z_blocks_per_sm();
// water volume of every instance: the cells' 64-bit fixed-point sums (K, S,
// bulk and, with `slope`, dK/dC) are added to acc[4 * inst + c] (zero on
// entry) by a streaming pass over the tiles of map 2 (grid2 CTAs) that also
// lists the interface cells (list: at least one entry per cell of the batch;
// count: one word, reset here) and a pass over that list; volume_final writes vols[4 * inst + 0..3] = (K, S,
// bulk, total) and clears acc; with `mass` (target volumes `target`, NaN =
// none) it also forms each instance's mass correction into mass[inst] and,
// when mrec is not null, mrec[inst]
template <typename T>
void volume(int grid2, const Inst* inst, const Brick* bmap2, int nb2, const Flat& fl, FieldsT<T> f, const T* phi,
            unsigned long long* acc, bool slope, unsigned* list, unsigned* count, cudaStream_t s);
template <typename T>
int vol_scan_blocks_per_sm();
void volume_final(int ninst, unsigned long long* acc, double* vols, const double* target, Mass* mass, Mass* mrec,
                  cudaStream_t s);
// FP64 W = dt (grad xi_m . u) of one instance (n nodes from `off`) from the
// FP64 metrics m64[9] and velocity u64[3] (arrays of device pointers, in
// device memory)
void w64(long long off, long long n, double dt, const double* const* m64, const double* const* u64,
         double* const* w, cudaStream_t s);
// fixed-point hexahedron volume of every cell of one instance (static
// geometry); x, y, z and cellfix are the packed base arrays, `off` the
// instance's first node
void cell_hex(long long off, int ni, int nj, int nk, const double* x, const double* y, const double* z,
              long long* cellfix, cudaStream_t s);
// the relative vertex coordinates of every cell of one instance (FieldsT
// cellrel; the same packed base arrays)
void cell_rel(long long off, int ni, int nj, int nk, const double* x, const double* y, const double* z, float* rel,
              cudaStream_t s);
// resident CTAs per SM of the brick kernel k_contra of tile shape `shape`
// (FP32; `kernel` is 0)
int max_blocks_per_sm(int shape, int kernel);

// ------------------------------------------------------------ adjoint
// Tile maps besides the forward brick table (output nodes per tile ox x oy
// x oz, adj_shape): 0 stage adjoint x part (8 whole rows, one warp marching
// each), 1 stage adjoint y march, 2 the k marches over 32 x 8 columns (RK
// stage, pseudo-steps, stage adjoint z part, reverse pseudo-step from
// stored coefficients), 3 reverse pseudo-step recomputing its coefficients
// (overlapped 32 x kReinRY tile marching in k).
// The face and velocity adjoints walk the packed nodes with one thread per
// node (instance found by binary search over the node offsets `offs`).
struct AdjShape { int ox, oy, oz; };
constexpr int kReinRY = 12;
// (map 0: ox = 0 means a brick spans whole rows)
__host__ __device__ constexpr AdjShape adj_shape(int map) {
    return map == 0 ? AdjShape{0, 8, 1}
                    : map == 1 ? AdjShape{32, 32, 8} : map == 2 ? AdjShape{32, 8, 32} : AdjShape{30, kReinRY - 2, 32};
}
// Reverse of one bcond_lsm face (face = 0..5: i1, im, j1, jm, k1, km) on the
// adjoint field lam, in place.  The forward values that decide the BigPhi
// switch are evaluated from the pre-BC field P0, given as
//   kind 0 (stage):  interior = out, boundary = c1*phin + c2*in
//   kind 1 (field):  P0 = src (passed as `out`) everywhere
// nface 2 reverses the odd `face` and the opposite face face - 1 of the same
// axis in one launch (valid when every instance has at least 6 nodes along
// that axis: the two faces' nodes and targets are then disjoint)
template <typename T>
void adj_face(const Flat& fl, int face, long long nface_nodes, int nface, BC bc, int kind, const T* phin,
              const T* in, const T* out, double c1, double c2, T* lam, cudaStream_t s);
// Reverse of one RK stage in three passes (x on adjoint map 0 by warp
// shuffles, y and z marches on maps 1 and 2).  lamP0: adjoint of the
// stage's pre-BC field; writes lam_in = c2 lamP0 - c3 (dR/din)^T lamP0
// (+ lamPhin + c1 lamP0 when last, which also clears lamPhin), otherwise
// accumulates lamPhin += c1 lamP0; and lamW_m -= c3 lamP0 D_m.
template <typename T>
void adj_stage(const int* grid, const Inst* inst, const Brick* const* bmap, const int* nb, FieldsT<T> f, const T* in,
               const T* lamP0, T* lam_in, T* lamPhin, T* lamW0, T* lamW1, T* lamW2, double c1, double c2, double c3,
               bool last, cudaStream_t s);
// Reverse of one reinitialisation pseudo-step d' = d - dtau s (G(d) - 1)
// from its input d: lam_out = (dd'/dd)^T lam (adjoint map 3).
template <typename T>
void adj_reinit(int grid, const Inst* inst, const Brick* bmap, int nb, FieldsT<T> f, const T* d, const T* lam,
                T* lam_out, cudaStream_t s);
// Reverse of one recorded pseudo-step from the coefficients reinit_rec
// stored: a 7-point stencil on lam, on the tiles of adjoint map 2 (grid
// from adj_reinit_c_blocks_per_sm)
template <typename T>
void adj_reinit_c(int grid, const Inst* inst, const Brick* bmap2, int nb, const T* cf, long long ld, const T* lam,
                  T* lam_out, cudaStream_t s);
template <typename T>
int adj_reinit_c_blocks_per_sm();
// resident blocks per SM of the kernel of adjoint map `map`
template <typename T>
int adj_blocks_per_sm(int map);
// Mass correction: dst = src + mass[inst].C on every node (dst may alias src)
template <typename T>
void mass_shift(const Flat& fl, const Mass* mass, const T* src, T* dst, cudaStream_t s);
// Reverse of the shift phi' = phi + C(phi) in place on lam (the adjoint of
// phi'): lam -= (sum(lam) / A) (dK/dphi + C d(dK/dC)/dphi), evaluated on
// the step's pre-correction field phi_pre; wfix (N 64-bit words, zero on
// entry and on exit), part (one double per tile of adjoint map 2) and ssum
// (one per instance) are scratch; (list, count) are the interface cells of
// phi_pre as the forward step's volume pass listed them
template <typename T>
void mass_adjoint(const Inst* inst, const Brick* bmap2, int nb2, const Flat& fl, FieldsT<T> f, const T* phi_pre,
                  const Mass* mass, T* lam, unsigned long long* wfix, double* part, double* ssum, const unsigned* list,
                  const unsigned* count, cudaStream_t s);
// lam_u_c += sum_m M[m][c] dt lamW_m  (the W = dt M u chain rule)
template <typename T>
void adj_contra(const Flat& fl, FieldsT<T> f, const T* lamW0, const T* lamW1, const T* lamW2, T* lu0, T* lu1,
                T* lu2, cudaStream_t s);

}  // namespace batch
}  // namespace lsm
