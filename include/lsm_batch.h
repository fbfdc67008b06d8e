/*
 * lsm_batch.h -- batched FP32 level-set transport on one GPU.
 *
 * Many independent instances of uneven sizes (each one rank's single-zone
 * grid: all faces physical, no ghost planes, fine-grid spacing dc=de=dz=1)
 * advance together: one launch per pass covers every instance, the
 * per-step launch sequence is captured once in a CUDA graph, and the tile
 * shape of the stencil kernels is chosen by timing the candidates on the
 * batch itself.  A physical step is the reference's `levelsetmethod`
 * (src/levelsetmethod.F90:1-372) per instance: pre-advection water volume,
 * contravariant velocity, one TVD-RK3 step of WENO3 advection with
 * bcond_lsm after every stage, RNitermax pseudo-steps of `reinitialization`
 * and a final bcond_lsm.
 *
 * Precision: the stencils run in FP32 (precision 0, throughput) or FP64
 * (precision 1, gradient checks); the water volume sums FP64 hexahedron
 * volumes of the bulk water cells and the interface cells' shares (the
 * reference's marching tetrahedra, in the stencil precision on coordinates
 * relative to each cell's first vertex), each rounded to a multiple of
 * 2^-48 and summed as 64-bit integers, so each instance's sum is exact and
 * independent of the summation order (valid below 2^15 units^3).
 *
 * Adjoint: lsm_batch_forward_record runs `nsteps` steps keeping the state
 * every `checkpoint_every` steps (the last segment with all its internals);
 * after seeding dL/dphi^{nsteps} per instance, lsm_batch_backward recomputes
 * every other segment from its checkpoint and runs the hand-written reverse
 * kernels (WENO3 nonlinear weights
 * differentiated, upwind side frozen; Godunov selections and the sign field
 * frozen), giving dL/dphi^0 and dL/dq(2:4) (the velocity is held fixed over
 * the recorded steps).
 *
 * Near the interface the FP32 stencils keep FP64 metric terms: stage nodes
 * whose input |phi| is below 2 eps take their contravariant velocity from
 * the FP64 metrics and velocity passed to set_geometry / set_velocity (kept
 * per node, 15 FP64 arrays) and combine the stage in FP64 over the FP32
 * WENO differences; the adjoint uses the FP32 contravariant velocity there
 * too.  The environment variable LSM_BATCH_BAND64=0 at lsm_batch_create
 * leaves this out (measurements).
 *
 * Mass correction (config.mass_correction = 1; no counterpart in the
 * reference's Sussman branch, whose GlobalMassCorrection, src/levelsetmethod.
 * F90:245-266, feeds the geometric reinitialisation instead): after each
 * step's final bcond_lsm, the FP64 water volume V of the result and its
 * derivative A = dV/dC under a uniform shift phi + C are formed, and phi +=
 * C with C = (target - V) / A (one Newton step towards the instance's
 * target volume; instances without a target are not corrected).  The
 * adjoint differentiates C exactly, including dA/dphi.
 *
 * No counterpart exists in the reference, which advances one subdomain per
 * MPI rank and has no adjoint.
 */
#ifndef LSM_BATCH_H
#define LSM_BATCH_H

#include "lsm_c.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lsm_batch_instance {
    int ni, nj, nk;     /* nodes per axis (>= 4 each) */
    double dt;          /* advection time step (delti_lsm) */
    double dtau;        /* reinitialisation pseudo time step (RNtimestep) */
    double eps;         /* smoothing half-width (epslsm) */
} lsm_batch_instance;

typedef struct lsm_batch_config {
    int RNitermax;      /* reinitialisation pseudo-steps per physical step (0: none) */
    int btype_lsm[6];   /* bcond_lsm face types (0 absorb, 1 extrapolate, 2 advect) */
    double BigPhi;      /* first-order extrapolation cut-off */
    int use_graph;      /* 1: capture the per-step launches in a CUDA graph */
    int autotune;       /* 1: time the candidates on this batch and keep the fastest */
    int shape;          /* when autotune == 0: 0..4 tile shape (pseudo-steps on the brick
                           table), 5 tile shape 0 with the pseudo-steps marching in k */
    int precision;      /* 0: FP32 stencils, 1: FP64 stencils (tile shape 0, no autotune) */
    int adjoint_mode;   /* 0: recorded pseudo-steps store their adjoint coefficients (6 arrays
                           each; the reverse sweep is a stencil), 1: the reverse sweep
                           recomputes them from the stored pseudo-step inputs (1 array each) */
    int mass_correction;  /* 1: FP64 mass correction after every step towards the targets of
                             lsm_batch_set_mass_target (the step's volume pass then measures the
                             step's result instead of its input) */
} lsm_batch_config;

typedef struct lsm_batch* lsm_batch_handle;

/* Allocate the packed device arrays of `ninst` instances on `device`
   (N = total nodes, below 2^32): 21
   stencil-precision arrays of N, the FP64 coordinates and cell volumes (4 N
   doubles), and for FP32 batches the FP64 metrics, velocity and
   contravariant velocity (15 N doubles) and, when they fit, the relative
   vertex coordinates of every cell (24 N floats; a cache: without it the
   volume kernels form the same values per use). */
int lsm_batch_create(lsm_batch_handle* h, int device, void* cuda_stream, int ninst,
                     const lsm_batch_instance* inst, const lsm_batch_config* cfg);
int lsm_batch_destroy(lsm_batch_handle h);

/* Per-instance inputs in the reference's layout (FP64, host or device):
   coordinates x, y, z and metrics csi, eta, zet (1:3, ...); velocity q (1:4, ...)
   of which q(2:4) is read; phi.
   Every array argument of the batch (inputs and outputs) may be pageable
   host memory (copied through a device staging buffer), page-locked host
   memory registered on the batch's device (cudaHostAlloc / cudaHostRegister:
   read and written in place by the conversion kernels, the fastest host
   path), or device memory (used in place on the batch's device, copied from
   another device).  Each call returns once the transfer is complete. */
int lsm_batch_set_geometry(lsm_batch_handle h, int inst, const double* x, const double* y,
                           const double* z, const double* csi, const double* eta, const double* zet);
int lsm_batch_set_velocity(lsm_batch_handle h, int inst, const double* q);
int lsm_batch_set_phi(lsm_batch_handle h, int inst, const double* phi);
/* Read phi of one instance back as FP64 (host or device array). */
int lsm_batch_get_phi(lsm_batch_handle h, int inst, double* phi);
/* The same for every instance in one call: q[k] / phi[k] is instance k's
   array (ninst pointers, none null).  The transfers of all instances are
   queued and waited for once, where a loop over the single-instance calls
   waits for each (a coupled solver that exchanges every instance's
   velocity and phi each step).  No reference counterpart. */
int lsm_batch_set_velocities(lsm_batch_handle h, const double* const* q);
int lsm_batch_get_phis(lsm_batch_handle h, double* const* phi);

/* Advance every instance by `nsteps` physical steps.  `volumes` (nullable,
   host, 4*ninst doubles) receives each instance's pre-advection volumes of
   the last step (K-tetrahedra, second tetrahedra, bulk, total); with the
   mass correction, the volumes of the last step's result before its
   correction. */
int lsm_batch_step(lsm_batch_handle h, int nsteps, double* volumes);

/* Water volumes (K, S, bulk, total; host, 4*ninst doubles) of the current
   phi of every instance. */
int lsm_batch_water_volume(lsm_batch_handle h, double* volumes);
/* Target water volume of one instance for the mass correction (NaN: no
   correction of that instance; the default).  The adjoint treats it as a
   constant.  LSM_ERR_BAD_PARAM when the batch has no mass correction. */
int lsm_batch_set_mass_target(lsm_batch_handle h, int inst, double volume);
/* The last step's mass correction per instance (host, 4*ninst doubles):
   volume before the correction V, slope A = dV/dC, shift C, target. */
int lsm_batch_mass_state(lsm_batch_handle h, double* out);

/* Adjoint.  Run `nsteps` steps from the current phi (which becomes phi^0),
   keeping a checkpoint every `checkpoint_every` steps; the last segment
   runs with every step's internals kept.  lsm_batch_backward reverses the
   last segment from those and each earlier one after recomputing it once
   from its checkpoint (keeping its internals); with nsteps <=
   checkpoint_every nothing is recomputed.  Device memory: N (ceil(nsteps /
   k) + k (5 + m + c RNitermax) + 9) elements of the batch precision, k =
   checkpoint_every, c = 6 (adjoint_mode 0) or 1 (adjoint_mode 1), m = 2
   with the mass correction (each recorded step keeps its pre-correction
   field and that field's interface cells; N 8-byte words of scratch more)
   else 0. */
int lsm_batch_forward_record(lsm_batch_handle h, int nsteps, int checkpoint_every);
/* Seed dL/dphi at the end of the recorded steps for one instance (FP64, host
   or device; instances not seeded get zero). */
int lsm_batch_set_grad_phi(lsm_batch_handle h, int inst, const double* grad);
/* Reverse the recorded steps. */
int lsm_batch_backward(lsm_batch_handle h);
/* dL/dphi^0 of one instance (FP64, host or device, ni*nj*nk). */
int lsm_batch_get_grad_phi0(lsm_batch_handle h, int inst, double* grad);
/* dL/dq of one instance in the layout of q (4, ni, nj, nk); q(1) gets zero. */
int lsm_batch_get_grad_velocity(lsm_batch_handle h, int inst, double* grad_q);

/* Tile shape in use (index 0..5 as lsm_batch_config.shape, and the brick
   table's TX, TY, TZ). */
int lsm_batch_shape(lsm_batch_handle h, int* index, int* tx, int* ty, int* tz);
/* RK stage kernel in use after the first step: 1 plane tiles staged by TMA
   copies (FP32 batches of one instance with ni a multiple of 4, when the
   autotuner finds it faster; the environment variable LSM_BATCH_STAGE=tma
   or =smem forces the choice), 0 staged by the threads, -1 no handle. */
int lsm_batch_stage_kernel(lsm_batch_handle h);
/* Total nodes of the batch and kernels launched per physical step. */
long long lsm_batch_nodes(lsm_batch_handle h);
int lsm_batch_launches_per_step(lsm_batch_handle h);
/* Last detailed error text of the batch handle. */
const char* lsm_batch_last_error(lsm_batch_handle h);

#ifdef __cplusplus
}
#endif
#endif /* LSM_BATCH_H */
