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
 * Precision: the stencils run in FP32; the water volume is FP64 (FP32 phi,
 * FP64 coordinates, the reference's marching tetrahedra) with fixed-order
 * sums per instance.  No counterpart exists in the reference, which
 * advances one subdomain per MPI rank.
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
    int autotune;       /* 1: time every tile shape on this batch and keep the fastest */
    int shape;          /* tile shape index when autotune == 0 (0..4) */
} lsm_batch_config;

typedef struct lsm_batch* lsm_batch_handle;

/* Allocate the packed device arrays of `ninst` instances on `device`. */
int lsm_batch_create(lsm_batch_handle* h, int device, void* cuda_stream, int ninst,
                     const lsm_batch_instance* inst, const lsm_batch_config* cfg);
int lsm_batch_destroy(lsm_batch_handle h);

/* Per-instance inputs in the reference's layout (FP64, host or device):
   coordinates x, y, z and metrics csi, eta, zet (1:3, ...); velocity q (1:4, ...)
   of which q(2:4) is read; phi. */
int lsm_batch_set_geometry(lsm_batch_handle h, int inst, const double* x, const double* y,
                           const double* z, const double* csi, const double* eta, const double* zet);
int lsm_batch_set_velocity(lsm_batch_handle h, int inst, const double* q);
int lsm_batch_set_phi(lsm_batch_handle h, int inst, const double* phi);
/* Read phi of one instance back as FP64 (host or device array). */
int lsm_batch_get_phi(lsm_batch_handle h, int inst, double* phi);

/* Advance every instance by `nsteps` physical steps.  `volumes` (nullable,
   host, 4*ninst doubles) receives each instance's pre-advection volumes of
   the last step (K-tetrahedra, second tetrahedra, bulk, total). */
int lsm_batch_step(lsm_batch_handle h, int nsteps, double* volumes);

/* Tile shape in use (index, and its TX, TY, TZ). */
int lsm_batch_shape(lsm_batch_handle h, int* index, int* tx, int* ty, int* tz);
/* Total nodes of the batch and kernels launched per physical step. */
long long lsm_batch_nodes(lsm_batch_handle h);
int lsm_batch_launches_per_step(lsm_batch_handle h);
/* Last detailed error text of the batch handle. */
const char* lsm_batch_last_error(lsm_batch_handle h);

#ifdef __cplusplus
}
#endif
#endif /* LSM_BATCH_H */
