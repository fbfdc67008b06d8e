/*
 * lsm_c.h -- C-ABI of the GB300-native level-set transport step.
 *
 * This is the drop-in boundary for the level-set layer of the curvilinear
 * free-surface solver NS-LSM-Single-Phase.  Every entry point here replaces one
 * Fortran subroutine of that layer (cited per declaration, paths relative to
 * the reference project).  The Fortran routines are internal procedures of
 * `levelsetmethod` that reach their data by host association and through the
 * modules `global_lsm`, `global_mpi` and `global_app`; here those hidden inputs
 * become two explicit structs: `lsm_grid` (bounds, ghost planes, computational
 * spacing, which subdomain faces are physical boundaries) and `lsm_params`
 * (the `global_lsm` switches read from `ind3dmg_LSM.dat`).
 *
 * Conventions
 *  - Arrays are FP64 (REAL(8); `rdf = selected_real_kind(p=7)`,
 *    src/precision.F90:11), Fortran column-major with explicit bounds
 *    (il:iu, jl:ju, kl:ku): element (i,j,k) sits at offset
 *    (i-il) + ni*((j-jl) + nj*(k-kl)), ni = iu-il+1, nj = ju-jl+1.
 *    Vector fields are (1:3, il:iu, ...) with the component fastest; q is
 *    (1:4, ...), of which only q(2:4) (the Cartesian velocity) is read.
 *  - Integer masks and lists are 32-bit `int` (Fortran default INTEGER).
 *  - Every array of one call lives either in host memory or in device memory
 *    of the handle's GPU (detected per call).  Host arrays are staged through
 *    the handle's device pool; device arrays are used in place on the
 *    handle's stream and the call returns once the stream has finished.
 *  - Every entry point returns an `int` status (LSM_OK = 0).  Nothing aborts;
 *    the reference's `stop` on a negative tetrahedron water volume
 *    (src/TetrahedronMethods.F90:944-952) becomes LSM_ERR_NEGATIVE_VOLUME.
 *  - Threading: one handle per host thread / stream.  A handle is
 *    thread-compatible, not thread-safe.  Passing a NULL handle uses a
 *    lazily created default handle on the current device (legacy stream).
 *  - One rank: the reference's MPI halo exchange (src/rhs_exchng3_3d.F90) and
 *    volume allreduce (src/levelsetmethod.F90:193) have no work to do on one
 *    GPU.  Subdomains with ghost planes are accepted (igp/jgp/kgp and
 *    `physical_face`); their ghost values are the caller's, and the callback
 *    set with lsm_set_exchange_callback() is invoked wherever the reference
 *    calls rhs_exchng3_3d.
 */
#ifndef LSM_C_H
#define LSM_C_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define LSM_OK                   0
#define LSM_ERR_NULL             1  /* a required pointer is NULL */
#define LSM_ERR_BAD_SHAPE        2  /* bounds/ghost planes inconsistent or a dimension too small */
#define LSM_ERR_BAD_PARAM        3  /* a parameter is outside what the reference accepts */
#define LSM_ERR_UNSUPPORTED      4  /* a switch selects a branch outside the level-set transport path */
#define LSM_ERR_NONFINITE        5  /* non-finite value found where the step would propagate it */
#define LSM_ERR_NEGATIVE_VOLUME  6  /* a tetrahedron water volume < -epsilon (reference stops) */
#define LSM_ERR_MIXED_MEMORY     7  /* arrays of one call are split between host and device */
#define LSM_ERR_CAPACITY         8  /* output buffer too small (required size is still returned) */
#define LSM_ERR_CUDA             9  /* a CUDA runtime call failed (see lsm_last_error) */
#define LSM_ERR_NO_DEVICE       10  /* no usable CUDA device */

/* ---- grid: bounds of every array + subdomain description ----------------- */
typedef struct lsm_grid {
    int il, iu, jl, ju, kl, ku;  /* Fortran bounds of all arrays (inclusive) */
    int igp, jgp, kgp;           /* ghost planes per side (0 on one rank) */
    double dc, de, dz;           /* 1/dxi, 1/deta, 1/dzeta (1 on the fine grid, src/init.F90:1170-1174) */
    /* 1 where the face is a physical boundary (my* == MPI_PROC_NULL),
       order: i1 (myback), im (myfront), j1 (myleft), jm (myright), k1 (mydown), km (myup) */
    int physical_face[6];
} lsm_grid;

/* ---- parameters: the global_lsm switches (src/global_lsm.F90:8-56) ------- */
typedef struct lsm_params {
    double epslsm;                   /* smoothing half-width of sign/delta/heaviside */
    int    numiter_lsm;              /* RK3 sub-iterations per physical step */
    double delti_lsm;                /* advection time step (delti/numiter_lsm) */
    int    RNitermax;                /* reinitialisation pseudo-steps */
    double RNtimestep;               /* reinitialisation pseudo time step */
    int    RNfreq;                   /* reinitialise when mod(ntime, RNfreq) == 0 */
    int    btype_lsm[6];             /* per face: 0 absorb, 1 extrapolate, 2 advect */
    int    bc_extrapolation_order;   /* read but unused by bcond_lsm's live branches */
    int    isnarrow;                 /* 0: narrow band is every node */
    double narrowcoef;               /* band = |phi_n| < narrowcoef*epslsm + 1.0E-5 */
    int    orderAD;                  /* 0: first-order UPWIND, 1: WENO3 */
    int    sussman_correction_method;/* 0 only (method 1 needs testfilter, outside the path) */
    int    call_levelsetmethod;      /* advect */
    int    call_reinitialisation;    /* reinitialise */
    int    hybrid_reinitialisation;  /* 1: geometric reinitialisation (src/levelsetmethod.F90:300-309) and
                                        advection on the AdvectionNodes band only (:218-219) */
    int    TotalVolumeComputation;   /* informational (volume is always computed) */
    int    GlobalMassCorrection;     /* 1: post-advection volume pass (lsm_convergence_volume) */
    double BigPhi;                   /* |phi| cut-off for BC order and ghost-fluid list */
    double epsReinitialisation;      /* convergence threshold of reinitialisation_test2 */
    int    M_Sphi0;                  /* sign model in calc_sign_ini: 1 Kang piecewise, 0 phi/sqrt(phi^2+(|grad|eps)^2) */
    int    reinit_scheme;            /* 0: `reinitialization` (Sussman-Fatemi, forward Euler + lambda);
                                        1: `reinitialisation_test2` (the reference's live call,
                                           src/levelsetmethod.F90:313: ENO2 gradients, TVD-RK3 in
                                           pseudo time, convergence mask and early exit) */
    int    write_global_volume;      /* 1: append pre-advection volume to GlobalVolume.txt */
    int    OrderReinitialisationBoundaries; /* 1, 2 or 3: one-sided derivative order on physical faces
                                               in calc_NormGrad_d (BiasedDerivative) */
    int    ENOBCReinitialisation;    /* 1: with order 2, ENO2Boundary instead of the 2nd-order formula */
    double ConvergenceToleranceGeomReini; /* volume tolerance of the geometric reinitialisation's
                                             global (Newton) and per-tetrahedron (secant, /1000)
                                             corrections; the deck's 1.0E-09 */
} lsm_params;

/* Fill a params struct with the values of the reference's example deck
   (control.dat): WENO3, btype 1 everywhere, BigPhi 5, M_Sphi0 1,
   ConvergenceToleranceGeomReini 1e-9, ...  One exception: the deck sets
   hybrid_reinitialisation = .true. (control.dat:200); the default here is
   0 (the Sussman branch, which runs on decomposed subdomains too), and
   read_ind3dmg_lsm / a caller copying global_lsm sets it from the deck. */
void lsm_params_default(lsm_params* p);

/* ---- handle -------------------------------------------------------------- */
typedef struct lsm_context* lsm_handle;

int lsm_create(lsm_handle* h, int device, void* cuda_stream);
int lsm_destroy(lsm_handle h);
int lsm_set_stream(lsm_handle h, void* cuda_stream);
/* Called wherever the reference calls rhs_exchng3_3d(var) on a field of the
   subdomain; `field` is a device pointer with the grid's bounds. */
typedef int (*lsm_exchange_fn)(void* user, double* field, const lsm_grid* g);
int lsm_set_exchange_callback(lsm_handle h, lsm_exchange_fn fn, void* user);
const char* lsm_status_string(int status);
/* Last detailed error text of the handle (or of the default handle). */
const char* lsm_last_error(lsm_handle h);
/* Number of kernels this library has launched since the handle was made. */
long long lsm_kernel_launch_count(lsm_handle h);

/* Per-kernel timing with CUDA events recorded on the launching stream
   around every launch while enabled (process-wide; off by default).  No
   reference counterpart: the reference only times whole steps
   (src/main.F90:72-82).  lsm_profile_entry synchronises on the recorded
   events and reports, for the i-th kernel, its name, launches and total ms. */
int lsm_profile_enable(int on);
int lsm_profile_reset(void);
int lsm_profile_count(void);
int lsm_profile_entry(int i, char* name, int name_len, long long* launches, double* total_ms);

/* ---- the level-set step (drop-in for the whole layer) --------------------- */
/* Replaces `levelsetmethod` (src/levelsetmethod.F90:1-372), called from
   src/mg_driver.F90:567-580.  Sequence: pre-advection water volume (and the
   AdvectionNodes band), contravariant velocity, numiter_lsm x TVD-RK3,
   optional post-advection volume, reinitialisation when
   mod(iteraciontiempo, RNfreq) == 0, bcond_lsm.  phi is advected starting
   from phi_n (ad_RKTVD3 initialises phi^{n+1} = phi^n).  `volumes_out`
   (nullable, host, 4 doubles) receives the pre-advection K-tetrahedra,
   second-tetrahedra, bulk-cell and total volumes.  With
   GlobalMassCorrection the advected phi's volume is computed too (see
   lsm_convergence_volume).  With call_reinitialisation and
   hybrid_reinitialisation (the deck's choice, control.dat) only the
   AdvectionNodes band is advected and the reinitialisation is
   lsm_geometric_reinitialisation (one subdomain without ghost planes);
   otherwise every node is advected and reinit_scheme picks the Sussman
   routine. */
int lsm_levelsetmethod(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                       const double* q, const double* csi, const double* eta,
                       const double* zet, const double* aj,
                       double* phi, const double* phi_n,
                       const double* x, const double* y, const double* z,
                       int iteraciontiempo, double* volumes_out);

/* ---- the inner routines ---------------------------------------------------- */
/* rhs_contra_j (src/rhs_contra_j.F90:2-53): ucn_j(m) = (1/aj) (metric_m . u).
   Nodes outside the reference's loop range are set to 0 (levelsetmethod
   zeroes ucn_j before the call, src/levelsetmethod.F90:225). */
int lsm_rhs_contra_j(lsm_handle h, const lsm_grid* g, const double* q,
                     const double* csi, const double* eta, const double* zet,
                     const double* aj, double* ucn_j);

/* calc_RH_AD_WENO3 (src/calc_RH_AD_WENO3.F90:1-407) with
   GetWENO3Reconstruction (src/AdvectionMethods.F90:195-245).  rh is zeroed
   first, as ad_RKTVD3 does (src/ad_RKTVD3.F90:55).  advection_nodes may be
   NULL (every node advected). */
int lsm_calc_rh_ad_weno3(lsm_handle h, const lsm_grid* g, const double* phi,
                         const double* ucn_j, const int* advection_nodes, double* rh);

/* calc_RH_AD, first-order upwind (src/calc_RH_AD.F90:1-273, orderAD == 0). */
int lsm_calc_rh_ad(lsm_handle h, const lsm_grid* g, const double* phi,
                   const double* ucn_j, const int* advection_nodes, double* rh);

/* ad_RKTVD3 (src/ad_RKTVD3.F90:1-88): phi_n1 = TVD-RK3 step of phi_n with
   time step p->delti_lsm; bcond_lsm + exchange after every stage. */
int lsm_ad_rktvd3(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                  double* phi_n1, const double* phi_n, const int* advection_nodes,
                  const double* ucn_j, const double* aj);

/* bcond_lsm (src/bcond_lsm.F90:2-287), faces in the order i1, im, j1, jm, k1, km. */
int lsm_bcond_lsm(lsm_handle h, const lsm_grid* g, const lsm_params* p, double* phi);

/* calc_sign_ini (src/calc_sign_ini.F90:1-286): smoothed sign s(phi0) and the
   Godunov |grad phi0|.  M_Sphi0: 1 Kang piecewise sign, 0 continuous sign. */
int lsm_calc_sign_ini(lsm_handle h, const lsm_grid* g, const double* phi0,
                      const double* csi, const double* eta, const double* zet,
                      double epslsm, int M_Sphi0, double* sign, double* normgrad);

/* calc_RH_RN (src/calc_RH_RN.F90:1-244): rh = s (|grad d|_Godunov - 1). */
int lsm_calc_rh_rn(lsm_handle h, const lsm_grid* g, const double* d, const double* sign,
                   const double* csi, const double* eta, const double* zet, double* rh);

/* calc_lambda_RN, method 0 (src/calc_lambda_RN.F90:42-63). */
int lsm_calc_lambda_rn(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                       const double* phi0, const double* normgrad0, const double* d,
                       double time_step, double* lambda);

/* reinitialization (src/reinitialization.F90:1-106): RNitermax forward-Euler
   pseudo-steps of d_t + s(phi0)(|grad d| - 1) = 0 with the Sussman-Fatemi
   lambda correction; phi_out = d after the last step (no bcond_lsm). */
int lsm_reinitialization(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                         const double* phi0, const double* csi, const double* eta,
                         const double* zet, double* phi_out);

/* calc_NormGrad_d (src/calc_NormGrad_d.F90:1-2448): |grad phi_rn| by ENO2 in
   every direction (stencil choice by the sign of phizero), one-sided
   BiasedDerivative of order OrderReinitialisationBoundaries (ENO2Boundary
   when ENOBCReinitialisation and order 2) along a direction whose face is
   physical at the node; 0 on ghost nodes.  Kept from the reference: the two
   i-face blocks choose their ENO2 stencils with phizero at the last
   interior node, because they never assign phi0. */
int lsm_calc_normgrad_d(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                        const double* phi_rn, const double* phizero, const double* csi,
                        const double* eta, const double* zet, double* normgrad);

/* reinitialisation_test2 (src/reinitialisation_test2.F90:1-221, non-hybrid):
   the reinitialisation the reference calls (src/levelsetmethod.F90:313).
   Up to RNitermax pseudo-time iterations of TVD-RK3 with step RNtimestep on
   the nodes whose |grad d| at the start of the iteration exceeds
   1 + epsReinitialisation, with the GetLambdaMassCorrection term; stops
   when max and min of |grad d| are both within epsReinitialisation of 1.
   No halo exchange inside, as in the reference.  *iterations (nullable)
   receives the iterations run.  phi_out = d (no bcond_lsm). */
int lsm_reinitialisation_test2(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                               const double* phizero, const double* csi, const double* eta,
                               const double* zet, double* phi_out, int* iterations);

/* narrowband (src/narrowband.F90:2-19): nband = |phi_n| < narrowcoef*epslsm + 1.0E-5
   on every node (ghosts included); every node 1 when isnarrow == 0. */
int lsm_narrowband(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                   const double* phi_n, int* nband);

/* TotalWaterVolume (src/TotalWaterVolume.F90:1-297): water (phi > 0) volume of
   the cells, split into K-tetrahedra, second-tetrahedra and bulk cells
   (volumes[0..2], host); volumes[3] = their sum (levelsetmethod.F90:187-189).
   advection_nodes (nullable) receives the AdvectionNodes band. */
int lsm_total_water_volume(lsm_handle h, const lsm_grid* g, const double* phi,
                           const double* x, const double* y, const double* z,
                           double* volumes, int* advection_nodes);

/* Allocation-free variant of lsm_total_water_volume.  It has no counterpart
   in the reference.  It is for callers that cannot call cudaMalloc -- code
   running under another framework's memory pool or allocator hooks that
   forbid raw device allocations, or a real-time loop where an allocation's
   latency or failure is not allowed -- and so cannot create a handle (a
   handle allocates its pool).  phi, x, y, z must be device arrays of the
   current GPU; `volumes` (4 doubles, host or device) receives the same
   numbers as lsm_total_water_volume.  The call allocates nothing: its
   scratch is one file-scope device array of fixed size (about 6 MiB, held by
   every GPU that loads this library until the process exits), sized for at
   most LSM_NOALLOC_MAX_CELLS cells; larger grids return LSM_ERR_CAPACITY.
   The first call on each device looks the array's address up and keeps it
   for the life of the process, so make that first call before any stream
   capture, and do not call this entry point again on a device after a
   cudaDeviceReset of it (the array may then sit at another address).
   Every call shares the one array:
   calls that overlap on the GPU (other streams or threads) race and must be
   serialised by the caller.  `volumes` on another GPU returns
   LSM_ERR_MIXED_MEMORY.  The call returns after `stream` has drained. */
#define LSM_NOALLOC_MAX_CELLS (64LL * 1024 * 1024)
int lsm_total_water_volume_noalloc(const lsm_grid* g, const double* phi, const double* x,
                                   const double* y, const double* z, double* volumes,
                                   void* cuda_stream);

/* Per-cell water volume (diagnostic restatement of the same loop): cellvol
   has the grid's node shape; entry (i,j,k) holds the volume of cell
   (i..i+1, j..j+1, k..k+1), 0 where the loop does not visit. */
int lsm_cell_water_volumes(lsm_handle h, const lsm_grid* g, const double* phi,
                           const double* x, const double* y, const double* z,
                           double* cellvol);

/* get_gfm_list (src/get_gfm_list.F90:1-143): air nodes (phi <= epsilon) with
   |phi| <= BigPhi and a water neighbour in their 3x3x3 box, ordered k, j, i.
   *count receives the number of nodes.  `list` (nullable) is Fortran
   (ld, 3): list[c + ld*0] = i, list[c + ld*1] = j, list[c + ld*2] = k.
   If ld < *count nothing is written and LSM_ERR_CAPACITY is returned. */
int lsm_get_gfm_list(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                     const double* phi, int* count, int* list, int ld);

/* mg_metrics on one rank's fine grid (src/mg_metrics.F90:44-264): central
   differences of x, y, z inside, one-sided on the faces, aj = 1/det and
   csi/eta/zet = aj * cofactors.  Input preparation (the reference computes
   the metrics once in `init`), offered so that callers and tests feed the
   level-set step the metrics the reference would; grids without ghost
   planes only. */
int lsm_mg_metrics(lsm_handle h, const lsm_grid* g, const double* x, const double* y,
                   const double* z, double* csi, double* eta, double* zet, double* aj);

/* WriteTotalWaterVolume (src/WriteTotalWaterVolume.F90:1-29): append one
   list-directed REAL(8) line to `path` (NULL: "GlobalVolume.txt"). */
int lsm_write_total_water_volume(double volume, const char* path);
/* geometric_reinitialisation (src/geometric_reinitialisation.F90:1-94), the
   hybrid path's reinitialisation, TriangulationCase 1, one subdomain without
   ghost planes (every face physical):
    1. GetTetrahedraList (src/GetTetrahedraList.F90:1-450): the phase-change
       ("K") tetrahedra of the six-tetrahedra split of every cell
       (CellPnodeTetrahedronIdentification, src/TetrahedronMethods.F90:2124-2361)
       and their vertices, the pnodes, numbered 1.. in k, j, i order;
    2. GetIsosurfaceAndDistances (src/GetIsosurfaceAndDistances.F90:1-335):
       the marching-tetrahedra isosurface of every K tetrahedron and, per
       pnode, the signed distance to the triangles of the K tetrahedra of the
       pnodes within 4 nodes; non-pnodes within 4 nodes of a pnode are tagged -1;
    3. with GlobalMassCorrection: PiecewiseConstantFunction (secant method per
       tetrahedron, src/PiecewiseConstantFunction.F90:1-102,
       src/TetrahedronMethods.F90:2439-2588), OrthogonalProjection
       (src/OrthogonalProjection.F90:1-49) and the global constant C of
       NewtonRaphson (src/NewtonRaphsonSolver.F90) that makes the K
       tetrahedra hold `total_water_volume`;
    4. NeighboursPhiCorrection (src/NeighboursPhiCorrection.F90:1-346):
       phicorrected = distance + C xi on the pnodes, and on the -1 nodes the
       smaller of |phicorrected| and their distance to those triangles, sign
       kept.
   phicorrected is in/out: nodes that are neither pnodes nor tagged keep the
   caller's value (levelsetmethod sets +-9.9 off the interface, :303-304).
   interface_nodes_id (in/out, int) is set to 0 first, as levelsetmethod does
   (:293), and returns the pnode ids, -1 and 0.  info (nullable, host)
   receives the list sizes and the Newton result. */
typedef struct lsm_geom_info {
    int    nnodes;             /* pnodes */
    int    ntetrahedra;        /* K tetrahedra */
    int    nsecond;            /* nodes tagged -1 */
    int    newton_iterations;  /* `its` after newt (0 without GlobalMassCorrection) */
    int    newton_converged;   /* 1 when NewtonRaphson kept its C */
    double C;                  /* CCorrected (0 without GlobalMassCorrection) */
} lsm_geom_info;
int lsm_geometric_reinitialisation(lsm_handle h, const lsm_grid* g, const lsm_params* p,
                                   const double* phizero, const double* x, const double* y,
                                   const double* z, double total_water_volume,
                                   double* phicorrected, int* interface_nodes_id,
                                   lsm_geom_info* info);

/* ConvergenceVolume of the last lsm_levelsetmethod call on `h`
   (src/levelsetmethod.F90:245-264): the pre-advection total volume minus the
   K- and second-tetrahedra volumes of the advected phi when
   GlobalMassCorrection is set, else the pre-advection total.  The reference
   hands it to the geometric (hybrid) reinitialisation. */
int lsm_convergence_volume(lsm_handle h, double* volume);

#ifdef __cplusplus
}
#endif
#endif /* LSM_C_H */
