// lsm_kernels.h -- host launchers of the level-set kernels (internal to the
// library; the public interface is include/lsm_c.h).
#pragma once

#include <cuda_runtime.h>

#include "lsm_common.cuh"

namespace lsm {

// ---- FP64 reference-arithmetic kernels (lsm_fp64.cu, built with --fmad=false)
void launch_contra(const DevGrid& g, const double* q, const double* csi, const double* eta,
                   const double* zet, const double* aj, double* ucn, cudaStream_t s);
void launch_rh_ad(const DevGrid& g, int orderAD, const double* phi, const double* ucn,
                  const int* mask, double* rh, cudaStream_t s);
void launch_rk_stage(const DevGrid& g, int orderAD, const double* phin, const double* phi1,
                     const double* ucn, const double* aj, const int* mask, double c1, double c2,
                     double c3, double dt, double* out, cudaStream_t s);
void launch_bc_rk(const DevGrid& g, const DevBC& bc, int orderAD, const double* phin,
                  const double* phi1, const double* ucn, const double* aj, const int* mask,
                  double c1, double c2, double c3, double dt, double* dst, cudaStream_t s);
void launch_bc_full(const DevGrid& g, const DevBC& bc, const double* src, double* dst,
                    unsigned* errflag, cudaStream_t s);
void launch_sign_ini(const DevGrid& g, const double* phi0, const double* csi, const double* eta,
                     const double* zet, double eps, int M_Sphi0, double* sgn, double* ng,
                     double* delta, cudaStream_t s);
void launch_rh_rn(const DevGrid& g, const double* d, const double* sgn, const double* csi,
                  const double* eta, const double* zet, double* rh, cudaStream_t s);
void launch_lambda_rn(const DevGrid& g, double eps, const double* phi0, const double* ng,
                      const double* d, double dt, double* lam, cudaStream_t s);
void launch_reinit_step(const DevGrid& g, double dt, const double* din, const double* sgn,
                        const double* ng, const double* delta, const double* phi0,
                        const double* csi, const double* eta, const double* zet, double* dout,
                        cudaStream_t s);
void launch_narrowband(const DevGrid& g, double thr, int isnarrow, const double* phin, int* nb,
                       cudaStream_t s);
void launch_metrics(const DevGrid& g, const double* x, const double* y, const double* z,
                    double* csi, double* eta, double* zet, double* aj, cudaStream_t s);
void launch_copy(const double* src, double* dst, long long n, cudaStream_t s);

// reinitialisation_test2 and calc_NormGrad_d (lsm_sussman.cu)
void launch_sign_phi0(long long n, const double* phi0, double eps, double* sg, cudaStream_t s);
void launch_normgrad_d(const DevGrid& g, int order, int enobc, const double* phi, const double* phizero,
                       long long stale, const double* csi, const double* eta, const double* zet, double* out,
                       cudaStream_t s);
void launch_sussman_rk(const DevGrid& g, const double* dn, double* dn1, const double* ng, const double* ngc,
                       const double* sg, double eps, double epsr, double dt, double c1, double c2, double c3,
                       cudaStream_t s);
int minmax_partials(long long n);
void launch_minmax(long long n, const double* a, double* part, double* res, cudaStream_t s);

// ---- water volume, band and ghost-fluid list (lsm_volume.cu, --fmad=false)
// Number of per-block partial slots the volume kernel needs for this grid.
int volume_partial_blocks(const DevGrid& g);
// partials: volume_partial_blocks(g)*3 doubles; result: 4 doubles (VK, V2, VB, total)
void launch_volume(const DevGrid& g, const double* phi, const double* x, const double* y,
                   const double* z, double* partials, double* result, unsigned char* pcflag,
                   double* cellvol, unsigned* errflag, cudaStream_t s);
void launch_adv_nodes(const DevGrid& g, const unsigned char* pcflag, int* adv, cudaStream_t s);
// scratch: gfm_scratch_ints(g) ints; count_out: 1 int (device)
long long gfm_scratch_ints(const DevGrid& g);
void launch_gfm_list(const DevGrid& g, double BigPhi, const double* phi, int* scratch,
                     int* count_out, int* list, int ld, int il, int jl, int kl, cudaStream_t s);

// launch bookkeeping: every launcher holds a ProfScope across its launch,
// which counts the launch and, while profiling is on, brackets it with a
// CUDA event pair on the launching stream.
extern unsigned long long g_launches;
class ProfScope {
public:
    ProfScope(const char* name, cudaStream_t s);
    ~ProfScope();
    ProfScope(const ProfScope&) = delete;
    ProfScope& operator=(const ProfScope&) = delete;
private:
    const char* name_;
    cudaStream_t s_;
    void* a_ = nullptr;
    void* b_ = nullptr;
    bool active_ = false;
};

}  // namespace lsm
