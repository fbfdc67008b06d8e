// lsm_capi.cu -- the C-ABI of include/lsm_c.h: handles, the device pool,
// host<->device staging and the orchestration of the level-set step.
//
// Every entry point validates the grid the way the reference's loops assume
// it (at least 4 non-ghost nodes per axis, two ghost planes on every
// non-physical face), resolves whether the caller's arrays live on the host
// or on the handle's GPU, stages host arrays through pooled device buffers,
// launches the kernels on the handle's stream and returns after the stream
// has drained, with device-side error flags folded into the status.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "lsm_c.h"
#include "lsm_common.cuh"
#include "lsm_geometric.h"
#include "lsm_kernels.h"

struct lsm_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    lsm_exchange_fn xfn = nullptr;
    void* xuser = nullptr;
    std::string last_error;
    unsigned long long launches0 = 0;
    struct Buf { void* p = nullptr; size_t bytes = 0; };
    std::map<std::string, Buf> pool;
    unsigned* d_err = nullptr;
    double* d_result = nullptr;
    int* d_count = nullptr;
    double conv_volume = 0.0;   // ConvergenceVolume of the last lsm_levelsetmethod
};

namespace {

using lsm::DevGrid;

lsm_context* g_default[64] = {nullptr};
std::mutex g_default_mu;
thread_local std::string t_err;

int set_err(lsm_context* c, int st, const std::string& msg) {
    if (c) c->last_error = msg;
    t_err = msg;
    return st;
}

int cuda_fail(lsm_context* c, cudaError_t e, const char* where) {
    return set_err(c, LSM_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define LSM_CU(c, call)                                              \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return cuda_fail((c), e_, #call);     \
    } while (0)

int make_context(lsm_context** out, int device, cudaStream_t stream) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return set_err(nullptr, LSM_ERR_NO_DEVICE, "no CUDA device");
    }
    if (device < 0 || device >= ndev) return set_err(nullptr, LSM_ERR_BAD_PARAM, "device index out of range");
    auto* c = new lsm_context();
    c->device = device;
    c->stream = stream;
    c->launches0 = lsm::g_launches;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    cudaError_t e = cudaMalloc(&c->d_err, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_result, 8 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_count, 4 * sizeof(int));
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(nullptr, e, "cudaMalloc(handle)");
    }
    *out = c;
    return LSM_OK;
}

int resolve(lsm_handle h, lsm_context** out) {
    if (h) { *out = h; return LSM_OK; }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, LSM_ERR_NO_DEVICE, "no CUDA device");
    }
    if (dev < 0 || dev >= 64) return set_err(nullptr, LSM_ERR_NO_DEVICE, "device index too large");
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (!g_default[dev]) {
        int st = make_context(&g_default[dev], dev, nullptr);
        if (st) return st;
    }
    *out = g_default[dev];
    return LSM_OK;
}

// RAII: make the handle's device current for the duration of a call.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

void* pool_get(lsm_context* c, const std::string& name, size_t bytes, cudaError_t* e) {
    auto& b = c->pool[name];
    if (b.bytes >= bytes && b.p) { *e = cudaSuccess; return b.p; }
    if (b.p) {
        cudaStreamSynchronize(c->stream);
        cudaFree(b.p);
        b.p = nullptr; b.bytes = 0;
    }
    *e = cudaMalloc(&b.p, bytes < 256 ? 256 : bytes);
    if (*e != cudaSuccess) { b.p = nullptr; return nullptr; }
    b.bytes = bytes < 256 ? 256 : bytes;
    return b.p;
}

int check_grid(lsm_context* c, const lsm_grid* g, DevGrid* dg) {
    if (!g) return set_err(c, LSM_ERR_NULL, "grid is NULL");
    if (g->igp < 0 || g->jgp < 0 || g->kgp < 0) return set_err(c, LSM_ERR_BAD_SHAPE, "negative ghost planes");
    const int ni = g->iu - g->il + 1, nj = g->ju - g->jl + 1, nk = g->ku - g->kl + 1;
    if (ni - 2 * g->igp < 4 || nj - 2 * g->jgp < 4 || nk - 2 * g->kgp < 4)
        return set_err(c, LSM_ERR_BAD_SHAPE, "fewer than 4 non-ghost nodes along an axis");
    const int gp[3] = {g->igp, g->jgp, g->kgp};
    for (int f = 0; f < 3; ++f)
        if ((!g->physical_face[2 * f] || !g->physical_face[2 * f + 1]) && gp[f] < 2)
            return set_err(c, LSM_ERR_BAD_SHAPE, "a non-physical face needs two ghost planes");
    if (!(g->dc > 0.0) || !(g->de > 0.0) || !(g->dz > 0.0))
        return set_err(c, LSM_ERR_BAD_PARAM, "dc, de, dz must be positive");
    if ((double)ni * nj * nk > 4.0e9) return set_err(c, LSM_ERR_BAD_SHAPE, "grid too large");
    dg->ni = ni; dg->nj = nj; dg->nk = nk;
    dg->sj = ni; dg->sk = (long long)ni * nj;
    dg->ia = g->igp; dg->ib = ni - 1 - g->igp;
    dg->ja = g->jgp; dg->jb = nj - 1 - g->jgp;
    dg->ka = g->kgp; dg->kb = nk - 1 - g->kgp;
    dg->pb = g->physical_face[0] != 0; dg->pf = g->physical_face[1] != 0;
    dg->pl = g->physical_face[2] != 0; dg->pr = g->physical_face[3] != 0;
    dg->pd = g->physical_face[4] != 0; dg->pu = g->physical_face[5] != 0;
    dg->dc = g->dc; dg->de = g->de; dg->dz = g->dz;
    return LSM_OK;
}

int check_params(lsm_context* c, const lsm_params* p) {
    if (!p) return set_err(c, LSM_ERR_NULL, "params is NULL");
    if (p->orderAD != 0 && p->orderAD != 1) return set_err(c, LSM_ERR_BAD_PARAM, "orderAD must be 0 or 1");
    for (int f = 0; f < 6; ++f)
        if (p->btype_lsm[f] < 0 || p->btype_lsm[f] > 2) return set_err(c, LSM_ERR_BAD_PARAM, "btype_lsm not in 0..2");
    if (p->numiter_lsm < 0 || p->RNitermax < 0) return set_err(c, LSM_ERR_BAD_PARAM, "negative iteration count");
    return LSM_OK;
}

lsm::DevBC make_bc(const lsm_params* p) {
    lsm::DevBC bc;
    for (int f = 0; f < 6; ++f) bc.type[f] = p->btype_lsm[f];
    bc.BigPhi = p->BigPhi;
    return bc;
}

// Host/device staging of the arrays of one call.
class Staging {
public:
    enum Dir { IN, OUT, INOUT };
    Staging(lsm_context* c) : c_(c) {}
    void add(const void* p, size_t bytes, Dir d, void** dev) { args_.push_back({p, bytes, d, dev}); }
    int resolve() {
        int nhost = 0, ndev = 0;
        for (auto& a : args_) {
            if (!a.p) { *a.dev = nullptr; continue; }
            cudaPointerAttributes at;
            cudaError_t e = cudaPointerGetAttributes(&at, a.p);
            if (e != cudaSuccess) { cudaGetLastError(); at.type = cudaMemoryTypeUnregistered; }
            const bool on_dev = at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
            if (on_dev && at.device != c_->device)
                return set_err(c_, LSM_ERR_MIXED_MEMORY, "array lives on another GPU than the handle's");
            a.host = !on_dev;
            nhost += a.host; ndev += !a.host;
        }
        if (nhost && ndev) return set_err(c_, LSM_ERR_MIXED_MEMORY, "arrays of one call split between host and device");
        host_ = nhost > 0;
        int slot = 0;
        for (auto& a : args_) {
            if (!a.p) continue;
            if (!a.host) { *a.dev = const_cast<void*>(a.p); continue; }
            cudaError_t e;
            void* d = pool_get(c_, "stage" + std::to_string(slot++), a.bytes, &e);
            if (!d) return cuda_fail(c_, e, "cudaMalloc(stage)");
            *a.dev = d;
            if (a.d != OUT) LSM_CU(c_, cudaMemcpyAsync(d, a.p, a.bytes, cudaMemcpyHostToDevice, c_->stream));
        }
        return LSM_OK;
    }
    int finish() {
        for (auto& a : args_) {
            if (!a.p || !a.host || a.d == IN) continue;
            LSM_CU(c_, cudaMemcpyAsync(const_cast<void*>(a.p), *a.dev, a.bytes, cudaMemcpyDeviceToHost, c_->stream));
        }
        LSM_CU(c_, cudaStreamSynchronize(c_->stream));
        return LSM_OK;
    }
    bool host() const { return host_; }

private:
    struct Arg { const void* p; size_t bytes; Dir d; void** dev; bool host = false; };
    lsm_context* c_;
    std::vector<Arg> args_;
    bool host_ = false;
};

// Common prologue: handle, device, grid.
#define LSM_PROLOGUE(h, g)                                           \
    lsm_context* c = nullptr;                                        \
    {                                                                \
        int st_ = resolve((h), &c);                                  \
        if (st_) return st_;                                         \
    }                                                                \
    DeviceGuard guard_(c->device);                                   \
    DevGrid dg;                                                      \
    {                                                                \
        int st_ = check_grid(c, (g), &dg);                           \
        if (st_) return st_;                                         \
    }                                                                \
    const size_t N = (size_t)dg.ni * dg.nj * dg.nk;                  \
    (void)N;

#define LSM_TRY(x)                 \
    do {                           \
        int st_ = (x);             \
        if (st_) return st_;       \
    } while (0)

int after_launch(lsm_context* c) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, e, "kernel launch");
    return LSM_OK;
}

int exchange(lsm_context* c, double* field, const lsm_grid* g) {
    if (!c->xfn) return LSM_OK;
    LSM_CU(c, cudaStreamSynchronize(c->stream));
    int st = c->xfn(c->xuser, field, g);
    if (st) return set_err(c, st, "exchange callback failed");
    return LSM_OK;
}

int read_err(lsm_context* c, unsigned* flags) {
    LSM_CU(c, cudaMemcpyAsync(flags, c->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    LSM_CU(c, cudaStreamSynchronize(c->stream));
    return LSM_OK;
}

// TVD-RK3 coefficients (a, b, c) per stage, src/ad_RKTVD3.F90:36-48
const double kRK[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};

// One ad_RKTVD3 call on device buffers.  phin is read-only; the result lands
// in bufs[0]; bufs[1] is scratch.  Neither may alias phin.
int rk3_device(lsm_context* c, const lsm_grid* g, const DevGrid& dg, const lsm_params* p, const double* phin,
               const double* ucn, const double* aj, const int* mask, double* out, double* tmp) {
    const lsm::DevBC bc = make_bc(p);
    const double* in[3] = {phin, out, tmp};
    double* dst[3] = {out, tmp, out};
    for (int rk = 0; rk < 3; ++rk) {
        lsm::launch_rk_stage(dg, p->orderAD, phin, in[rk], ucn, aj, mask, kRK[rk][0], kRK[rk][1], kRK[rk][2],
                             p->delti_lsm, dst[rk], c->stream);
        lsm::launch_bc_rk(dg, bc, p->orderAD, phin, in[rk], ucn, aj, mask, kRK[rk][0], kRK[rk][1], kRK[rk][2],
                          p->delti_lsm, dst[rk], c->stream);
        LSM_TRY(after_launch(c));
        LSM_TRY(exchange(c, dst[rk], g));
    }
    return LSM_OK;
}

// `reinitialization` on device buffers: phi0 read-only, result in *res (one of d1/d2).
int reinit_device(lsm_context* c, const lsm_grid* g, const DevGrid& dg, const lsm_params* p, const double* phi0,
                  const double* csi, const double* eta, const double* zet, double* d1, double* d2, double** res) {
    cudaError_t e;
    const size_t N = (size_t)dg.ni * dg.nj * dg.nk;
    double* sg = (double*)pool_get(c, "rn_sign", N * 8, &e);
    double* ng = sg ? (double*)pool_get(c, "rn_ngrad", N * 8, &e) : nullptr;
    double* dl = ng ? (double*)pool_get(c, "rn_delta", N * 8, &e) : nullptr;
    if (!dl) return cuda_fail(c, e, "cudaMalloc(reinit)");
    lsm::launch_sign_ini(dg, phi0, csi, eta, zet, p->epslsm, p->M_Sphi0, sg, ng, dl, c->stream);
    LSM_TRY(after_launch(c));
    LSM_TRY(exchange(c, sg, g));
    LSM_TRY(exchange(c, ng, g));
    const double* cur = phi0;
    double* bufs[2] = {d1, d2};
    if (p->RNitermax == 0) {
        lsm::launch_copy(phi0, d1, (long long)N, c->stream);
        *res = d1;
        return after_launch(c);
    }
    for (int it = 0; it < p->RNitermax; ++it) {
        double* out = bufs[it & 1];
        lsm::launch_reinit_step(dg, p->RNtimestep, cur, sg, ng, dl, phi0, csi, eta, zet, out, c->stream);
        LSM_TRY(after_launch(c));
        LSM_TRY(exchange(c, out, g));
        cur = out;
    }
    *res = const_cast<double*>(cur);
    return LSM_OK;
}

// reinitialisation_test2 (src/reinitialisation_test2.F90:1-221, non-hybrid)
// from phizero into dn1 (dn: scratch); *iters = pseudo-time iterations run.
// The convergence test needs the field's maximum and minimum on the host
// once per iteration (the reference's maxval/minval, then `exit`).
int sussman_device(lsm_context* c, const DevGrid& dg, const lsm_params* p, const double* phizero,
                   const double* csi, const double* eta, const double* zet, double* dn1, double* dn, int* iters) {
    if (p->OrderReinitialisationBoundaries < 1 || p->OrderReinitialisationBoundaries > 3)
        return set_err(c, LSM_ERR_BAD_PARAM, "OrderReinitialisationBoundaries must be 1, 2 or 3");
    cudaError_t e;
    const long long N = (long long)dg.ni * dg.nj * dg.nk;
    double* sg = (double*)pool_get(c, "ss_sign", 8 * N, &e);
    double* ng = sg ? (double*)pool_get(c, "ss_ng", 8 * N, &e) : nullptr;
    double* ngc = ng ? (double*)pool_get(c, "ss_ngc", 8 * N, &e) : nullptr;
    double* part = ngc ? (double*)pool_get(c, "ss_part", 16 * (size_t)lsm::minmax_partials(N) + 16, &e) : nullptr;
    if (!part) return cuda_fail(c, e, "cudaMalloc(reinitialisation_test2)");
    double* res = part + 2 * lsm::minmax_partials(N);
    // the i-face blocks of calc_NormGrad_d take phizero at the last node of
    // the interior loop (src/calc_NormGrad_d.F90:41-56, 186-376)
    const long long stale = lsm::gid(dg, dg.ib - (dg.pf ? 1 : 0), dg.jb - (dg.pr ? 1 : 0), dg.kb - (dg.pu ? 1 : 0));
    const int order = p->OrderReinitialisationBoundaries, enobc = p->ENOBCReinitialisation ? 1 : 0;
    const double C[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
    lsm::launch_sign_phi0(N, phizero, p->epslsm, sg, c->stream);
    lsm::launch_copy(phizero, dn1, N, c->stream);
    lsm::launch_normgrad_d(dg, order, enobc, dn1, phizero, stale, csi, eta, zet, ng, c->stream);
    LSM_TRY(after_launch(c));
    int done = 0;
    for (int it = 1; it <= p->RNitermax; ++it) {
        double mm[2];
        lsm::launch_minmax(N, ng, part, res, c->stream);
        LSM_CU(c, cudaMemcpyAsync(mm, res, sizeof(mm), cudaMemcpyDeviceToHost, c->stream));
        LSM_CU(c, cudaStreamSynchronize(c->stream));
        if (std::fabs(mm[0] - 1.0) < p->epsReinitialisation && std::fabs(mm[1] - 1.0) < p->epsReinitialisation) break;
        lsm::launch_copy(dn1, dn, N, c->stream);
        lsm::launch_normgrad_d(dg, order, enobc, dn, phizero, stale, csi, eta, zet, ngc, c->stream);
        for (int rk = 0; rk < 3; ++rk) {
            lsm::launch_normgrad_d(dg, order, enobc, dn1, phizero, stale, csi, eta, zet, ng, c->stream);
            lsm::launch_sussman_rk(dg, dn, dn1, ng, ngc, sg, p->epslsm, p->epsReinitialisation, p->RNtimestep,
                                   C[rk][0], C[rk][1], C[rk][2], c->stream);
        }
        LSM_TRY(after_launch(c));
        done = it;
    }
    if (iters) *iters = done;
    return LSM_OK;
}

// list-directed REAL(8) output in the shape gfortran gives it
void format_real8(double v, char* buf, size_t n) {
    const double a = v < 0 ? -v : v;
    if (v == 0.0) snprintf(buf, n, "   0.0000000000000000     ");
    else if (a >= 0.1 && a < 1.0e16) {
        int digits_before = 1;
        for (double t = a; t >= 10.0; t /= 10.0) ++digits_before;
        int prec = 17 - digits_before;
        if (prec < 0) prec = 0;
        snprintf(buf, n, "   %.*f     ", prec, v);
    } else {
        snprintf(buf, n, "   %.16E", v);
    }
}

}  // namespace

// ============================================================= public API
extern "C" {

void lsm_params_default(lsm_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->epslsm = 0.0;
    p->numiter_lsm = 1;
    p->delti_lsm = 0.0;
    p->RNitermax = 15;          // control.dat: reinitialization_iterations
    p->RNtimestep = 0.00078125; // control.dat: reinitialization_dtau
    p->RNfreq = 1;
    for (int f = 0; f < 6; ++f) p->btype_lsm[f] = 1;
    p->bc_extrapolation_order = 1;
    p->isnarrow = 0;            // narrow_band = off
    p->narrowcoef = 3.0;
    p->orderAD = 1;             // WENO3
    p->sussman_correction_method = 0;
    p->call_levelsetmethod = 1;
    p->call_reinitialisation = 1;
    p->hybrid_reinitialisation = 0;
    p->TotalVolumeComputation = 1;
    p->GlobalMassCorrection = 0;
    p->BigPhi = 5.0;
    p->epsReinitialisation = 1.0e-5;
    p->M_Sphi0 = 1;
    p->reinit_scheme = 0;
    p->write_global_volume = 0;
    p->OrderReinitialisationBoundaries = 1;  // control.dat
    p->ENOBCReinitialisation = 0;            // control.dat: .false.
    p->ConvergenceToleranceGeomReini = 1.0e-9;  // control.dat
}

int lsm_create(lsm_handle* h, int device, void* stream) {
    if (!h) return LSM_ERR_NULL;
    return make_context(h, device, (cudaStream_t)stream);
}

int lsm_destroy(lsm_handle h) {
    if (!h) return LSM_ERR_NULL;
    DeviceGuard guard(h->device);
    cudaStreamSynchronize(h->stream);
    for (auto& kv : h->pool)
        if (kv.second.p) cudaFree(kv.second.p);
    cudaFree(h->d_err);
    cudaFree(h->d_result);
    cudaFree(h->d_count);
    {
        std::lock_guard<std::mutex> lk(g_default_mu);
        for (auto& d : g_default)
            if (d == h) d = nullptr;
    }
    delete h;
    return LSM_OK;
}

int lsm_set_stream(lsm_handle h, void* stream) {
    lsm_context* c = nullptr;
    LSM_TRY(resolve(h, &c));
    c->stream = (cudaStream_t)stream;
    return LSM_OK;
}

int lsm_set_exchange_callback(lsm_handle h, lsm_exchange_fn fn, void* user) {
    lsm_context* c = nullptr;
    LSM_TRY(resolve(h, &c));
    c->xfn = fn;
    c->xuser = user;
    return LSM_OK;
}

const char* lsm_status_string(int s) {
    switch (s) {
    case LSM_OK: return "ok";
    case LSM_ERR_NULL: return "required pointer is NULL";
    case LSM_ERR_BAD_SHAPE: return "bad grid shape";
    case LSM_ERR_BAD_PARAM: return "bad parameter";
    case LSM_ERR_UNSUPPORTED: return "branch outside the level-set transport path";
    case LSM_ERR_NONFINITE: return "non-finite value";
    case LSM_ERR_NEGATIVE_VOLUME: return "negative tetrahedron water volume";
    case LSM_ERR_MIXED_MEMORY: return "arrays split between host and device";
    case LSM_ERR_CAPACITY: return "output buffer too small";
    case LSM_ERR_CUDA: return "CUDA runtime error";
    case LSM_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

const char* lsm_last_error(lsm_handle h) {
    if (h) return h->last_error.c_str();
    return t_err.c_str();
}

long long lsm_kernel_launch_count(lsm_handle h) {
    if (h) return (long long)(lsm::g_launches - h->launches0);
    return (long long)lsm::g_launches;
}

// ------------------------------------------------------------------ A1
int lsm_rhs_contra_j(lsm_handle h, const lsm_grid* g, const double* q, const double* csi, const double* eta,
                     const double* zet, const double* aj, double* ucn) {
    LSM_PROLOGUE(h, g);
    if (!q || !csi || !eta || !zet || !aj || !ucn) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dq, *dcsi, *deta, *dzet, *daj, *du;
    Staging S(c);
    S.add(q, 32 * N, Staging::IN, &dq);
    S.add(csi, 24 * N, Staging::IN, &dcsi);
    S.add(eta, 24 * N, Staging::IN, &deta);
    S.add(zet, 24 * N, Staging::IN, &dzet);
    S.add(aj, 8 * N, Staging::IN, &daj);
    S.add(ucn, 24 * N, Staging::OUT, &du);
    LSM_TRY(S.resolve());
    lsm::launch_contra(dg, (const double*)dq, (const double*)dcsi, (const double*)deta, (const double*)dzet,
                       (const double*)daj, (double*)du, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------- A2 / A7
static int rh_ad_common(lsm_handle h, const lsm_grid* g, int order, const double* phi, const double* ucn,
                        const int* mask, double* rh) {
    LSM_PROLOGUE(h, g);
    if (!phi || !ucn || !rh) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dphi, *du, *dm, *drh;
    Staging S(c);
    S.add(phi, 8 * N, Staging::IN, &dphi);
    S.add(ucn, 24 * N, Staging::IN, &du);
    S.add(mask, 4 * N, Staging::IN, &dm);
    S.add(rh, 8 * N, Staging::OUT, &drh);
    LSM_TRY(S.resolve());
    lsm::launch_rh_ad(dg, order, (const double*)dphi, (const double*)du, (const int*)dm, (double*)drh, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

int lsm_calc_rh_ad_weno3(lsm_handle h, const lsm_grid* g, const double* phi, const double* ucn, const int* mask,
                         double* rh) {
    return rh_ad_common(h, g, 1, phi, ucn, mask, rh);
}

int lsm_calc_rh_ad(lsm_handle h, const lsm_grid* g, const double* phi, const double* ucn, const int* mask,
                   double* rh) {
    return rh_ad_common(h, g, 0, phi, ucn, mask, rh);
}

// ------------------------------------------------------------------ A4
int lsm_ad_rktvd3(lsm_handle h, const lsm_grid* g, const lsm_params* p, double* phi_n1, const double* phi_n,
                  const int* mask, const double* ucn, const double* aj) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (!phi_n1 || !phi_n || !ucn || !aj) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dout, *din, *dm, *du, *daj;
    Staging S(c);
    S.add(phi_n1, 8 * N, Staging::OUT, &dout);
    S.add(phi_n, 8 * N, Staging::IN, &din);
    S.add(mask, 4 * N, Staging::IN, &dm);
    S.add(ucn, 24 * N, Staging::IN, &du);
    S.add(aj, 8 * N, Staging::IN, &daj);
    LSM_TRY(S.resolve());
    cudaError_t e;
    double* A = (double*)pool_get(c, "rk_a", 8 * N, &e);
    double* B = A ? (double*)pool_get(c, "rk_b", 8 * N, &e) : nullptr;
    if (!B) return cuda_fail(c, e, "cudaMalloc(rk)");
    LSM_TRY(rk3_device(c, g, dg, p, (const double*)din, (const double*)du, (const double*)daj, (const int*)dm, A, B));
    lsm::launch_copy(A, (double*)dout, (long long)N, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ A5
int lsm_bcond_lsm(lsm_handle h, const lsm_grid* g, const lsm_params* p, double* phi) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (!phi) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void* dphi;
    Staging S(c);
    S.add(phi, 8 * N, Staging::INOUT, &dphi);
    LSM_TRY(S.resolve());
    cudaError_t e;
    double* T = (double*)pool_get(c, "bc_tmp", 8 * N, &e);
    if (!T) return cuda_fail(c, e, "cudaMalloc(bc)");
    lsm::launch_copy((const double*)dphi, T, (long long)N, c->stream);
    lsm::launch_bc_full(dg, make_bc(p), T, (double*)dphi, nullptr, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ R1
int lsm_calc_sign_ini(lsm_handle h, const lsm_grid* g, const double* phi0, const double* csi, const double* eta,
                      const double* zet, double epslsm, int M_Sphi0, double* sgn, double* ng) {
    LSM_PROLOGUE(h, g);
    if (!phi0 || !csi || !eta || !zet || !sgn || !ng) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dcsi, *deta, *dzet, *ds, *dn;
    Staging S(c);
    S.add(phi0, 8 * N, Staging::IN, &dp);
    S.add(csi, 24 * N, Staging::IN, &dcsi);
    S.add(eta, 24 * N, Staging::IN, &deta);
    S.add(zet, 24 * N, Staging::IN, &dzet);
    S.add(sgn, 8 * N, Staging::OUT, &ds);
    S.add(ng, 8 * N, Staging::OUT, &dn);
    LSM_TRY(S.resolve());
    lsm::launch_sign_ini(dg, (const double*)dp, (const double*)dcsi, (const double*)deta, (const double*)dzet, epslsm,
                         M_Sphi0, (double*)ds, (double*)dn, nullptr, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ R2
int lsm_calc_rh_rn(lsm_handle h, const lsm_grid* g, const double* d, const double* sgn, const double* csi,
                   const double* eta, const double* zet, double* rh) {
    LSM_PROLOGUE(h, g);
    if (!d || !sgn || !csi || !eta || !zet || !rh) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dd, *ds, *dcsi, *deta, *dzet, *drh;
    Staging S(c);
    S.add(d, 8 * N, Staging::IN, &dd);
    S.add(sgn, 8 * N, Staging::IN, &ds);
    S.add(csi, 24 * N, Staging::IN, &dcsi);
    S.add(eta, 24 * N, Staging::IN, &deta);
    S.add(zet, 24 * N, Staging::IN, &dzet);
    S.add(rh, 8 * N, Staging::OUT, &drh);
    LSM_TRY(S.resolve());
    lsm::launch_rh_rn(dg, (const double*)dd, (const double*)ds, (const double*)dcsi, (const double*)deta,
                      (const double*)dzet, (double*)drh, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ R3
int lsm_calc_lambda_rn(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* phi0,
                       const double* ng0, const double* d, double dt, double* lam) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (p->sussman_correction_method != 0)
        return set_err(c, LSM_ERR_UNSUPPORTED, "sussman_correction_method 1 (testfilter) is outside the path");
    if (!phi0 || !ng0 || !d || !lam) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dn, *dd, *dl;
    Staging S(c);
    S.add(phi0, 8 * N, Staging::IN, &dp);
    S.add(ng0, 8 * N, Staging::IN, &dn);
    S.add(d, 8 * N, Staging::IN, &dd);
    S.add(lam, 8 * N, Staging::OUT, &dl);
    LSM_TRY(S.resolve());
    lsm::launch_lambda_rn(dg, p->epslsm, (const double*)dp, (const double*)dn, (const double*)dd, dt, (double*)dl,
                          c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ R0
int lsm_reinitialization(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* phi0,
                         const double* csi, const double* eta, const double* zet, double* out) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (p->sussman_correction_method != 0)
        return set_err(c, LSM_ERR_UNSUPPORTED, "sussman_correction_method 1 (testfilter) is outside the path");
    if (!phi0 || !csi || !eta || !zet || !out) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dcsi, *deta, *dzet, *dout;
    Staging S(c);
    S.add(phi0, 8 * N, Staging::IN, &dp);
    S.add(csi, 24 * N, Staging::IN, &dcsi);
    S.add(eta, 24 * N, Staging::IN, &deta);
    S.add(zet, 24 * N, Staging::IN, &dzet);
    S.add(out, 8 * N, Staging::OUT, &dout);
    LSM_TRY(S.resolve());
    cudaError_t e;
    double* D1 = (double*)pool_get(c, "rn_d1", 8 * N, &e);
    double* D2 = D1 ? (double*)pool_get(c, "rn_d2", 8 * N, &e) : nullptr;
    if (!D2) return cuda_fail(c, e, "cudaMalloc(reinit)");
    double* res = nullptr;
    LSM_TRY(reinit_device(c, g, dg, p, (const double*)dp, (const double*)dcsi, (const double*)deta,
                          (const double*)dzet, D1, D2, &res));
    lsm::launch_copy(res, (double*)dout, (long long)N, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ L0
int lsm_calc_normgrad_d(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* phi_rn,
                        const double* phizero, const double* csi, const double* eta, const double* zet,
                        double* normgrad) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (p->OrderReinitialisationBoundaries < 1 || p->OrderReinitialisationBoundaries > 3)
        return set_err(c, LSM_ERR_BAD_PARAM, "OrderReinitialisationBoundaries must be 1, 2 or 3");
    if (!phi_rn || !phizero || !csi || !eta || !zet || !normgrad) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dz0, *dcsi, *deta, *dzet, *dout;
    Staging S(c);
    S.add(phi_rn, 8 * N, Staging::IN, &dp);
    S.add(phizero, 8 * N, Staging::IN, &dz0);
    S.add(csi, 24 * N, Staging::IN, &dcsi);
    S.add(eta, 24 * N, Staging::IN, &deta);
    S.add(zet, 24 * N, Staging::IN, &dzet);
    S.add(normgrad, 8 * N, Staging::OUT, &dout);
    LSM_TRY(S.resolve());
    const long long stale = lsm::gid(dg, dg.ib - (dg.pf ? 1 : 0), dg.jb - (dg.pr ? 1 : 0), dg.kb - (dg.pu ? 1 : 0));
    lsm::launch_normgrad_d(dg, p->OrderReinitialisationBoundaries, p->ENOBCReinitialisation ? 1 : 0,
                           (const double*)dp, (const double*)dz0, stale, (const double*)dcsi, (const double*)deta,
                           (const double*)dzet, (double*)dout, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

int lsm_reinitialisation_test2(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* phizero,
                               const double* csi, const double* eta, const double* zet, double* out,
                               int* iterations) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (!phizero || !csi || !eta || !zet || !out) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dcsi, *deta, *dzet, *dout;
    Staging S(c);
    S.add(phizero, 8 * N, Staging::IN, &dp);
    S.add(csi, 24 * N, Staging::IN, &dcsi);
    S.add(eta, 24 * N, Staging::IN, &deta);
    S.add(zet, 24 * N, Staging::IN, &dzet);
    S.add(out, 8 * N, Staging::OUT, &dout);
    LSM_TRY(S.resolve());
    cudaError_t e;
    double* D1 = (double*)pool_get(c, "rn_d1", 8 * N, &e);
    double* D2 = D1 ? (double*)pool_get(c, "rn_d2", 8 * N, &e) : nullptr;
    if (!D2) return cuda_fail(c, e, "cudaMalloc(reinitialisation_test2)");
    LSM_TRY(sussman_device(c, dg, p, (const double*)dp, (const double*)dcsi, (const double*)deta,
                           (const double*)dzet, D1, D2, iterations));
    lsm::launch_copy(D1, (double*)dout, (long long)N, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ N1
int lsm_narrowband(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* phin, int* nb) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (!phin || !nb) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dn;
    Staging S(c);
    S.add(phin, 8 * N, Staging::IN, &dp);
    S.add(nb, 4 * N, Staging::OUT, &dn);
    LSM_TRY(S.resolve());
    // tol = 1.0E-5 is a default-real (single precision) literal, src/narrowband.F90:9
    const double thr = p->narrowcoef * p->epslsm + (double)1.0E-5f;
    lsm::launch_narrowband(dg, thr, p->isnarrow, (const double*)dp, (int*)dn, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

// ------------------------------------------------------------------ V1
static int volume_common(lsm_handle h, const lsm_grid* g, const double* phi, const double* x, const double* y,
                         const double* z, double* vols, int* adv, double* cellvol) {
    LSM_PROLOGUE(h, g);
    if (!phi || !x || !y || !z) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dx, *dy, *dz, *da, *dcv;
    Staging S(c);
    S.add(phi, 8 * N, Staging::IN, &dp);
    S.add(x, 8 * N, Staging::IN, &dx);
    S.add(y, 8 * N, Staging::IN, &dy);
    S.add(z, 8 * N, Staging::IN, &dz);
    S.add(adv, 4 * N, Staging::OUT, &da);
    S.add(cellvol, 8 * N, Staging::OUT, &dcv);
    LSM_TRY(S.resolve());
    cudaError_t e;
    const int nblk = lsm::volume_partial_blocks(dg);
    double* part = (double*)pool_get(c, "vol_part", 24 * (size_t)nblk, &e);
    unsigned char* pcf = nullptr;
    if (!part) return cuda_fail(c, e, "cudaMalloc(volume)");
    if (adv) {
        pcf = (unsigned char*)pool_get(c, "vol_pcflag", N, &e);
        if (!pcf) return cuda_fail(c, e, "cudaMalloc(volume)");
    }
    LSM_CU(c, cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
    if (cellvol) LSM_CU(c, cudaMemsetAsync(dcv, 0, 8 * N, c->stream));
    lsm::launch_volume(dg, (const double*)dp, (const double*)dx, (const double*)dy, (const double*)dz, part,
                       c->d_result, pcf, (double*)dcv, c->d_err, c->stream);
    if (adv) lsm::launch_adv_nodes(dg, pcf, (int*)da, c->stream);
    LSM_TRY(after_launch(c));
    double res[4];
    LSM_CU(c, cudaMemcpyAsync(res, c->d_result, sizeof(res), cudaMemcpyDeviceToHost, c->stream));
    LSM_TRY(S.finish());
    if (vols) std::memcpy(vols, res, sizeof(res));
    unsigned fl = 0;
    LSM_TRY(read_err(c, &fl));
    if (fl & lsm::kErrNegativeVolume) return set_err(c, LSM_ERR_NEGATIVE_VOLUME, "negative tetrahedron water volume");
    return LSM_OK;
}

int lsm_total_water_volume(lsm_handle h, const lsm_grid* g, const double* phi, const double* x, const double* y,
                           const double* z, double* vols, int* adv) {
    if (!vols) return set_err(nullptr, LSM_ERR_NULL, "volumes is NULL");
    return volume_common(h, g, phi, x, y, z, vols, adv, nullptr);
}

int lsm_cell_water_volumes(lsm_handle h, const lsm_grid* g, const double* phi, const double* x, const double* y,
                           const double* z, double* cellvol) {
    if (!cellvol) return set_err(nullptr, LSM_ERR_NULL, "cellvol is NULL");
    return volume_common(h, g, phi, x, y, z, nullptr, nullptr, cellvol);
}

// ------------------------------------------------------------------ N3
int lsm_get_gfm_list(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* phi, int* count,
                     int* list, int ld) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    if (!phi || !count) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp;
    Staging S(c);
    S.add(phi, 8 * N, Staging::IN, &dp);
    LSM_TRY(S.resolve());
    cudaError_t e;
    int* scratch = (int*)pool_get(c, "gfm_scratch", 4 * (size_t)lsm::gfm_scratch_ints(dg), &e);
    if (!scratch) return cuda_fail(c, e, "cudaMalloc(gfm)");
    lsm::launch_gfm_list(dg, p->BigPhi, (const double*)dp, scratch, c->d_count, nullptr, 0, g->il, g->jl, g->kl,
                         c->stream);
    LSM_TRY(after_launch(c));
    int cnt = 0;
    LSM_CU(c, cudaMemcpyAsync(&cnt, c->d_count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    LSM_CU(c, cudaStreamSynchronize(c->stream));
    *count = cnt;
    if (!list) return S.finish();
    if (ld < cnt) {
        S.finish();
        return set_err(c, LSM_ERR_CAPACITY, "ghost-fluid list capacity smaller than the node count");
    }
    // the list may live on the host or the device independently of phi
    cudaPointerAttributes at;
    bool list_dev = cudaPointerGetAttributes(&at, list) == cudaSuccess &&
                    (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    int* dlist = list;
    if (!list_dev) {
        dlist = (int*)pool_get(c, "gfm_list", 12 * (size_t)(ld > 0 ? ld : 1), &e);
        if (!dlist) return cuda_fail(c, e, "cudaMalloc(gfm list)");
    }
    if (cnt > 0) {
        lsm::launch_gfm_list(dg, p->BigPhi, (const double*)dp, scratch, c->d_count, dlist, ld, g->il, g->jl, g->kl,
                             c->stream);
        LSM_TRY(after_launch(c));
        if (!list_dev)
            for (int d = 0; d < 3; ++d)
                LSM_CU(c, cudaMemcpyAsync(list + (size_t)d * ld, dlist + (size_t)d * ld, 4 * (size_t)cnt,
                                          cudaMemcpyDeviceToHost, c->stream));
    }
    return S.finish();
}

// ------------------------------------------------ geometric reinitialisation
namespace {
void* geo_alloc(void* ctx, const char* name, size_t bytes, cudaError_t* e) {
    return pool_get(static_cast<lsm_context*>(ctx), name, bytes, e);
}

int geo_check(lsm_context* c, const lsm_grid* g) {
    if (g->igp || g->jgp || g->kgp)
        return set_err(c, LSM_ERR_UNSUPPORTED, "geometric reinitialisation runs on a grid without ghost planes");
    for (int f = 0; f < 6; ++f)
        if (!g->physical_face[f])
            return set_err(c, LSM_ERR_UNSUPPORTED, "geometric reinitialisation needs every face physical");
    return LSM_OK;
}

int geo_run(lsm_context* c, const DevGrid& dg, const lsm_params* p, const double* phi0, const double* x,
            const double* y, const double* z, double target, double* pc, int* tag, lsm_geom_info* info) {
    lsm::GeoInfo gi{};
    cudaError_t e = lsm::geo_reinit(dg, phi0, x, y, z, target, p->GlobalMassCorrection ? 1 : 0,
                                    p->ConvergenceToleranceGeomReini, pc, tag, geo_alloc, c, c->d_err, c->d_count,
                                    &gi, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "geometric reinitialisation");
    if (info) {
        info->nnodes = gi.nnodes; info->ntetrahedra = gi.ntetrahedra; info->nsecond = gi.nsecond;
        info->newton_iterations = gi.newton_iterations; info->newton_converged = gi.newton_converged;
        info->C = gi.C;
    }
    return LSM_OK;
}
}  // namespace

int lsm_geometric_reinitialisation(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* phizero,
                                   const double* x, const double* y, const double* z, double total_water_volume,
                                   double* phicorrected, int* interface_nodes_id, lsm_geom_info* info) {
    LSM_PROLOGUE(h, g);
    if (!p) return set_err(c, LSM_ERR_NULL, "params is NULL");
    LSM_TRY(geo_check(c, g));
    if (!phizero || !x || !y || !z || !phicorrected || !interface_nodes_id)
        return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dp, *dx, *dy, *dz, *dpc, *did;
    Staging S(c);
    S.add(phizero, 8 * N, Staging::IN, &dp);
    S.add(x, 8 * N, Staging::IN, &dx);
    S.add(y, 8 * N, Staging::IN, &dy);
    S.add(z, 8 * N, Staging::IN, &dz);
    S.add(phicorrected, 8 * N, Staging::INOUT, &dpc);
    S.add(interface_nodes_id, 4 * N, Staging::OUT, &did);
    LSM_TRY(S.resolve());
    LSM_CU(c, cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
    LSM_TRY(geo_run(c, dg, p, (const double*)dp, (const double*)dx, (const double*)dy, (const double*)dz,
                    total_water_volume, (double*)dpc, (int*)did, info));
    LSM_TRY(S.finish());
    unsigned fl = 0;
    LSM_TRY(read_err(c, &fl));
    if (fl & lsm::kErrNegativeVolume) return set_err(c, LSM_ERR_NEGATIVE_VOLUME, "negative tetrahedron water volume");
    return LSM_OK;
}

// ------------------------------------------------------------------ V2
int lsm_convergence_volume(lsm_handle h, double* out) {
    if (!h || !out) return LSM_ERR_NULL;
    *out = h->conv_volume;
    return LSM_OK;
}

int lsm_write_total_water_volume(double v, const char* path) {
    FILE* f = std::fopen(path ? path : "GlobalVolume.txt", "a");
    if (!f) return set_err(nullptr, LSM_ERR_BAD_PARAM, "cannot open the global volume file");
    char buf[64];
    format_real8(v, buf, sizeof(buf));
    std::fprintf(f, "%s\n", buf);
    std::fclose(f);
    return LSM_OK;
}

// ------------------------------------------------------------------ A0
int lsm_levelsetmethod(lsm_handle h, const lsm_grid* g, const lsm_params* p, const double* q, const double* csi,
                       const double* eta, const double* zet, const double* aj, double* phi, const double* phi_n,
                       const double* x, const double* y, const double* z, int iter, double* vols_out) {
    LSM_PROLOGUE(h, g);
    LSM_TRY(check_params(c, p));
    const bool hybrid = p->call_reinitialisation && p->hybrid_reinitialisation;
    if (hybrid) LSM_TRY(geo_check(c, g));
    if (p->reinit_scheme != 0 && p->reinit_scheme != 1)
        return set_err(c, LSM_ERR_UNSUPPORTED, "reinit_scheme must be 0 or 1");
    if (p->sussman_correction_method != 0)
        return set_err(c, LSM_ERR_UNSUPPORTED, "sussman_correction_method 1 (testfilter) is outside the path");
    if (!q || !csi || !eta || !zet || !aj || !phi || !phi_n || !x || !y || !z)
        return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dq, *dcsi, *deta, *dzet, *daj, *dphi, *dphin, *dx, *dy, *dz;
    Staging S(c);
    S.add(q, 32 * N, Staging::IN, &dq);
    S.add(csi, 24 * N, Staging::IN, &dcsi);
    S.add(eta, 24 * N, Staging::IN, &deta);
    S.add(zet, 24 * N, Staging::IN, &dzet);
    S.add(aj, 8 * N, Staging::IN, &daj);
    S.add(phi, 8 * N, Staging::INOUT, &dphi);
    S.add(phi_n, 8 * N, Staging::IN, &dphin);
    S.add(x, 8 * N, Staging::IN, &dx);
    S.add(y, 8 * N, Staging::IN, &dy);
    S.add(z, 8 * N, Staging::IN, &dz);
    LSM_TRY(S.resolve());
    cudaError_t e;
    double* ucn = (double*)pool_get(c, "ucn", 24 * N, &e);
    double* B0 = ucn ? (double*)pool_get(c, "lsm_b0", 8 * N, &e) : nullptr;
    double* B1 = B0 ? (double*)pool_get(c, "lsm_b1", 8 * N, &e) : nullptr;
    double* B2 = B1 ? (double*)pool_get(c, "lsm_b2", 8 * N, &e) : nullptr;
    const int nblk = lsm::volume_partial_blocks(dg);
    double* part = B2 ? (double*)pool_get(c, "vol_part", 24 * (size_t)nblk, &e) : nullptr;
    if (!part) return cuda_fail(c, e, "cudaMalloc(levelsetmethod)");
    unsigned char* pcf = nullptr;
    int* adv = nullptr;
    if (hybrid) {
        pcf = (unsigned char*)pool_get(c, "vol_pcflag", N, &e);
        adv = pcf ? (int*)pool_get(c, "lsm_adv", 4 * N, &e) : nullptr;
        if (!adv) return cuda_fail(c, e, "cudaMalloc(levelsetmethod)");
    }
    LSM_CU(c, cudaMemsetAsync(c->d_err, 0, sizeof(unsigned), c->stream));
    // 1. pre-advection water volume, levelsetmethod.F90:178-196.  Without the
    //    hybrid reinitialisation every node is advected (:218-219); with it
    //    the advection runs on the AdvectionNodes band of this pass.
    lsm::launch_volume(dg, (const double*)dphi, (const double*)dx, (const double*)dy, (const double*)dz, part,
                       c->d_result, pcf, nullptr, c->d_err, c->stream);
    if (hybrid) lsm::launch_adv_nodes(dg, pcf, adv, c->stream);
    LSM_TRY(after_launch(c));
    // 2. advection, levelsetmethod.F90:221-243
    const double* cur = (const double*)dphi;
    double* bufs[3] = {B0, B1, B2};
    if (p->call_levelsetmethod) {
        lsm::launch_contra(dg, (const double*)dq, (const double*)dcsi, (const double*)deta, (const double*)dzet,
                           (const double*)daj, ucn, c->stream);
        LSM_TRY(after_launch(c));
        cur = (const double*)dphin;
        for (int it = 0; it < p->numiter_lsm; ++it) {
            double* X = nullptr;
            double* Y = nullptr;
            for (double* b : bufs) {
                if (b == cur) continue;
                if (!X) X = b; else if (!Y) Y = b;
            }
            LSM_TRY(rk3_device(c, g, dg, p, cur, ucn, (const double*)daj, adv, X, Y));
            cur = X;
        }
    }
    // 2b. GlobalMassCorrection: TotalWaterVolume of the advected phi,
    //     levelsetmethod.F90:245-264 (the same routine and tetrahedra split
    //     as the pre-advection pass); its K and second-tetrahedra volumes
    //     give ConvergenceVolume below
    if (p->GlobalMassCorrection) {
        lsm::launch_volume(dg, cur, (const double*)dx, (const double*)dy, (const double*)dz, part, c->d_result + 4,
                           nullptr, nullptr, c->d_err, c->stream);
        LSM_TRY(after_launch(c));
    }
    // 3. reinitialisation, levelsetmethod.F90:290-326
    const bool do_rn = p->call_reinitialisation && p->RNfreq > 0 && iter % p->RNfreq == 0;
    if (do_rn) {
        double* X = nullptr;
        double* Y = nullptr;
        for (double* b : bufs) {
            if (b == cur) continue;
            if (!X) X = b; else if (!Y) Y = b;
        }
        double* res = nullptr;
        if (p->hybrid_reinitialisation) {
            // levelsetmethod.F90:300-309: phicorrected is the advected phi
            // (zero without advection) with +-9.9 away from the interface,
            // then the geometric reinitialisation against ConvergenceVolume
            double rv[8];
            LSM_CU(c, cudaMemcpyAsync(rv, c->d_result, sizeof(rv), cudaMemcpyDeviceToHost, c->stream));
            LSM_CU(c, cudaStreamSynchronize(c->stream));
            const double conv = p->GlobalMassCorrection ? rv[3] - (rv[4] + rv[5]) : rv[3];
            if (p->call_levelsetmethod) LSM_CU(c, cudaMemcpyAsync(X, cur, 8 * N, cudaMemcpyDeviceToDevice, c->stream));
            else LSM_CU(c, cudaMemsetAsync(X, 0, 8 * N, c->stream));
            lsm::launch_geo_seed((long long)N, cur, X, c->stream);
            LSM_TRY(after_launch(c));
            int* tag = (int*)pool_get(c, "geo_tag", 4 * N, &e);
            if (!tag) return cuda_fail(c, e, "cudaMalloc(levelsetmethod)");
            LSM_TRY(geo_run(c, dg, p, cur, (const double*)dx, (const double*)dy, (const double*)dz, conv, X, tag,
                            nullptr));
            res = X;
        } else if (p->reinit_scheme == 1) {
            // the reference's live call, src/levelsetmethod.F90:313
            LSM_TRY(sussman_device(c, dg, p, cur, (const double*)dcsi, (const double*)deta, (const double*)dzet, X,
                                   Y, nullptr));
            res = X;
        } else {
            LSM_TRY(reinit_device(c, g, dg, p, cur, (const double*)dcsi, (const double*)deta, (const double*)dzet,
                                  X, Y, &res));
        }
        lsm::launch_bc_full(dg, make_bc(p), res, (double*)dphi, c->d_err, c->stream);
        LSM_TRY(after_launch(c));
        LSM_TRY(exchange(c, (double*)dphi, g));
    } else if (cur != (const double*)dphi) {
        lsm::launch_copy(cur, (double*)dphi, (long long)N, c->stream);
        LSM_TRY(after_launch(c));
    }
    double res[8];
    LSM_CU(c, cudaMemcpyAsync(res, c->d_result, sizeof(res), cudaMemcpyDeviceToHost, c->stream));
    LSM_TRY(S.finish());
    if (vols_out) std::memcpy(vols_out, res, 4 * sizeof(double));
    // ConvergenceVolume = TotVol_PreAdv - (K + second tetrahedra after
    // advection) with GlobalMassCorrection, else TotVol_PreAdv
    // (levelsetmethod.F90:245-264; one rank: the reductions are identities)
    c->conv_volume = p->GlobalMassCorrection ? res[3] - (res[4] + res[5]) : res[3];
    if (p->write_global_volume) LSM_TRY(lsm_write_total_water_volume(res[3], nullptr));
    unsigned fl = 0;
    LSM_TRY(read_err(c, &fl));
    if (fl & lsm::kErrNegativeVolume) return set_err(c, LSM_ERR_NEGATIVE_VOLUME, "negative tetrahedron water volume");
    if (fl & lsm::kErrNonFinite) return set_err(c, LSM_ERR_NONFINITE, "non-finite phi after the level-set step");
    return LSM_OK;
}

// ------------------------------------------------- grid metrics (input prep)
// mg_metrics on one rank's fine grid (src/mg_metrics.F90:44-264); not part
// of the reference's level-set layer but the way its inputs are made.
int lsm_mg_metrics(lsm_handle h, const lsm_grid* g, const double* x, const double* y, const double* z, double* csi,
                   double* eta, double* zet, double* aj) {
    LSM_PROLOGUE(h, g);
    if (g->igp || g->jgp || g->kgp)
        return set_err(c, LSM_ERR_UNSUPPORTED, "metrics are computed on a grid without ghost planes");
    for (int f = 0; f < 6; ++f)
        if (!g->physical_face[f]) return set_err(c, LSM_ERR_UNSUPPORTED, "metrics need all faces physical");
    if (!x || !y || !z || !csi || !eta || !zet || !aj) return set_err(c, LSM_ERR_NULL, "array is NULL");
    void *dx, *dy, *dz, *dcsi, *deta, *dzet, *daj;
    Staging S(c);
    S.add(x, 8 * N, Staging::IN, &dx);
    S.add(y, 8 * N, Staging::IN, &dy);
    S.add(z, 8 * N, Staging::IN, &dz);
    S.add(csi, 24 * N, Staging::OUT, &dcsi);
    S.add(eta, 24 * N, Staging::OUT, &deta);
    S.add(zet, 24 * N, Staging::OUT, &dzet);
    S.add(aj, 8 * N, Staging::OUT, &daj);
    LSM_TRY(S.resolve());
    lsm::launch_metrics(dg, (const double*)dx, (const double*)dy, (const double*)dz, (double*)dcsi, (double*)deta,
                        (double*)dzet, (double*)daj, c->stream);
    LSM_TRY(after_launch(c));
    return S.finish();
}

}  // extern "C"

// ===================================================== allocation-free volume
// lsm_total_water_volume_noalloc: the TotalWaterVolume reduction for callers
// that must not allocate device memory themselves.  Its only scratch (the
// per-block partial sums, the four result words and the error flag) lives in
// one file-scope device array that every GPU loading this library holds
// until the process exits.
namespace {

// layout: [0, 32) result (VK, V2, VB, total); [32, 36) error flag;
//         [256, 256 + 24 * kNoAllocMaxBlocks) per-block partials (K, S, B)
constexpr size_t kNoAllocMaxBlocks = (size_t)LSM_NOALLOC_MAX_CELLS / 256;
constexpr size_t kNoAllocBytes = 256 + 24 * kNoAllocMaxBlocks;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[64] = {nullptr};  // device address of the array, per device

// Once per device, with that device current: the host-side name of a
// __device__ array is not a device address, so look the address up.
int noalloc_scratch(int dev, unsigned char** out) {
    if (dev < 0 || dev >= 64) return set_err(nullptr, LSM_ERR_NO_DEVICE, "device index too large");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaGetSymbolAddress(no-alloc scratch)");
        g_noalloc_ptr[dev] = (unsigned char*)p;
    }
    *out = g_noalloc_ptr[dev];
    return LSM_OK;
}

// Where a pointer lives: 0 plain host memory (unregistered or page-locked),
// 1 device or managed memory of GPU `dev`, -1 device or managed memory of
// another GPU (or an address the runtime cannot classify).
int classify_ptr(const void* p, int dev) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    if (at.type == cudaMemoryTypeUnregistered || at.type == cudaMemoryTypeHost) return 0;
    return at.device == dev ? 1 : -1;
}
bool is_device_ptr(const void* p, int dev) { return classify_ptr(p, dev) == 1; }

}  // namespace

extern "C" int lsm_total_water_volume_noalloc(const lsm_grid* g, const double* phi, const double* x,
                                              const double* y, const double* z, double* volumes, void* stream) {
    DevGrid dg;
    LSM_TRY(check_grid(nullptr, g, &dg));
    const long long ncell = (long long)((dg.ib - (dg.pf ? 1 : 0)) - dg.ia + 1) *
                            ((dg.jb - (dg.pr ? 1 : 0)) - dg.ja + 1) * ((dg.kb - (dg.pu ? 1 : 0)) - dg.ka + 1);
    if (ncell > (long long)LSM_NOALLOC_MAX_CELLS || (size_t)lsm::volume_partial_blocks(dg) > kNoAllocMaxBlocks)
        return set_err(nullptr, LSM_ERR_CAPACITY,
                       "grid has more cells than LSM_NOALLOC_MAX_CELLS; use lsm_total_water_volume");
    if (!phi || !x || !y || !z || !volumes) return set_err(nullptr, LSM_ERR_NULL, "array is NULL");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return set_err(nullptr, LSM_ERR_NO_DEVICE, "no CUDA device");
    }
    for (const double* a : {phi, x, y, z})
        if (!is_device_ptr(a, dev))
            return set_err(nullptr, LSM_ERR_MIXED_MEMORY, "inputs must be device arrays of the current GPU");
    const int vol_where = classify_ptr(volumes, dev);
    if (vol_where < 0)
        return set_err(nullptr, LSM_ERR_MIXED_MEMORY, "volumes must be host memory or device memory of the current GPU");
    unsigned char* base = nullptr;
    LSM_TRY(noalloc_scratch(dev, &base));
    cudaStream_t s = (cudaStream_t)stream;
    double* result = (double*)base;
    unsigned* err = (unsigned*)(base + 32);
    double* partials = (double*)(base + 256);
    // the array keeps the previous call's contents: only the error flag must start at zero
    LSM_CU(nullptr, cudaMemsetAsync(err, 0, sizeof(unsigned), s));
    lsm::launch_volume(dg, phi, x, y, z, partials, result, nullptr, nullptr, err, s);
    LSM_TRY(after_launch(nullptr));
    double res[4];
    unsigned flags = 0;
    const cudaMemcpyKind k = vol_where == 1 ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    LSM_CU(nullptr, cudaMemcpyAsync(k == cudaMemcpyDeviceToHost ? (void*)res : (void*)volumes, result,
                                    sizeof(res), k, s));
    LSM_CU(nullptr, cudaMemcpyAsync(&flags, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    LSM_CU(nullptr, cudaStreamSynchronize(s));
    if (k == cudaMemcpyDeviceToHost) std::memcpy(volumes, res, sizeof(res));
    if (flags & lsm::kErrNegativeVolume)
        return set_err(nullptr, LSM_ERR_NEGATIVE_VOLUME, "negative tetrahedron water volume");
    return LSM_OK;
}
