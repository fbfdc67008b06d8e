// lsm_batch_capi.cu -- host side of include/lsm_batch.h: packed device
// buffers of a batch of instances, the brick tables of the persistent
// kernels, the tile-shape autotuner and the CUDA graph of one physical step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lsm_batch.cuh"
#include "lsm_batch.h"
#include "lsm_c.h"
#include "lsm_kernels.h"

using lsm::batch::Fields;
using lsm::batch::Inst;

struct lsm_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int ninst = 0;
    std::vector<lsm_batch_instance> inst;
    lsm_batch_config cfg{};
    std::vector<long long> off;
    long long N = 0, nface = 0, max_inst_nodes = 0;
    Fields f{};
    float* bufs[6] = {};         // phi, stage0, stage1, d0, d1, sgn
    float* comps[15] = {};       // W[3], m[9], u[3]
    double* xyz = nullptr;       // 3*N FP64 coordinates
    double* staging = nullptr;   // FP64 scratch for input conversion (4 * max instance nodes)
    Inst* d_inst = nullptr;
    int* d_brick = nullptr;
    int nbricks = 0;
    double* d_part = nullptr;
    size_t part_cap = 0;
    double* d_vols = nullptr;
    double* h_vols = nullptr;    // pinned
    unsigned* d_err = nullptr;
    int shape = 0, grid = 0;
    bool tuned = false;
    cudaGraphExec_t exec = nullptr;
    std::string err;
};

namespace {

int fail(lsm_batch* b, int st, const std::string& m) {
    if (b) b->err = m;
    return st;
}
#define BCU(b, call)                                                                              \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail((b), LSM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct Dev {
    int prev = -1;
    explicit Dev(int d) { cudaGetDevice(&prev); if (prev != d) cudaSetDevice(d); }
    ~Dev() { int c = -1; cudaGetDevice(&c); if (prev >= 0 && c != prev) cudaSetDevice(prev); }
};

__global__ void k_cvt_f32(const double* __restrict__ src, int stride, int comp, long long n, float* __restrict__ dst) {
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n; l += (long long)gridDim.x * blockDim.x)
        dst[l] = (float)src[l * stride + comp];
}
__global__ void k_cvt_f64(const float* __restrict__ src, long long n, double* __restrict__ dst) {
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n; l += (long long)gridDim.x * blockDim.x)
        dst[l] = (double)src[l];
}

bool on_device(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// copy an FP64 array (host or device) of `n` doubles into the staging buffer
int stage_in(lsm_batch* b, const double* src, long long n) {
    BCU(b, cudaMemcpyAsync(b->staging, src, sizeof(double) * n,
                           on_device(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream));
    return LSM_OK;
}

void cvt(lsm_batch* b, int stride, int comp, long long n, float* dst) {
    lsm::ProfScope ps("k_cvt_f32", b->stream);
    k_cvt_f32<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 8), 256, 0, b->stream>>>(b->staging, stride,
                                                                                              comp, n, dst);
}

int build_bricks(lsm_batch* b, int shape) {
    const auto sh = lsm::batch::kShapes[shape];
    std::vector<Inst> hi(b->ninst);
    std::vector<int> brick;
    long long face = 0;
    for (int q = 0; q < b->ninst; ++q) {
        const auto& I = b->inst[q];
        Inst& d = hi[q];
        d.off = b->off[q];
        d.ni = I.ni; d.nj = I.nj; d.nk = I.nk;
        d.nbx = (I.ni + sh.tx - 1) / sh.tx;
        d.nby = (I.nj + sh.ty - 1) / sh.ty;
        const int nbz = (I.nk + sh.tz - 1) / sh.tz;
        d.brick0 = (int)brick.size();
        d.dt = (float)I.dt; d.dtau = (float)I.dtau; d.eps = (float)I.eps; d.pad = 0.f;
        d.face0 = face;
        d.cell0 = 0;
        face += 2LL * ((long long)I.nj * I.nk + (long long)I.ni * I.nk + (long long)I.ni * I.nj);
        brick.insert(brick.end(), (size_t)d.nbx * d.nby * nbz, q);
    }
    b->nface = face;
    b->nbricks = (int)brick.size();
    if (b->d_brick) cudaFree(b->d_brick);
    BCU(b, cudaMalloc(&b->d_brick, sizeof(int) * brick.size()));
    BCU(b, cudaMemcpyAsync(b->d_brick, brick.data(), sizeof(int) * brick.size(), cudaMemcpyHostToDevice, b->stream));
    BCU(b, cudaMemcpyAsync(b->d_inst, hi.data(), sizeof(Inst) * hi.size(), cudaMemcpyHostToDevice, b->stream));
    const size_t need = 3 * (size_t)b->nbricks;
    if (need > b->part_cap) {
        if (b->d_part) cudaFree(b->d_part);
        BCU(b, cudaMalloc(&b->d_part, sizeof(double) * need));
        b->part_cap = need;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const int per = std::max(1, lsm::batch::max_blocks_per_sm(shape, 0));
    b->grid = std::max(1, std::min(b->nbricks, sms * per));
    b->shape = shape;
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

// TVD-RK3 coefficients, src/ad_RKTVD3.F90:36-48
const float kC[3][3] = {{1.0f, 0.0f, 1.0f}, {0.75f, 0.25f, 0.25f}, {1.0f / 3.0f, 2.0f / 3.0f, 2.0f / 3.0f}};

// enqueue one physical step on b->stream
void enqueue_step(lsm_batch* b) {
    namespace B = lsm::batch;
    const int sh = b->shape, gr = b->grid, nb = b->nbricks;
    B::BC bc;
    for (int q = 0; q < 6; ++q) bc.type[q] = b->cfg.btype_lsm[q];
    bc.BigPhi = (float)b->cfg.BigPhi;
    Fields& f = b->f;
    B::volume(sh, gr, b->d_inst, b->d_brick, nb, f, f.phi, b->d_part, b->stream);
    B::volume_final(b->d_inst, b->ninst, b->d_brick, nb, b->d_part, b->d_vols, b->stream);
    float one[3] = {1.0f, 1.0f, 1.0f};
    B::contra(sh, gr, b->d_inst, b->d_brick, nb, f, one, b->stream);
    const float* in[3] = {f.phi, f.stage[0], f.stage[1]};
    float* out[3] = {f.stage[0], f.stage[1], f.stage[0]};
    for (int s = 0; s < 3; ++s) {
        B::stage(sh, gr, b->d_inst, b->d_brick, nb, f, f.phi, in[s], out[s], kC[s][0], kC[s][1], kC[s][2], b->stream);
        B::bc_stage(b->d_inst, b->ninst, b->nface, f, bc, f.phi, in[s], out[s], kC[s][0], kC[s][1], b->stream);
    }
    const float* cur = f.stage[0];
    if (b->cfg.RNitermax > 0) {
        B::sign(sh, gr, b->d_inst, b->d_brick, nb, f, f.stage[0], b->stream);
        for (int it = 0; it < b->cfg.RNitermax; ++it) {
            float* o = f.d[it & 1];
            B::reinit(sh, gr, b->d_inst, b->d_brick, nb, f, cur, o, b->stream);
            cur = o;
        }
    }
    B::bc_full(sh, gr, b->d_inst, b->d_brick, nb, bc, cur, f.phi, b->d_err, b->stream);
}

int autotune(lsm_batch* b) {
    namespace B = lsm::batch;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int best_shape = 0;
    for (int s = 0; s < B::kNumShapes; ++s) {
        int st = build_bricks(b, s);
        if (st) return st;
        B::sign(s, b->grid, b->d_inst, b->d_brick, b->nbricks, b->f, b->f.phi, b->stream);
        auto pass = [&]() {
            B::stage(s, b->grid, b->d_inst, b->d_brick, b->nbricks, b->f, b->f.phi, b->f.phi, b->f.stage[0], 1.f, 0.f,
                     1.f, b->stream);
            B::reinit(s, b->grid, b->d_inst, b->d_brick, b->nbricks, b->f, b->f.phi, b->f.d[0], b->stream);
        };
        pass();
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < 5; ++r) pass();
        cudaEventRecord(e1, b->stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0); cudaEventDestroy(e1);
            return fail(b, LSM_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) { best = ms; best_shape = s; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return build_bricks(b, best_shape);
}

int prepare(lsm_batch* b) {
    if (!b->tuned) {
        int st = b->cfg.autotune ? autotune(b) : build_bricks(b, std::min(std::max(b->cfg.shape, 0), 4));
        if (st) return st;
        b->tuned = true;
    }
    if (b->cfg.use_graph && !b->exec) {
        cudaGraph_t g = nullptr;
        BCU(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(b);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) return fail(b, LSM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(b, LSM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    return LSM_OK;
}

}  // namespace

extern "C" {

int lsm_batch_create(lsm_batch_handle* out, int device, void* stream, int ninst, const lsm_batch_instance* inst,
                     const lsm_batch_config* cfg) {
    if (!out || !inst || !cfg || ninst <= 0) return LSM_ERR_NULL;
    for (int q = 0; q < ninst; ++q)
        if (inst[q].ni < 4 || inst[q].nj < 4 || inst[q].nk < 4) return LSM_ERR_BAD_SHAPE;
    for (int f = 0; f < 6; ++f)
        if (cfg->btype_lsm[f] < 0 || cfg->btype_lsm[f] > 2) return LSM_ERR_BAD_PARAM;
    if (cfg->RNitermax < 0) return LSM_ERR_BAD_PARAM;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return LSM_ERR_NO_DEVICE;
    }
    auto* b = new lsm_batch();
    Dev guard(device);
    b->device = device;
    b->ninst = ninst;
    b->inst.assign(inst, inst + ninst);
    b->cfg = *cfg;
    if (stream) {
        b->stream = (cudaStream_t)stream;
    } else {
        cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        b->own_stream = true;
    }
    long long n = 0;
    for (int q = 0; q < ninst; ++q) {
        b->off.push_back(n);
        const long long nq = (long long)inst[q].ni * inst[q].nj * inst[q].nk;
        n += nq;
        b->max_inst_nodes = std::max(b->max_inst_nodes, nq);
    }
    b->N = n;
    auto cleanup = [&](int st) { lsm_batch_destroy(b); return st; };
    for (auto& p : b->bufs)
        if (cudaMalloc(&p, sizeof(float) * n) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    for (auto& p : b->comps)
        if (cudaMalloc(&p, sizeof(float) * n) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->xyz, sizeof(double) * 3 * n) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->staging, sizeof(double) * 4 * b->max_inst_nodes) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_inst, sizeof(Inst) * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_vols, sizeof(double) * 4 * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMallocHost(&b->h_vols, sizeof(double) * 4 * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_err, sizeof(unsigned)) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    cudaMemsetAsync(b->d_err, 0, sizeof(unsigned), b->stream);
    for (auto& p : b->bufs) cudaMemsetAsync(p, 0, sizeof(float) * n, b->stream);
    for (auto& p : b->comps) cudaMemsetAsync(p, 0, sizeof(float) * n, b->stream);
    cudaMemsetAsync(b->xyz, 0, sizeof(double) * 3 * n, b->stream);
    Fields& f = b->f;
    f.phi = b->bufs[0]; f.stage[0] = b->bufs[1]; f.stage[1] = b->bufs[2];
    f.d[0] = b->bufs[3]; f.d[1] = b->bufs[4]; f.sgn = b->bufs[5];
    for (int c = 0; c < 3; ++c) { f.W[c] = b->comps[c]; f.u[c] = b->comps[12 + c]; }
    for (int c = 0; c < 9; ++c) f.m[c] = b->comps[3 + c];
    for (int c = 0; c < 3; ++c) f.xyz[c] = b->xyz + c * n;
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    *out = b;
    return LSM_OK;
}

int lsm_batch_destroy(lsm_batch_handle b) {
    if (!b) return LSM_ERR_NULL;
    Dev guard(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (auto p : b->bufs) if (p) cudaFree(p);
    for (auto p : b->comps) if (p) cudaFree(p);
    if (b->xyz) cudaFree(b->xyz);
    if (b->staging) cudaFree(b->staging);
    if (b->d_inst) cudaFree(b->d_inst);
    if (b->d_brick) cudaFree(b->d_brick);
    if (b->d_part) cudaFree(b->d_part);
    if (b->d_vols) cudaFree(b->d_vols);
    if (b->h_vols) cudaFreeHost(b->h_vols);
    if (b->d_err) cudaFree(b->d_err);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return LSM_OK;
}

int lsm_batch_set_geometry(lsm_batch_handle b, int q, const double* x, const double* y, const double* z,
                           const double* csi, const double* eta, const double* zet) {
    if (!b || !x || !y || !z || !csi || !eta || !zet) return LSM_ERR_NULL;
    if (q < 0 || q >= b->ninst) return fail(b, LSM_ERR_BAD_PARAM, "instance index out of range");
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    const double* c3[3] = {x, y, z};
    for (int c = 0; c < 3; ++c)
        BCU(b, cudaMemcpyAsync(b->xyz + c * b->N + o, c3[c], sizeof(double) * n,
                               on_device(c3[c]) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream));
    const double* m3[3] = {csi, eta, zet};
    for (int d = 0; d < 3; ++d) {
        int st = stage_in(b, m3[d], 3 * n);
        if (st) return st;
        for (int c = 0; c < 3; ++c) cvt(b, 3, c, n, b->f.m[3 * d + c] + o);
    }
    BCU(b, cudaGetLastError());
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_set_velocity(lsm_batch_handle b, int q, const double* qv) {
    if (!b || !qv) return LSM_ERR_NULL;
    if (q < 0 || q >= b->ninst) return fail(b, LSM_ERR_BAD_PARAM, "instance index out of range");
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    int st = stage_in(b, qv, 4 * n);
    if (st) return st;
    for (int c = 0; c < 3; ++c) cvt(b, 4, c + 1, n, b->f.u[c] + o);
    BCU(b, cudaGetLastError());
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_set_phi(lsm_batch_handle b, int q, const double* phi) {
    if (!b || !phi) return LSM_ERR_NULL;
    if (q < 0 || q >= b->ninst) return fail(b, LSM_ERR_BAD_PARAM, "instance index out of range");
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    int st = stage_in(b, phi, n);
    if (st) return st;
    cvt(b, 1, 0, n, b->f.phi + o);
    BCU(b, cudaGetLastError());
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_get_phi(lsm_batch_handle b, int q, double* phi) {
    if (!b || !phi) return LSM_ERR_NULL;
    if (q < 0 || q >= b->ninst) return fail(b, LSM_ERR_BAD_PARAM, "instance index out of range");
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    {
        lsm::ProfScope ps("k_cvt_f64", b->stream);
        k_cvt_f64<<<(unsigned)std::min<long long>((n + 255) / 256, 152 * 8), 256, 0, b->stream>>>(b->f.phi + o, n,
                                                                                                 b->staging);
    }
    BCU(b, cudaGetLastError());
    BCU(b, cudaMemcpyAsync(phi, b->staging, sizeof(double) * n,
                           on_device(phi) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_step(lsm_batch_handle b, int nsteps, double* volumes) {
    if (!b) return LSM_ERR_NULL;
    if (nsteps < 0) return fail(b, LSM_ERR_BAD_PARAM, "negative step count");
    Dev guard(b->device);
    int st = prepare(b);
    if (st) return st;
    for (int s = 0; s < nsteps; ++s) {
        if (b->exec) {
            lsm::g_launches += (unsigned long long)lsm_batch_launches_per_step(b);
            BCU(b, cudaGraphLaunch(b->exec, b->stream));
        } else {
            enqueue_step(b);
        }
    }
    BCU(b, cudaGetLastError());
    unsigned flags = 0;
    BCU(b, cudaMemcpyAsync(&flags, b->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    if (volumes) BCU(b, cudaMemcpyAsync(b->h_vols, b->d_vols, sizeof(double) * 4 * b->ninst, cudaMemcpyDeviceToHost,
                                        b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    if (volumes) std::memcpy(volumes, b->h_vols, sizeof(double) * 4 * b->ninst);
    if (flags & lsm::kErrNonFinite) return fail(b, LSM_ERR_NONFINITE, "non-finite phi in the batch");
    return LSM_OK;
}

int lsm_batch_shape(lsm_batch_handle b, int* index, int* tx, int* ty, int* tz) {
    if (!b) return LSM_ERR_NULL;
    const auto sh = lsm::batch::kShapes[b->shape];
    if (index) *index = b->shape;
    if (tx) *tx = sh.tx;
    if (ty) *ty = sh.ty;
    if (tz) *tz = sh.tz;
    return LSM_OK;
}

long long lsm_batch_nodes(lsm_batch_handle b) { return b ? b->N : 0; }

int lsm_batch_launches_per_step(lsm_batch_handle b) {
    if (!b) return 0;
    return 2 + 1 + 6 + (b->cfg.RNitermax > 0 ? 1 + b->cfg.RNitermax : 0) + 1;
}

const char* lsm_batch_last_error(lsm_batch_handle b) { return b ? b->err.c_str() : ""; }

}  // extern "C"
