// lsm_batch_capi.cu -- host side of include/lsm_batch.h: packed device
// buffers of a batch of instances, the brick and tile tables of the
// persistent kernels, the autotuner (tile shape; brick or marching
// pseudo-steps), the CUDA graph of one physical step, the FP64 mass
// correction and the checkpointed adjoint (forward_record keeping the last
// segment's internals / backward).
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <initializer_list>
#include <type_traits>
#include <vector>

#include "lsm_batch.cuh"
#include "lsm_batch.h"
#include "lsm_c.h"
#include "lsm_kernels.h"

using lsm::batch::Flat;
using lsm::batch::Inst;
using lsm::batch::Mass;
template <typename T>
using FieldsT = lsm::batch::FieldsT<T>;

struct lsm_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int prec = 0;                // 0 FP32, 1 FP64
    size_t esz = 4;              // bytes per element of the scalar fields
    int ninst = 0;
    std::vector<lsm_batch_instance> inst;
    lsm_batch_config cfg{};
    std::vector<long long> off;  // ninst + 1 node offsets
    long long N = 0, nface = 0, max_inst_nodes = 0, nplane[3] = {0, 0, 0};
    // the adjoint reverses the two faces of axis a in one launch when every
    // instance has at least 6 nodes along a (their targets are then disjoint)
    bool face_pair[3] = {false, false, false};
    FieldsT<float> f32{};
    FieldsT<double> f64{};
    // Per-node arrays live in arenas with a stride between arrays that is a
    // 4 KiB multiple plus 2304 B, so that the same node of different arrays
    // does not fall on the same DRAM channel (power-of-two node counts would
    // otherwise put every array at a multiple of a large power of two).
    void* field_arena = nullptr; // bufs and comps
    size_t ld = 0;               // elements between consecutive arrays (batch precision)
    size_t ld8 = 0;              // the same for 8-byte arrays
    void* bufs[6] = {};          // phi, stage0, stage1, d0, d1, sgn
    void* comps[15] = {};        // W[3], m[9], u[3]
    double* xyz = nullptr;       // FP64 coordinates x, y, z (stride ld8); cellfix follows
    // FP32 batches: FP64 metrics (9), velocity (3) and contravariant velocity
    // x dt (3) for the stage nodes near the interface (stride ld8), their
    // device pointer table, and which instances have geometry / velocity set
    double* f64x = nullptr;
    double** d_p64 = nullptr;
    std::vector<char> geom_set, vel_set;
    long long* cellfix = nullptr;  // N fixed-point cell hexahedron volumes
    float* cellrel = nullptr;      // FP32 batches: 24 N floats, relative vertex coordinates per cell
    double* staging = nullptr;   // FP64 scratch for conversions (4 * max instance nodes)
    Inst* d_inst = nullptr;
    long long* d_offs = nullptr;
    lsm::batch::Brick* d_brick = nullptr;
    int nbricks = 0;
    lsm::batch::Brick* d_amap[4] = {};  // brick tables of the adjoint stencil kernels (lsm::batch::adj_shape)
    int namap[4] = {0, 0, 0, 0}, agrid[4] = {1, 1, 1, 1};
    int sgrid = 1, acgrid = 1, rzgrid = 1;   // CTAs of the map-2 kernels: stage, k_adj_reinit_c, reinit_z
    int vgrid = 1;                           // CTAs of the map-2 volume scan
    bool reinit_march = true;   // plain pseudo-steps march in k (reinit_z) rather than walk the brick table
    unsigned long long* d_vacc = nullptr;   // volume accumulators, 4 per instance
    unsigned* d_ilist = nullptr;            // interface cells of a volume pass (N entries) and their count
    unsigned* d_icount = nullptr;
    double* d_vols = nullptr;
    // mass correction: per-instance target volumes (NaN: none) and the last
    // step's correction; adjoint scratch (N fixed-point weights, one partial
    // per tile of adjoint map 2, one sum per instance)
    double* d_target = nullptr;
    Mass* d_mass = nullptr;
    unsigned long long* wfix = nullptr;
    double* d_tpart = nullptr;
    double* d_ssum = nullptr;
    double* h_vols = nullptr;    // pinned
    unsigned* d_err = nullptr;
    int shape = 0, grid = 0;
    bool tuned = false;
    // the contravariant velocity W = dt (metrics . u) depends only on the
    // geometry and the velocity: formed once after either changes
    bool w_stale = true;
    // TMA-staged RK stage (FP32, one instance, ni a multiple of 4): 4-D
    // tensor maps (ni, nj, nk, arrays) over the field arena and the adjoint
    // arena, whose arrays are ld elements apart
    bool tma_eligible = false, tma_stage = false, tma_adj = false;
    CUtensorMap tm_field{}, tm_adjmap{};
    int tgrid = 1;
    cudaGraphExec_t exec = nullptr;
    // adjoint state: one allocation, carved by adj_view
    int rec_steps = 0, rec_ck = 0;
    bool rec_live = false;   // the slots hold the last recorded segment's internals
    void* adj = nullptr;
    size_t adj_bytes = 0;
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
#define BTRY(x)              \
    do {                     \
        int st_ = (x);       \
        if (st_) return st_; \
    } while (0)

struct Dev {
    int prev = -1;
    explicit Dev(int d) {
        cudaGetDevice(&prev);
        if (prev != d) cudaSetDevice(d);
    }
    ~Dev() {
        int c = -1;
        cudaGetDevice(&c);
        if (prev >= 0 && c != prev) cudaSetDevice(prev);
    }
};

// Caller arrays are records of `stride` doubles per node in the reference's
// layout (a scalar field: stride 1; q(1:4, .): 4; csi(1:3, .): 3).  Each
// conversion is one pass over the records, all components at once.
// Components c0 .. c0 + nc - 1 of every record -> d[0 .. nc - 1] (type T),
// and to the FP64 arrays e[c] too where those are not null.
struct CvtDst {
    void* d[3];
    double* e[3];
};
template <typename T>
__global__ void k_cvt_in(const double* __restrict__ src, int stride, int c0, int nc, long long n, CvtDst o) {
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n;
         l += (long long)gridDim.x * blockDim.x) {
        const double* r = src + l * stride + c0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (c >= nc) break;
            const double v = r[c];
            static_cast<T*>(o.d[c])[l] = (T)v;
            if (o.e[c]) o.e[c][l] = v;
        }
    }
}
// src[0 .. nc - 1] (type T) -> components c0 .. c0 + nc - 1 of every record,
// the record's other components zero
struct CvtSrc {
    const void* s[3];
};
template <typename T>
__global__ void k_cvt_out(CvtSrc in, int stride, int c0, int nc, long long n, double* __restrict__ dst) {
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n;
         l += (long long)gridDim.x * blockDim.x) {
        double* r = dst + l * stride;
        for (int c = 0; c < stride; ++c) {
            const int k = c - c0;
            r[c] = k >= 0 && k < nc ? (double)static_cast<const T*>(in.s[k])[l] : 0.0;
        }
    }
}
// FP64 W of instance q once its FP64 geometry and velocity are both in place
void update_w64(lsm_batch* b, int q) {
    if (!b->f64x || !b->geom_set[q] || !b->vel_set[q]) return;
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk;
    lsm::batch::w64(b->off[q], n, I.dt, b->d_p64, b->d_p64 + 9, b->d_p64 + 12, b->stream);
}

template <typename T>
__global__ void k_zero(long long n, T* __restrict__ a) {
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n; l += (long long)gridDim.x * blockDim.x)
        a[l] = T(0);
}

inline unsigned cblocks(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 8)); }

// bytes between consecutive per-node arrays of n elements of esz bytes
size_t array_stride(long long n, size_t esz) {
    const size_t raw = (size_t)n * esz;
    return (raw + 4095) / 4096 * 4096 + 2304;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library)
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_tiled() {
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiled)p;
        else
            cudaGetLastError();
    }
    return fn;
}

// 4-D map (x, y, z, array) of `narrays` FP32 arrays of one instance, ld
// elements apart from `base`, box 40 x 12 x 1 x 1 (the stage's plane tile
// with its halo); false when the driver refuses it
bool encode_stage_map(const lsm_batch* b, void* base, long long narrays, CUtensorMap* out) {
    EncodeTiled fn = encode_tiled();
    if (!fn || narrays < 1) return false;
    const auto& I = b->inst[0];
    const cuuint64_t dim[4] = {(cuuint64_t)I.ni, (cuuint64_t)I.nj, (cuuint64_t)I.nk, (cuuint64_t)narrays};
    const cuuint64_t stride[3] = {(cuuint64_t)I.ni * 4, (cuuint64_t)I.ni * I.nj * 4, (cuuint64_t)b->ld * 4};
    const cuuint32_t box[4] = {40, 12, 1, 1}, estr[4] = {1, 1, 1, 1};
    return fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dim, stride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The address at which this batch's kernels can use a caller's array in
// place: memory of the batch's device, or page-locked host memory registered
// on that device (its mapped alias; the conversion kernels then read and
// write it across the host link).  nullptr for anything else (pageable host
// memory, another device's memory), which goes through the staging buffer
// by a copy.  After long kernels over most of HBM the first transfer of a
// host array pays for its page translations again; many SMs take those
// misses in parallel, a copy engine does not (measured on GB300: 5-10 ms
// against 17-31 ms for 268 MB; 1.3 ms either way once warm).
double* kernel_view(const lsm_batch* b, const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.device != b->device) return nullptr;
    if (a.type == cudaMemoryTypeDevice) return static_cast<double*>(const_cast<void*>(p));
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return static_cast<double*>(a.devicePointer);
    return nullptr;
}

// n records of the caller's `src` -> components c0 .. c0 + nc - 1 into
// o.d (the batch's type, or FP64 with `f64`) and o.e
int load_in(lsm_batch* b, const double* src, long long n, int stride, int c0, int nc, CvtDst o, bool f64 = false) {
    const double* v = kernel_view(b, src);
    if (!v) {
        BCU(b, cudaMemcpyAsync(b->staging, src, sizeof(double) * n * stride, cudaMemcpyDefault, b->stream));
        v = b->staging;
    }
    lsm::ProfScope ps("k_cvt_in", b->stream);
    if (f64 || b->prec) k_cvt_in<double><<<cblocks(n), 256, 0, b->stream>>>(v, stride, c0, nc, n, o);
    else k_cvt_in<float><<<cblocks(n), 256, 0, b->stream>>>(v, stride, c0, nc, n, o);
    BCU(b, cudaGetLastError());
    return LSM_OK;
}
// the batch's arrays `in` -> n records of the caller's `dst` (components c0
// .. c0 + nc - 1; the others zero); with `wait`, returns once dst holds them
int store_out(lsm_batch* b, double* dst, long long n, int stride, int c0, int nc, CvtSrc in, bool wait = true) {
    double* v = kernel_view(b, dst);
    {
        lsm::ProfScope ps("k_cvt_out", b->stream);
        if (b->prec) k_cvt_out<double><<<cblocks(n), 256, 0, b->stream>>>(in, stride, c0, nc, n, v ? v : b->staging);
        else k_cvt_out<float><<<cblocks(n), 256, 0, b->stream>>>(in, stride, c0, nc, n, v ? v : b->staging);
    }
    BCU(b, cudaGetLastError());
    if (!v) BCU(b, cudaMemcpyAsync(dst, b->staging, sizeof(double) * n * stride, cudaMemcpyDefault, b->stream));
    if (wait) BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int build_bricks(lsm_batch* b, int shape) {
    if (b->prec) shape = 0;     // FP64 kernels exist for tile shape 0 only
    const auto sh = lsm::batch::kShapes[shape];
    std::vector<Inst> hi(b->ninst);
    using lsm::batch::Brick;
    std::vector<Brick> brick, amap[4];
    // bricks in x-fastest order, each with its instance and coordinates
    auto add = [](std::vector<Brick>& v, int q, int bx, int by, int bz) {
        for (int z = 0; z < bz; ++z)
            for (int y = 0; y < by; ++y)
                for (int x = 0; x < bx; ++x) v.push_back(Brick{q, x, y, z});
    };
    long long face = 0, pre[3] = {0, 0, 0};
    for (int q = 0; q < b->ninst; ++q) {
        const auto& I = b->inst[q];
        Inst& d = hi[q];
        d.off = b->off[q];
        d.ni = I.ni;
        d.nj = I.nj;
        d.nk = I.nk;
        d.nbx = (I.ni + sh.tx - 1) / sh.tx;
        d.nby = (I.nj + sh.ty - 1) / sh.ty;
        const int nbz = (I.nk + sh.tz - 1) / sh.tz;
        d.brick0 = (int)brick.size();
        d.dt = (float)I.dt;
        d.dtau = (float)I.dtau;
        d.eps = (float)I.eps;
        d.pad = 0.f;
        d.dt64 = I.dt;
        d.dtau64 = I.dtau;
        d.eps64 = I.eps;
        d.face0 = face;
        face += 2LL * ((long long)I.nj * I.nk + (long long)I.ni * I.nk + (long long)I.ni * I.nj);
        for (int a = 0; a < 3; ++a) d.fpre[a] = pre[a];
        for (int m = 0; m < 4; ++m) {
            const auto a = lsm::batch::adj_shape(m);
            const int bx = a.ox > 0 ? (I.ni + a.ox - 1) / a.ox : 1;
            const int by = (I.nj + a.oy - 1) / a.oy, bz = (I.nk + a.oz - 1) / a.oz;
            d.am[m][0] = (int)amap[m].size();
            d.am[m][1] = bx;
            d.am[m][2] = by;
            add(amap[m], q, bx, by, bz);
        }
        pre[0] += (long long)I.nj * I.nk;
        pre[1] += (long long)I.ni * I.nk;
        pre[2] += (long long)I.ni * I.nj;
        add(brick, q, d.nbx, d.nby, nbz);
    }
    b->nface = face;
    for (int a = 0; a < 3; ++a) b->nplane[a] = pre[a];
    b->nbricks = (int)brick.size();
    if (b->d_brick) {
        cudaStreamSynchronize(b->stream);
        cudaFree(b->d_brick);
        b->d_brick = nullptr;
    }
    for (int m = 0; m < 4; ++m) {
        if (b->d_amap[m]) {
            cudaFree(b->d_amap[m]);
            b->d_amap[m] = nullptr;
        }
        b->namap[m] = (int)amap[m].size();
        BCU(b, cudaMalloc(&b->d_amap[m], sizeof(Brick) * amap[m].size()));
        BCU(b, cudaMemcpyAsync(b->d_amap[m], amap[m].data(), sizeof(Brick) * amap[m].size(), cudaMemcpyHostToDevice,
                               b->stream));
    }
    BCU(b, cudaMalloc(&b->d_brick, sizeof(Brick) * brick.size()));
    BCU(b, cudaMemcpyAsync(b->d_brick, brick.data(), sizeof(Brick) * brick.size(), cudaMemcpyHostToDevice, b->stream));
    BCU(b, cudaMemcpyAsync(b->d_inst, hi.data(), sizeof(Inst) * hi.size(), cudaMemcpyHostToDevice, b->stream));
    if (!b->d_vacc) {
        BCU(b, cudaMalloc(&b->d_vacc, sizeof(unsigned long long) * 4 * (size_t)b->ninst));
        BCU(b, cudaMemsetAsync(b->d_vacc, 0, sizeof(unsigned long long) * 4 * (size_t)b->ninst, b->stream));
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const int per = std::max(1, lsm::batch::max_blocks_per_sm(shape, 0));
    b->grid = std::max(1, std::min(b->nbricks, sms * per));
    for (int m = 0; m < 4; ++m) {
        const int pa = std::max(1, b->prec ? lsm::batch::adj_blocks_per_sm<double>(m)
                                           : lsm::batch::adj_blocks_per_sm<float>(m));
        b->agrid[m] = std::max(1, std::min(b->namap[m], sms * pa));
    }
    const int ps = std::max(1, b->prec ? lsm::batch::stage_blocks_per_sm<double>()
                                       : lsm::batch::stage_blocks_per_sm<float>());
    b->sgrid = std::max(1, std::min(b->namap[2], sms * ps));
    const int pac = std::max(1, b->prec ? lsm::batch::adj_reinit_c_blocks_per_sm<double>()
                                        : lsm::batch::adj_reinit_c_blocks_per_sm<float>());
    b->acgrid = std::max(1, std::min(b->namap[2], sms * pac));
    const int prz = std::max(1, b->prec ? lsm::batch::reinit_z_blocks_per_sm<double>()
                                        : lsm::batch::reinit_z_blocks_per_sm<float>());
    b->rzgrid = std::max(1, std::min(b->namap[2], sms * prz));
    const int pv = std::max(1, b->prec ? lsm::batch::vol_scan_blocks_per_sm<double>()
                                       : lsm::batch::vol_scan_blocks_per_sm<float>());
    b->vgrid = std::max(1, std::min(b->namap[2], sms * pv));
    if (b->tma_eligible)
        b->tgrid = std::max(1, std::min(b->namap[2], sms * std::max(1, lsm::batch::stage_tma_blocks_per_sm())));
    b->shape = shape;
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

// TVD-RK3 stage coefficients (c1, c2, c3): out = c1 phi^n + c2 in - c3 dt aj RH,
// src/ad_RKTVD3.F90:36-48
// (double here; each kernel takes them in its own precision)
const double kC[3][3] = {{1.0, 0.0, 1.0}, {0.75, 0.25, 0.25}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};

lsm::batch::BC make_bc(const lsm_batch* b) {
    lsm::batch::BC bc;
    for (int q = 0; q < 6; ++q) bc.type[q] = b->cfg.btype_lsm[q];
    bc.BigPhi = (float)b->cfg.BigPhi;
    return bc;
}

template <typename T>
FieldsT<T>& fields(lsm_batch* b);
template <>
FieldsT<float>& fields<float>(lsm_batch* b) { return b->f32; }
template <>
FieldsT<double>& fields<double>(lsm_batch* b) { return b->f64; }

// Recorded internals of one step (adjoint): the three stage outputs and
//   adjoint_mode 0: the raw last pseudo-step output (D) and each
//                   pseudo-step's adjoint coefficients (C + 6 k ld);
//   adjoint_mode 1: the RNitermax raw pseudo-step outputs (D + k ld) and
//                   the sign field.
//   with the mass correction, P: the step's result before the correction.
template <typename T>
struct Rec {
    T* A[3];
    T* D;
    T* sgn;   // mode 1 only
    T* C;     // mode 0 only
    T* P;     // mass correction only
    unsigned* list;    // mass correction only: the interface cells of P (the step's volume pass)
    unsigned* count;   // and their number
};

// raw output of pseudo-step k of a recorded step (mode 1: every k; mode 0:
// the last one only)
template <typename T>
T* rec_d(const lsm_batch* b, const Rec<T>& r, int k) {
    return b->cfg.adjoint_mode == 0 ? r.D : r.D + (long long)k * (long long)b->ld;
}

// One RK stage: the TMA-staged kernel when the batch uses it and the input
// is an array of a mapped arena, else the shared-memory-staged one.
template <typename T>
void enqueue_stage(lsm_batch* b, FieldsT<T> f, const T* phin, const T* in, T* out, int s) {
    namespace B = lsm::batch;
    if constexpr (sizeof(T) == 4) {
        if (b->tma_stage) {
            const char* p = (const char*)in;
            const size_t row = b->ld * sizeof(float);
            const CUtensorMap* map = nullptr;
            long long a = -1;
            const char* fb = (const char*)b->field_arena;
            if (p >= fb && p < fb + row * 21 && (size_t)(p - fb) % row == 0) {
                map = &b->tm_field;
                a = (long long)((size_t)(p - fb) / row);
            } else if (b->tma_adj && b->adj) {
                const char* ab = (const char*)b->adj;
                if (p >= ab && p < ab + b->adj_bytes && (size_t)(p - ab) % row == 0) {
                    map = &b->tm_adjmap;
                    a = (long long)((size_t)(p - ab) / row);
                }
            }
            if (map && a < (1LL << 31)) {
                B::stage_tma(b->tgrid, map, (int)a, b->d_inst, b->d_amap[2], b->namap[2], f, phin, in, out, kC[s][0],
                             kC[s][1], kC[s][2], b->d_err, b->stream);
                return;
            }
        }
    }
    B::stage<T>(b->sgrid, b->d_inst, b->d_amap[2], b->namap[2], f, phin, in, out, kC[s][0], kC[s][1], kC[s][2],
                b->stream);
}

// One physical step phin -> phi_out (phi_out may alias phin; nullptr skips
// the final bcond_lsm).  With `rec` the stage outputs, the pseudo-step
// outputs (before the final bcond_lsm) and the sign field are kept; `vol`
// adds the pre-advection water volume; a recorded step checks phi_out for
// non-finite values when `check` (plain steps always do).
// With the mass correction the volume pass moves after the final bcond_lsm:
// it measures the step's result (the slot's P in a recorded step, which is
// then kept even when phi_out is nullptr), forms the correction (into mrec
// too when given) and phi_out = result + C.
template <typename T>
void enqueue_step_io(lsm_batch* b, const T* phin, T* phi_out, const Rec<T>* rec, bool vol, bool check = false,
                     Mass* mrec = nullptr) {
    namespace B = lsm::batch;
    const int sh = b->shape, gr = b->grid, nb = b->nbricks;
    const B::BC bc = make_bc(b);
    FieldsT<T> f = fields<T>(b);
    const bool mc = b->cfg.mass_correction != 0;
    const bool coef = rec && b->cfg.adjoint_mode == 0;   // recorded step storing adjoint coefficients
    if (rec && !coef) f.sgn = rec->sgn;
    const Flat fl{b->d_inst, b->d_offs, b->ninst, b->N};
    if (vol && !mc) {
        B::volume<T>(b->vgrid, b->d_inst, b->d_amap[2], b->namap[2], fl, f, phin, b->d_vacc, false, b->d_ilist,
                     b->d_icount, b->stream);
        B::volume_final(b->ninst, b->d_vacc, b->d_vols, nullptr, nullptr, nullptr, b->stream);
    }
    // the field the final bcond_lsm writes
    T* res = mc && rec ? rec->P : phi_out;
    T* S[3] = {rec ? rec->A[0] : f.stage[0], rec ? rec->A[1] : f.stage[1], rec ? rec->A[2] : f.stage[0]};
    const T* in[3] = {phin, S[0], S[1]};
    for (int s = 0; s < 3; ++s) {
        enqueue_stage<T>(b, f, phin, in[s], S[s], s);
        B::bc_stage<T>(b->d_inst, b->ninst, b->nface, bc, phin, in[s], S[s], kC[s][0], kC[s][1], b->stream);
    }
    const int R = b->cfg.RNitermax;
    if (R > 0) {
        // reinitialization (src/reinitialization.F90:55-104); the last
        // pseudo-step writes phi and gets the final bcond_lsm
        // (src/levelsetmethod.F90:318-321)
        // the sign field and the first pseudo-step in one pass, then one
        // launch per pseudo-step
        const T* cur = S[2];
        bool twice = false;
        for (int it = 0; it < R; ++it) {
            const bool last = it == R - 1;
            T* o = coef ? (last ? rec->D : f.d[it & 1]) : rec ? rec_d(b, *rec, it) : (last ? res : f.d[it & 1]);
            const bool march = coef || b->reinit_march;
            // a recorded step's last pseudo-step also writes phi^{n+1} (its
            // faces are then redone from the raw output)
            T* o2 = rec && last && res && march ? res : nullptr;
            twice = twice || o2 != nullptr;
            unsigned* err = (last && !rec) || (o2 && check) ? b->d_err : nullptr;
            T* cf = coef ? rec->C + 6LL * it * (long long)b->ld : nullptr;
            if (march)
                B::reinit_z<T>((it == 0 ? 2 : 0) + (coef ? 1 : 0), b->rzgrid, b->d_inst, b->d_amap[2], b->namap[2], f,
                               cur, o, o2, cf, (long long)b->ld, err, b->stream);
            else if (it == 0)
                B::sign_reinit<T>(sh, gr, b->d_inst, b->d_brick, nb, f, cur, o, err, b->stream);
            else
                B::reinit<T>(sh, gr, b->d_inst, b->d_brick, nb, f, cur, o, err, b->stream);
            if (last && !rec) B::bc_reinit<T>(b->d_inst, b->ninst, b->nface, f, bc, cur, res, b->stream);
            cur = o;
        }
        // recorded steps keep the raw last pseudo-step and write phi^{n+1} apart
        if (rec && res && twice)
            B::bc_faces<T>(b->d_inst, b->ninst, b->nface, bc, cur, res, check ? b->d_err : nullptr, b->stream);
        else if (rec && res)
            B::bc_full<T>(sh, gr, b->d_inst, b->d_brick, nb, bc, cur, res, check ? b->d_err : nullptr, b->stream);
    } else if (res) {
        B::bc_full<T>(sh, gr, b->d_inst, b->d_brick, nb, bc, S[2], res, rec && !check ? nullptr : b->d_err,
                      b->stream);
    }
    if (mc) {
        // FP64 water volume of the result, the correction C = (target - V) / A
        // and phi_out = result + C
        // a recorded step keeps the interface cells of its result for the
        // reverse of the correction
        B::volume<T>(b->vgrid, b->d_inst, b->d_amap[2], b->namap[2], fl, f, res, b->d_vacc, true,
                     rec ? rec->list : b->d_ilist, rec ? rec->count : b->d_icount, b->stream);
        B::volume_final(b->ninst, b->d_vacc, b->d_vols, b->d_target, b->d_mass, mrec, b->stream);
        if (phi_out) B::mass_shift<T>(fl, b->d_mass, res, phi_out, b->stream);
    }
}

void enqueue_step(lsm_batch* b) {
    if (b->prec) enqueue_step_io<double>(b, b->f64.phi, b->f64.phi, nullptr, true);
    else enqueue_step_io<float>(b, b->f32.phi, b->f32.phi, nullptr, true);
}

// W of every instance from the current metrics and velocity (the steps
// read it; set_geometry / set_velocity mark it stale)
int refresh_w(lsm_batch* b) {
    if (!b->w_stale) return LSM_OK;
    if (b->prec) lsm::batch::contra<double>(b->shape, b->grid, b->d_inst, b->d_brick, b->nbricks, b->f64, b->stream);
    else lsm::batch::contra<float>(b->shape, b->grid, b->d_inst, b->d_brick, b->nbricks, b->f32, b->stream);
    BCU(b, cudaGetLastError());
    b->w_stale = false;
    return LSM_OK;
}

// Chooses the tile shape of the brick-table kernels and whether the plain
// pseudo-steps march in k (reinit_z) or walk the brick table: times, on
// the batch itself, the brick pseudo-steps for every shape and the marching
// pseudo-steps once (the per-step kernels that depend on the choice).
int autotune(lsm_batch* b) {
    namespace B = lsm::batch;
    cudaEvent_t ev[3];
    for (auto& e : ev) cudaEventCreate(&e);
    auto done = [&](int st) {
        for (auto& e : ev) cudaEventDestroy(e);
        return st;
    };
    FieldsT<float>& f = b->f32;
    auto timed = [&](float* ms_a, float* ms_b, auto&& pa, auto&& pb) -> int {
        pa();
        pb();
        cudaEventRecord(ev[0], b->stream);
        for (int r = 0; r < 5; ++r) pa();
        cudaEventRecord(ev[1], b->stream);
        for (int r = 0; r < 5; ++r) pb();
        cudaEventRecord(ev[2], b->stream);
        const cudaError_t e = cudaEventSynchronize(ev[2]);
        if (e != cudaSuccess) return fail(b, LSM_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
        cudaEventElapsedTime(ms_a, ev[0], ev[1]);
        cudaEventElapsedTime(ms_b, ev[1], ev[2]);
        return LSM_OK;
    };
    float br[B::kNumShapes], zm = 0.f, dummy = 0.f;
    for (int s = 0; s < B::kNumShapes; ++s) {
        const int bs = build_bricks(b, s);
        if (bs != LSM_OK) return done(bs);
        const int st = timed(
            &dummy, &br[s], [&]() {},
            [&]() {
                B::sign_reinit<float>(s, b->grid, b->d_inst, b->d_brick, b->nbricks, f, f.phi, f.d[0], nullptr,
                                      b->stream);
                B::reinit<float>(s, b->grid, b->d_inst, b->d_brick, b->nbricks, f, f.d[0], f.d[1], nullptr, b->stream);
            });
        if (st != LSM_OK) return done(st);
    }
    // the marching pseudo-steps do not depend on the brick shape
    const int st = timed(&dummy, &zm, [&]() {}, [&]() {
        B::reinit_z<float>(2, b->rzgrid, b->d_inst, b->d_amap[2], b->namap[2], f, f.phi, f.d[0], nullptr, nullptr, 0,
                           nullptr, b->stream);
        B::reinit_z<float>(0, b->rzgrid, b->d_inst, b->d_amap[2], b->namap[2], f, f.d[0], f.d[1], nullptr, nullptr, 0,
                           nullptr, b->stream);
    });
    if (st != LSM_OK) return done(st);
    int best_b = 0;
    for (int s = 1; s < B::kNumShapes; ++s)
        if (br[s] < br[best_b]) best_b = s;
    b->reinit_march = zm < br[best_b];
    const int bs = build_bricks(b, best_b);
    if (bs != LSM_OK) return done(bs);
    // the RK stage: plane tiles staged by TMA copies or by the threads,
    // timed on this batch's contravariant velocity (its upwind choices)
    if (b->tma_eligible) {
        const int sw = refresh_w(b);
        if (sw != LSM_OK) return done(sw);
        float ms_plain = 0.f, ms_tma = 0.f;
        const int st2 = timed(
            &ms_plain, &ms_tma,
            [&]() {
                B::stage<float>(b->sgrid, b->d_inst, b->d_amap[2], b->namap[2], f, f.phi, f.phi, f.stage[0], 1.0, 0.0,
                                1.0, b->stream);
            },
            [&]() {
                B::stage_tma(b->tgrid, &b->tm_field, 0, b->d_inst, b->d_amap[2], b->namap[2], f, f.phi, f.phi,
                             f.stage[0], 1.0, 0.0, 1.0, b->d_err, b->stream);
            });
        if (st2 != LSM_OK) return done(st2);
        b->tma_stage = ms_tma < ms_plain;
    }
    return done(LSM_OK);
}

// LSM_BATCH_STAGE=tma or =smem forces the RK stage kernel (tests,
// measurements); otherwise the autotuner times both (when the batch is
// eligible for the TMA one), and without autotuning the TMA one is used
// where eligible.
int stage_override() {
    const char* e = std::getenv("LSM_BATCH_STAGE");
    if (!e) return -1;
    if (!std::strcmp(e, "tma")) return 1;
    if (!std::strcmp(e, "smem")) return 0;
    return -1;
}


int prepare(lsm_batch* b) {
    if (!b->tuned) {
        const bool tune = b->cfg.autotune && !b->prec;
        if (tune) {
            BTRY(autotune(b));
        } else {
            // shape 0..4: that tile shape, pseudo-steps on the brick table;
            // 5: tile shape 0, pseudo-steps marching in k
            const int sh = std::min(std::max(b->cfg.shape, 0), 5);
            BTRY(build_bricks(b, sh == 5 ? 0 : sh));
            b->reinit_march = sh == 5;
            b->tma_stage = b->tma_eligible;
        }
        const int ov = stage_override();
        if (ov >= 0) b->tma_stage = ov == 1 && b->tma_eligible;
        b->tuned = true;
    }
    BTRY(refresh_w(b));
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

int run_steps(lsm_batch* b, int nsteps) {
    for (int s = 0; s < nsteps; ++s) {
        if (b->exec) {
            lsm::g_launches += (unsigned long long)lsm_batch_launches_per_step(b);
            BCU(b, cudaGraphLaunch(b->exec, b->stream));
        } else {
            enqueue_step(b);
        }
    }
    return LSM_OK;
}

int check_inst(lsm_batch* b, int q) {
    if (q < 0 || q >= b->ninst) return fail(b, LSM_ERR_BAD_PARAM, "instance index out of range");
    return LSM_OK;
}

// ------------------------------------------------------------ adjoint state
// Checkpoints (nck arrays), segment states (ck), the recorded internals of
// every step of a segment (ck slots, Rec), adjoint fields lam, lam2,
// lamPhin (3), lamW (3), lam_u (3); arrays b->ld apart.
template <typename T>
struct AdjView {
    T *ckpt, *seg, *slots, *lam, *lam2, *lamPhin, *lamW[3], *lamU[3];
    Mass* mrec;   // mass correction of every step of the segment, ninst per step
    unsigned* lcount;   // interface-cell count of every step of the segment (Rec::count)
};

int n_ckpt(int nsteps, int ck) { return (nsteps + ck - 1) / ck; }
// arrays of one recorded step, each b->ld elements apart
long long slot_elems(const lsm_batch* b) {
    const long long R = b->cfg.RNitermax;
    // with the mass correction: the pre-correction field P and the interface
    // cells of P (32-bit node indices, one array)
    return ((b->cfg.adjoint_mode == 0 ? 4 + 6 * R : 4 + R) + (b->cfg.mass_correction ? 2 : 0)) * (long long)b->ld;
}

size_t adj_elems(const lsm_batch* b, int nsteps, int ck) {
    // the recorded steps' mass states, then their interface-cell counts
    const size_t mrec =
        ((size_t)ck * (size_t)b->ninst * sizeof(Mass) + (size_t)ck * sizeof(unsigned) + b->esz - 1) / b->esz;
    return b->ld * (size_t)(n_ckpt(nsteps, ck) + ck + 3 + 3 + 3) + (size_t)ck * (size_t)slot_elems(b) + mrec;
}

template <typename T>
Rec<T> slot(lsm_batch* b, const AdjView<T>& v, int q) {
    const long long L = (long long)b->ld;
    T* p = v.slots + (long long)q * slot_elems(b);
    Rec<T> r;
    for (int s = 0; s < 3; ++s) r.A[s] = p + s * L;
    r.D = p + 3 * L;
    if (b->cfg.adjoint_mode == 0) {
        r.C = p + 4 * L;
        r.sgn = nullptr;
    } else {
        r.C = nullptr;
        r.sgn = p + (3 + b->cfg.RNitermax) * L;
    }
    r.P = b->cfg.mass_correction ? p + slot_elems(b) - 2 * L : nullptr;
    r.list = b->cfg.mass_correction ? reinterpret_cast<unsigned*>(p + slot_elems(b) - L) : nullptr;
    r.count = b->cfg.mass_correction ? v.lcount + q : nullptr;
    return r;
}

template <typename T>
AdjView<T> adj_view(lsm_batch* b) {
    AdjView<T> v;
    const long long N = (long long)b->ld;
    T* p = (T*)b->adj;
    v.ckpt = p;
    p += (long long)n_ckpt(b->rec_steps, b->rec_ck) * N;
    v.seg = p;
    p += (long long)b->rec_ck * N;
    v.slots = p;
    p += (long long)b->rec_ck * slot_elems(b);
    v.lam = p;
    p += N;
    v.lam2 = p;
    p += N;
    v.lamPhin = p;
    p += N;
    for (int c = 0; c < 3; ++c) {
        v.lamW[c] = p;
        p += N;
    }
    for (int c = 0; c < 3; ++c) {
        v.lamU[c] = p;
        p += N;
    }
    v.mrec = (Mass*)p;   // arrays are multiples of 256 bytes apart
    v.lcount = reinterpret_cast<unsigned*>(v.mrec + (long long)b->rec_ck * b->ninst);
    return v;
}

template <typename T>
int forward_record_t(lsm_batch* b, int nsteps, int ck) {
    ck = std::min(ck, nsteps);   // one segment either way: no slots beyond the recorded steps
    const size_t bytes = adj_elems(b, nsteps, ck) * sizeof(T);
    if (bytes > b->adj_bytes) {
        if (b->adj) {
            cudaStreamSynchronize(b->stream);
            cudaFree(b->adj);
            b->adj = nullptr;
            b->adj_bytes = 0;
        }
        BCU(b, cudaMalloc(&b->adj, bytes));
        b->adj_bytes = bytes;
        b->tma_adj = b->tma_eligible &&
                     encode_stage_map(b, b->adj, (long long)(bytes / (b->ld * sizeof(float))), &b->tm_adjmap);
    }
    if (b->cfg.mass_correction && !b->wfix) {
        // adjoint scratch of the mass correction (the weights start at zero
        // and every reverse step leaves them at zero)
        BCU(b, cudaMalloc(&b->wfix, sizeof(unsigned long long) * (size_t)b->N));
        BCU(b, cudaMemsetAsync(b->wfix, 0, sizeof(unsigned long long) * (size_t)b->N, b->stream));
        BCU(b, cudaMalloc(&b->d_tpart, sizeof(double) * (size_t)std::max(1, b->namap[2])));
        BCU(b, cudaMalloc(&b->d_ssum, sizeof(double) * (size_t)b->ninst));
    }
    b->rec_steps = nsteps;
    b->rec_ck = ck;
    b->rec_live = false;
    AdjView<T> v = adj_view<T>(b);
    FieldsT<T>& f = fields<T>(b);
    const long long LD = (long long)b->ld;
    BCU(b, cudaMemsetAsync(v.lam, 0, sizeof(T) * b->N, b->stream));
    // every segment but the last: plain steps (graph) from a checkpoint
    const int nseg = n_ckpt(nsteps, ck), c_last = (nseg - 1) * ck;
    for (int n = 0; n < c_last; ++n) {
        if (n % ck == 0)
            BCU(b, cudaMemcpyAsync(v.ckpt + (long long)(n / ck) * LD, f.phi, sizeof(T) * b->N,
                                   cudaMemcpyDeviceToDevice, b->stream));
        BTRY(run_steps(b, 1));
    }
    // the last segment keeps its internals in the slots, so that the reverse
    // sweep starts there without recomputing it (the same steps, volumes and
    // non-finite check as plain steps)
    BCU(b, cudaMemcpyAsync(v.ckpt + (long long)(nseg - 1) * LD, f.phi, sizeof(T) * b->N, cudaMemcpyDeviceToDevice,
                           b->stream));
    BCU(b, cudaMemcpyAsync(v.seg, f.phi, sizeof(T) * b->N, cudaMemcpyDeviceToDevice, b->stream));
    const int L = nsteps - c_last;
    for (int q = 0; q < L; ++q) {
        const Rec<T> r = slot<T>(b, v, q);
        enqueue_step_io<T>(b, v.seg + (long long)q * LD, q + 1 < L ? v.seg + (long long)(q + 1) * LD : f.phi, &r,
                           true, true, v.mrec + (long long)q * b->ninst);
    }
    BCU(b, cudaGetLastError());
    unsigned flags = 0;
    BCU(b, cudaMemcpyAsync(&flags, b->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    if (flags & lsm::kErrTimeout) return fail(b, LSM_ERR_CUDA, "a TMA copy of the RK stage did not complete");
    if (flags & lsm::kErrNonFinite) return fail(b, LSM_ERR_NONFINITE, "non-finite phi in the batch");
    b->rec_live = true;
    return LSM_OK;
}

// Reverse of one physical step from its recorded internals `r`; on entry
// lam holds the adjoint of phi^{n+1}, on exit the adjoint of phi^n (the
// pointers of `v` swap along the way).
template <typename T>
void adj_step(lsm_batch* b, AdjView<T>& v, const Rec<T>& r, const T* phin, const Mass* m) {
    namespace B = lsm::batch;
    FieldsT<T> f = fields<T>(b);
    if (r.sgn) f.sgn = r.sgn;
    const B::BC bc = make_bc(b);
    const long long N = b->N;
    const Flat fl{b->d_inst, b->d_offs, b->ninst, N};
    const int R = b->cfg.RNitermax;
    // reverse of the mass correction phi^{n+1} = P + C(P), in place on lam
    if (b->cfg.mass_correction)
        B::mass_adjoint<T>(b->d_inst, b->d_amap[2], b->namap[2], fl, f, r.P, m, v.lam, b->wfix, b->d_tpart,
                           b->d_ssum, r.list, r.count, b->stream);
    auto faces = [&](int kind, const T* pn, const T* in, const T* out, double c1, double c2) {
        for (int ax = 2; ax >= 0; --ax) {
            if (b->face_pair[ax]) {
                B::adj_face<T>(fl, 2 * ax + 1, b->nplane[ax], 2, bc, kind, pn, in, out, c1, c2, v.lam, b->stream);
            } else {
                B::adj_face<T>(fl, 2 * ax + 1, b->nplane[ax], 1, bc, kind, pn, in, out, c1, c2, v.lam, b->stream);
                B::adj_face<T>(fl, 2 * ax, b->nplane[ax], 1, bc, kind, pn, in, out, c1, c2, v.lam, b->stream);
            }
        }
    };
    if (R > 0) {
        faces(1, nullptr, nullptr, rec_d(b, r, R - 1), 0.0, 0.0);
        for (int k = R - 1; k >= 0; --k) {
            if (r.C) {
                B::adj_reinit_c<T>(b->acgrid, b->d_inst, b->d_amap[2], b->namap[2], r.C + 6LL * k * (long long)b->ld,
                                   (long long)b->ld, v.lam, v.lam2, b->stream);
            } else {
                const T* dk = k == 0 ? r.A[2] : rec_d(b, r, k - 1);
                B::adj_reinit<T>(b->agrid[3], b->d_inst, b->d_amap[3], b->namap[3], f, dk, v.lam, v.lam2, b->stream);
            }
            std::swap(v.lam, v.lam2);
        }
    } else {
        faces(1, nullptr, nullptr, r.A[2], 0.0, 0.0);
    }
    // stages 3, 2, 1: inputs A2, A1, phi^n; outputs A3, A2, A1
    const T* ins[3] = {phin, r.A[0], r.A[1]};
    for (int s = 2; s >= 0; --s) {
        faces(0, phin, ins[s], r.A[s], kC[s][0], kC[s][1]);
        B::adj_stage<T>(b->agrid, b->d_inst, b->d_amap, b->namap, f, ins[s], v.lam, v.lam2, v.lamPhin, v.lamW[0],
                        v.lamW[1], v.lamW[2], kC[s][0], kC[s][1], kC[s][2], s == 0, b->stream);
        std::swap(v.lam, v.lam2);
    }
}

template <typename T>
int backward_t(lsm_batch* b) {
    if (!b->rec_steps) return fail(b, LSM_ERR_BAD_PARAM, "lsm_batch_backward needs lsm_batch_forward_record first");
    AdjView<T> v = adj_view<T>(b);
    const AdjView<T> canon = v;
    const long long N = b->N;
    T* const zero_fields[7] = {v.lamPhin, v.lamW[0], v.lamW[1], v.lamW[2], v.lamU[0], v.lamU[1], v.lamU[2]};
    for (T* p : zero_fields) {
        lsm::ProfScope ps("k_zero", b->stream);
        k_zero<T><<<cblocks(N), 256, 0, b->stream>>>(N, p);
    }
    const int ck = b->rec_ck, nsteps = b->rec_steps, nseg = n_ckpt(nsteps, ck);
    const long long LD = (long long)b->ld;
    for (int sg = nseg - 1; sg >= 0; --sg) {
        const int c0 = sg * ck, L = std::min(c0 + ck, nsteps) - c0;
        // recompute the segment once from its checkpoint, keeping every
        // step's internals (the last segment's are still in the slots after
        // lsm_batch_forward_record), then reverse it step by step
        if (!(sg == nseg - 1 && b->rec_live)) {
            BCU(b, cudaMemcpyAsync(v.seg, v.ckpt + (long long)sg * LD, sizeof(T) * N, cudaMemcpyDeviceToDevice,
                                   b->stream));
            for (int q = 0; q < L; ++q) {
                const Rec<T> r = slot<T>(b, v, q);
                enqueue_step_io<T>(b, v.seg + (long long)q * LD, q + 1 < L ? v.seg + (long long)(q + 1) * LD : nullptr,
                                   &r, false, false, v.mrec + (long long)q * b->ninst);
            }
        }
        for (int q = L - 1; q >= 0; --q)
            adj_step<T>(b, v, slot<T>(b, v, q), v.seg + (long long)q * LD, v.mrec + (long long)q * b->ninst);
    }
    const Flat fl{b->d_inst, b->d_offs, b->ninst, N};
    lsm::batch::adj_contra<T>(fl, fields<T>(b), v.lamW[0], v.lamW[1], v.lamW[2], v.lamU[0], v.lamU[1], v.lamU[2],
                              b->stream);
    if (v.lam != canon.lam)
        BCU(b, cudaMemcpyAsync(canon.lam, v.lam, sizeof(T) * N, cudaMemcpyDeviceToDevice, b->stream));
    // earlier segments were recomputed into the slots
    b->rec_live = nseg == 1;
    BCU(b, cudaGetLastError());
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

const void* adj_field(lsm_batch* b, int which) {  // 0: lam, 1..3: lam_u
    if (b->prec) {
        AdjView<double> v = adj_view<double>(b);
        return which ? (const void*)v.lamU[which - 1] : (const void*)v.lam;
    }
    AdjView<float> v = adj_view<float>(b);
    return which ? (const void*)v.lamU[which - 1] : (const void*)v.lam;
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
    if (cfg->RNitermax < 0 || (cfg->precision != 0 && cfg->precision != 1) ||
        (cfg->adjoint_mode != 0 && cfg->adjoint_mode != 1) || (cfg->mass_correction != 0 && cfg->mass_correction != 1))
        return LSM_ERR_BAD_PARAM;
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
    b->prec = cfg->precision;
    b->esz = b->prec ? sizeof(double) : sizeof(float);
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
    b->off.push_back(n);
    b->N = n;
    for (int a = 0; a < 3; ++a) {
        b->face_pair[a] = true;
        for (int q = 0; q < ninst; ++q) {
            const int na = a == 0 ? inst[q].ni : a == 1 ? inst[q].nj : inst[q].nk;
            if (na < 6) b->face_pair[a] = false;
        }
    }
    if (n >= (1LL << 32)) {   // the interface-cell list holds 32-bit node indices
        delete b;
        return LSM_ERR_BAD_SHAPE;
    }
    auto cleanup = [&](int st) {
        lsm_batch_destroy(b);
        return st;
    };
    b->ld = array_stride(n, b->esz) / b->esz;
    b->ld8 = array_stride(n, 8) / 8;
    if (cudaMalloc(&b->field_arena, b->esz * b->ld * 21) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    for (int a = 0; a < 6; ++a) b->bufs[a] = (char*)b->field_arena + b->esz * b->ld * a;
    for (int a = 0; a < 15; ++a) b->comps[a] = (char*)b->field_arena + b->esz * b->ld * (6 + a);
    if (cudaMalloc(&b->xyz, 8 * b->ld8 * 4) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    b->cellfix = (long long*)(b->xyz + 3 * b->ld8);
    // a cache (the volume kernels form the same values per use without it):
    // left out when it does not fit, or with LSM_BATCH_CELLREL=0 (A/B runs)
    {
        const char* e = std::getenv("LSM_BATCH_CELLREL");
        if (!b->prec && !(e && !std::strcmp(e, "0")) &&
            cudaMalloc(&b->cellrel, sizeof(float) * 24 * (size_t)n) != cudaSuccess) {
            cudaGetLastError();
            b->cellrel = nullptr;
        }
    }
    if (cudaMalloc(&b->staging, sizeof(double) * 4 * b->max_inst_nodes) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_inst, sizeof(Inst) * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_offs, sizeof(long long) * (ninst + 1)) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_vols, sizeof(double) * 4 * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMallocHost(&b->h_vols, sizeof(double) * 4 * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_err, sizeof(unsigned)) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_ilist, sizeof(unsigned) * (size_t)n) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    b->geom_set.assign((size_t)ninst, 0);
    b->vel_set.assign((size_t)ninst, 0);
    {
        // the FP64 stage near the interface (FP32 batches; LSM_BATCH_BAND64=0 leaves it out)
        const char* e = std::getenv("LSM_BATCH_BAND64");
        if (!b->prec && !(e && !std::strcmp(e, "0"))) {
            if (cudaMalloc(&b->f64x, 8 * b->ld8 * 15) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
            if (cudaMalloc(&b->d_p64, sizeof(double*) * 15) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
            double* hp[15];
            for (int a = 0; a < 15; ++a) hp[a] = b->f64x + (size_t)a * b->ld8;
            if (cudaMemcpy(b->d_p64, hp, sizeof(hp), cudaMemcpyHostToDevice) != cudaSuccess)
                return cleanup(LSM_ERR_CUDA);
            cudaMemsetAsync(b->f64x, 0, 8 * b->ld8 * 15, b->stream);
        }
    }
    if (cudaMalloc(&b->d_icount, sizeof(unsigned)) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_target, sizeof(double) * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    if (cudaMalloc(&b->d_mass, sizeof(Mass) * ninst) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    {
        // no target volume (no correction) until lsm_batch_set_mass_target
        std::vector<double> nan((size_t)ninst, std::nan(""));
        std::vector<Mass> zero((size_t)ninst, Mass{0.0, 0.0, 0.0, std::nan("")});
        if (cudaMemcpy(b->d_target, nan.data(), sizeof(double) * ninst, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(b->d_mass, zero.data(), sizeof(Mass) * ninst, cudaMemcpyHostToDevice) != cudaSuccess)
            return cleanup(LSM_ERR_CUDA);
    }
    cudaMemcpyAsync(b->d_offs, b->off.data(), sizeof(long long) * (ninst + 1), cudaMemcpyHostToDevice, b->stream);
    cudaMemsetAsync(b->d_err, 0, sizeof(unsigned), b->stream);
    cudaMemsetAsync(b->d_vols, 0, sizeof(double) * 4 * ninst, b->stream);
    cudaMemsetAsync(b->field_arena, 0, b->esz * b->ld * 21, b->stream);
    cudaMemsetAsync(b->xyz, 0, 8 * b->ld8 * 4, b->stream);
    auto wire = [&](auto& f, auto* tag) {
        using T = std::remove_pointer_t<decltype(tag)>;
        f.phi = (T*)b->bufs[0];
        f.stage[0] = (T*)b->bufs[1];
        f.stage[1] = (T*)b->bufs[2];
        f.d[0] = (T*)b->bufs[3];
        f.d[1] = (T*)b->bufs[4];
        f.sgn = (T*)b->bufs[5];
        for (int c = 0; c < 3; ++c) {
            f.W[c] = (T*)b->comps[c];
            f.u[c] = (T*)b->comps[12 + c];
            f.xyz[c] = b->xyz + c * b->ld8;
        }
        for (int c = 0; c < 9; ++c) f.m[c] = (T*)b->comps[3 + c];
        f.cellfix = b->cellfix;
        f.cellrel = b->cellrel;
        for (int c = 0; c < 3; ++c) f.W64[c] = b->f64x ? b->f64x + (size_t)(12 + c) * b->ld8 : nullptr;
    };
    if (b->prec) wire(b->f64, (double*)nullptr);
    else wire(b->f32, (float*)nullptr);
    // the TMA-staged stage needs whole 16-byte rows of one instance
    if (!b->prec && ninst == 1 && inst[0].ni % 4 == 0)
        b->tma_eligible = encode_stage_map(b, b->field_arena, 21, &b->tm_field);
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) return cleanup(LSM_ERR_CUDA);
    *out = b;
    return LSM_OK;
}

int lsm_batch_destroy(lsm_batch_handle b) {
    if (!b) return LSM_ERR_NULL;
    Dev guard(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (void* p : {b->field_arena, (void*)b->xyz, (void*)b->staging, (void*)b->d_inst, (void*)b->d_offs,
                    (void*)b->d_brick, (void*)b->d_amap[0], (void*)b->d_amap[1], (void*)b->d_amap[2],
                    (void*)b->d_amap[3], (void*)b->d_vacc, (void*)b->d_vols, (void*)b->d_err, b->adj,
                    (void*)b->d_target, (void*)b->d_mass, (void*)b->wfix, (void*)b->d_tpart, (void*)b->d_ssum,
                    (void*)b->d_ilist, (void*)b->d_icount, (void*)b->f64x, (void*)b->d_p64, (void*)b->cellrel})
        if (p) cudaFree(p);
    if (b->h_vols) cudaFreeHost(b->h_vols);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return LSM_OK;
}

int lsm_batch_set_geometry(lsm_batch_handle b, int q, const double* x, const double* y, const double* z,
                           const double* csi, const double* eta, const double* zet) {
    if (!b || !x || !y || !z || !csi || !eta || !zet) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    const double* c3[3] = {x, y, z};
    for (int c = 0; c < 3; ++c)
        BTRY(load_in(b, c3[c], n, 1, 0, 1, CvtDst{{b->xyz + c * b->ld8 + o}, {}}, true));
    const double* m3[3] = {csi, eta, zet};
    for (int d = 0; d < 3; ++d) {
        CvtDst to{};
        for (int c = 0; c < 3; ++c) {
            to.d[c] = (char*)b->comps[3 + 3 * d + c] + b->esz * o;
            to.e[c] = b->f64x ? b->f64x + (size_t)(3 * d + c) * b->ld8 + o : nullptr;
        }
        BTRY(load_in(b, m3[d], n, 3, 0, 3, to));
    }
    b->geom_set[q] = 1;
    b->w_stale = true;
    update_w64(b, q);
    // cell_hex indexes from the packed base arrays with the instance offset o
    lsm::batch::cell_hex(o, I.ni, I.nj, I.nk, b->xyz, b->xyz + b->ld8, b->xyz + 2 * b->ld8, b->cellfix, b->stream);
    if (b->cellrel)
        lsm::batch::cell_rel(o, I.ni, I.nj, I.nk, b->xyz, b->xyz + b->ld8, b->xyz + 2 * b->ld8, b->cellrel, b->stream);
    BCU(b, cudaGetLastError());
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

}  // extern "C"

namespace {
// q(2:4, .) of instance q into the batch (and its FP64 copy); enqueued only
int velocity_in(lsm_batch* b, int q, const double* qv) {
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    CvtDst to{};
    for (int c = 0; c < 3; ++c) {
        to.d[c] = (char*)b->comps[12 + c] + b->esz * o;
        to.e[c] = b->f64x ? b->f64x + (size_t)(9 + c) * b->ld8 + o : nullptr;
    }
    BTRY(load_in(b, qv, n, 4, 1, 3, to));
    b->vel_set[q] = 1;
    b->w_stale = true;
    update_w64(b, q);
    BCU(b, cudaGetLastError());
    return LSM_OK;
}
// phi of instance q out to the caller's array; enqueued only
int phi_out(lsm_batch* b, int q, double* phi) {
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    return store_out(b, phi, n, 1, 0, 1, CvtSrc{{(const char*)b->bufs[0] + b->esz * o}}, false);
}
}  // namespace

extern "C" {

int lsm_batch_set_velocity(lsm_batch_handle b, int q, const double* qv) {
    if (!b || !qv) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    Dev guard(b->device);
    BTRY(velocity_in(b, q, qv));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_set_velocities(lsm_batch_handle b, const double* const* qv) {
    if (!b || !qv) return LSM_ERR_NULL;
    for (int q = 0; q < b->ninst; ++q)
        if (!qv[q]) return LSM_ERR_NULL;
    Dev guard(b->device);
    for (int q = 0; q < b->ninst; ++q) BTRY(velocity_in(b, q, qv[q]));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_set_phi(lsm_batch_handle b, int q, const double* phi) {
    if (!b || !phi) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    BTRY(load_in(b, phi, n, 1, 0, 1, CvtDst{{(char*)b->bufs[0] + b->esz * o}, {}}));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_get_phi(lsm_batch_handle b, int q, double* phi) {
    if (!b || !phi) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    Dev guard(b->device);
    BTRY(phi_out(b, q, phi));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_get_phis(lsm_batch_handle b, double* const* phi) {
    if (!b || !phi) return LSM_ERR_NULL;
    for (int q = 0; q < b->ninst; ++q)
        if (!phi[q]) return LSM_ERR_NULL;
    Dev guard(b->device);
    for (int q = 0; q < b->ninst; ++q) BTRY(phi_out(b, q, phi[q]));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_step(lsm_batch_handle b, int nsteps, double* volumes) {
    if (!b) return LSM_ERR_NULL;
    if (nsteps < 0) return fail(b, LSM_ERR_BAD_PARAM, "negative step count");
    Dev guard(b->device);
    BTRY(prepare(b));
    BTRY(run_steps(b, nsteps));
    BCU(b, cudaGetLastError());
    unsigned flags = 0;
    BCU(b, cudaMemcpyAsync(&flags, b->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
    if (volumes)
        BCU(b, cudaMemcpyAsync(b->h_vols, b->d_vols, sizeof(double) * 4 * b->ninst, cudaMemcpyDeviceToHost,
                               b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    if (volumes) std::memcpy(volumes, b->h_vols, sizeof(double) * 4 * b->ninst);
    if (flags & lsm::kErrTimeout) return fail(b, LSM_ERR_CUDA, "a TMA copy of the RK stage did not complete");
    if (flags & lsm::kErrNonFinite) return fail(b, LSM_ERR_NONFINITE, "non-finite phi in the batch");
    return LSM_OK;
}

int lsm_batch_forward_record(lsm_batch_handle b, int nsteps, int checkpoint_every) {
    if (!b) return LSM_ERR_NULL;
    if (nsteps <= 0 || checkpoint_every <= 0)
        return fail(b, LSM_ERR_BAD_PARAM, "step count and checkpoint interval must be positive");
    Dev guard(b->device);
    BTRY(prepare(b));
    return b->prec ? forward_record_t<double>(b, nsteps, checkpoint_every)
                   : forward_record_t<float>(b, nsteps, checkpoint_every);
}

int lsm_batch_set_grad_phi(lsm_batch_handle b, int q, const double* g) {
    if (!b || !g) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    if (!b->rec_steps) return fail(b, LSM_ERR_BAD_PARAM, "seed the gradient after lsm_batch_forward_record");
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    BTRY(load_in(b, g, n, 1, 0, 1, CvtDst{{(char*)adj_field(b, 0) + b->esz * o}, {}}));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_backward(lsm_batch_handle b) {
    if (!b) return LSM_ERR_NULL;
    Dev guard(b->device);
    BTRY(refresh_w(b));
    return b->prec ? backward_t<double>(b) : backward_t<float>(b);
}

int lsm_batch_get_grad_phi0(lsm_batch_handle b, int q, double* g) {
    if (!b || !g) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    if (!b->rec_steps) return fail(b, LSM_ERR_BAD_PARAM, "no recorded steps");
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    return store_out(b, g, n, 1, 0, 1, CvtSrc{{(const char*)adj_field(b, 0) + b->esz * o}});
}

int lsm_batch_get_grad_velocity(lsm_batch_handle b, int q, double* gq) {
    if (!b || !gq) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    if (!b->rec_steps) return fail(b, LSM_ERR_BAD_PARAM, "no recorded steps");
    Dev guard(b->device);
    const auto& I = b->inst[q];
    const long long n = (long long)I.ni * I.nj * I.nk, o = b->off[q];
    CvtSrc from{};
    for (int c = 0; c < 3; ++c) from.s[c] = (const char*)adj_field(b, 1 + c) + b->esz * o;
    return store_out(b, gq, n, 4, 1, 3, from);
}

int lsm_batch_set_mass_target(lsm_batch_handle b, int q, double volume) {
    if (!b) return LSM_ERR_NULL;
    BTRY(check_inst(b, q));
    if (!b->cfg.mass_correction) return fail(b, LSM_ERR_BAD_PARAM, "the batch was created without mass correction");
    Dev guard(b->device);
    const double v = volume;   // copied before the call returns (synchronised below)
    BCU(b, cudaMemcpyAsync(b->d_target + q, &v, sizeof(double), cudaMemcpyHostToDevice, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    return LSM_OK;
}

int lsm_batch_water_volume(lsm_batch_handle b, double* volumes) {
    if (!b || !volumes) return LSM_ERR_NULL;
    Dev guard(b->device);
    BTRY(prepare(b));
    namespace B = lsm::batch;
    const Flat fl{b->d_inst, b->d_offs, b->ninst, b->N};
    if (b->prec)
        B::volume<double>(b->vgrid, b->d_inst, b->d_amap[2], b->namap[2], fl, b->f64, b->f64.phi, b->d_vacc, false,
                          b->d_ilist, b->d_icount, b->stream);
    else
        B::volume<float>(b->vgrid, b->d_inst, b->d_amap[2], b->namap[2], fl, b->f32, b->f32.phi, b->d_vacc, false,
                         b->d_ilist, b->d_icount, b->stream);
    B::volume_final(b->ninst, b->d_vacc, b->d_vols, nullptr, nullptr, nullptr, b->stream);
    BCU(b, cudaGetLastError());
    BCU(b, cudaMemcpyAsync(b->h_vols, b->d_vols, sizeof(double) * 4 * b->ninst, cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    std::memcpy(volumes, b->h_vols, sizeof(double) * 4 * b->ninst);
    return LSM_OK;
}

int lsm_batch_mass_state(lsm_batch_handle b, double* out) {
    if (!b || !out) return LSM_ERR_NULL;
    Dev guard(b->device);
    std::vector<Mass> m((size_t)b->ninst);
    BCU(b, cudaMemcpyAsync(m.data(), b->d_mass, sizeof(Mass) * b->ninst, cudaMemcpyDeviceToHost, b->stream));
    BCU(b, cudaStreamSynchronize(b->stream));
    for (int q = 0; q < b->ninst; ++q) {
        out[4 * q] = m[q].V;
        out[4 * q + 1] = m[q].A;
        out[4 * q + 2] = m[q].C;
        out[4 * q + 3] = m[q].target;
    }
    return LSM_OK;
}

int lsm_batch_shape(lsm_batch_handle b, int* index, int* tx, int* ty, int* tz) {
    if (!b) return LSM_ERR_NULL;
    const auto sh = lsm::batch::kShapes[b->shape];
    if (index) *index = b->reinit_march ? 5 : b->shape;
    if (tx) *tx = sh.tx;
    if (ty) *ty = sh.ty;
    if (tz) *tz = sh.tz;
    return LSM_OK;
}

long long lsm_batch_nodes(lsm_batch_handle b) { return b ? b->N : 0; }

int lsm_batch_stage_kernel(lsm_batch_handle b) { return b ? (b->tma_stage ? 1 : 0) : -1; }

int lsm_batch_launches_per_step(lsm_batch_handle b) {
    if (!b) return 0;
    // volume 3 (scan, interface cells, final), three stages x (stencil +
    // faces) 6, then RNitermax pseudo-steps (the first with the sign field)
    // + final faces, or one full bcond pass; the mass correction's shift 1
    // (W is formed outside the step, once per change of its inputs)
    const int R = b->cfg.RNitermax;
    return 3 + 6 + (R > 0 ? R + 1 : 1) + (b->cfg.mass_correction ? 1 : 0);
}

const char* lsm_batch_last_error(lsm_batch_handle b) { return b ? b->err.c_str() : ""; }

}  // extern "C"
