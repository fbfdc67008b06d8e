// lsm_geometric.cu -- the hybrid path's geometric reinitialisation
// (src/geometric_reinitialisation.F90:1-94) on one GPU, FP64 with the
// reference's rounding (this unit is built with --fmad=false).
//
// The reference builds two linked structures on the host: a list of pnodes
// (vertices of phase-change tetrahedra, numbered in k, j, i order) and a list
// of K tetrahedra (numbered by cell in k, j, i order, then by tetrahedron
// 1..6 inside the cell), each pnode holding the ids of its K tetrahedra in
// the order they were appended.  Here both lists are dense device arrays
// made by two prefix sums:
//   - pnode ids: an exclusive scan of the per-node pnode flag, in the
//     node array's own (Fortran) order;
//   - K-tetrahedron ids: an exclusive scan of popcount(cell bits) over the
//     cells in the same order, plus the rank of the tetrahedron's bit inside
//     its cell.
// A pnode's tetrahedron list is then not stored: it is re-enumerated from the
// (at most) eight cells around the node, in increasing cell index and
// tetrahedron number, which is exactly the order GetTetrahedraList appends
// them (src/GetTetrahedraList.F90:322-446).  The distance loops keep the
// reference's sequential running-minimum updates per node (their rounding
// depends on the order): one thread per pnode in k_geo_sd, one warp per
// -1 node in k_geo_neigh (the lanes share out the distances, the chain is
// replayed in order).
#include <cuda_runtime.h>

#include "lsm_common.cuh"
#include "lsm_geometric.h"
#include "lsm_kernels.h"
#include "lsm_volume_dev.cuh"

namespace lsm {
namespace {

constexpr int kThreads = 256;
constexpr int kTile = 4 * kThreads;  // elements per scan tile

// ------------------------------------------------------------- geometry

// Comparisons on the integer pipe: for non-negative doubles (+0 included)
// the IEEE order is the order of the bit patterns as signed integers, and
// x < 0 holds exactly when the sign bit is set and x is not -0.  GB300's
// FP64 pipe is its scarce resource; these are exact (no NaN reaches them).
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ bool nn_lt(double a, double b) { return dbits(a) < dbits(b); }   // a, b >= +0
__device__ __forceinline__ bool nn_le(double a, double b) { return dbits(a) <= dbits(b); }  // a, b >= +0
__device__ __forceinline__ bool neg(double x) {
    const long long b = dbits(x);
    return b < 0 && b != (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool pos(double x) { return dbits(x) > 0; }  // x > 0
constexpr long long kOneBits = 0x3FF0000000000000LL;                    // 1.0
__device__ __forceinline__ bool lt1(double x) { return dbits(x) < kOneBits; }  // x < 1

// NORM2 of a 3-vector as gfortran expands the intrinsic: a scaled sum of
// squares, zeros skipped, sqrt(sum) * scale.  While the scale is exactly 1
// the divisions ax / 1 and the final * 1 are skipped (both are exact).
__device__ __forceinline__ double norm2v(const double* a) {
    double scale = 1.0, r = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const long long b = dbits(a[c]) & 0x7FFFFFFFFFFFFFFFLL;  // |a[c]|
        if (b != 0) {
            const double ax = __longlong_as_double(b);
            if (dbits(scale) < b) {
                const double v = scale / ax;
                r = 1.0 + r * v * v;
                scale = ax;
            } else {
                const double v = dbits(scale) == kOneBits ? ax : ax / scale;
                r = r + v * v;
            }
        }
    }
    return dbits(scale) == kOneBits ? sqrt(r) : sqrt(r) * scale;
}
__device__ __forceinline__ void sub3(const double* a, const double* b, double* c) {
    c[0] = a[0] - b[0]; c[1] = a[1] - b[1]; c[2] = a[2] - b[2];
}
__device__ __forceinline__ double dot3g(const double* a, const double* b) {
    double s = 0.0;
    s = s + a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}
__device__ __forceinline__ void cross3g(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dmin(double a, double b) { return nn_lt(b, a) ? b : a; }  // a, b >= +0
__device__ __forceinline__ double sgn1(double x) { return copysign(1.0, x); }  // sign(one, x)

// GetTriangleArea, src/TetrahedronMethods.F90:691-707
__device__ double tri_area(const double (&T)[3][3]) {
    double u[3], v[3], c[3];
    sub3(T[1], T[0], u); sub3(T[2], T[0], v); cross3g(u, v, c);
    return 0.5 * norm2v(c);
}

// TetrahedronTriangles, src/TetrahedronMethods.F90:86-104 (edges 0..5)
__constant__ signed char c_tet_tris[16][6] = {
    {-1, -1, -1, -1, -1, -1}, {0, 3, 2, -1, -1, -1}, {0, 1, 4, -1, -1, -1}, {1, 4, 2, 2, 4, 3},
    {1, 2, 5, -1, -1, -1},    {0, 3, 5, 0, 5, 1},    {0, 2, 5, 0, 5, 4},    {5, 4, 3, -1, -1, -1},
    {3, 4, 5, -1, -1, -1},    {4, 5, 0, 5, 2, 0},    {1, 5, 0, 5, 3, 0},    {5, 2, 1, -1, -1, -1},
    {3, 4, 2, 2, 4, 1},       {4, 1, 0, -1, -1, -1}, {2, 3, 0, -1, -1, -1}, {-1, -1, -1, -1, -1, -1}};

// MarchingTetrahedron with its triangle and area outputs,
// src/TetrahedronMethods.F90:26-664.  ntri: 1 or 2 triangles, 0 none,
// -1/-2 a vertex/edge on the zero level (no triangle kept by the caller).
struct MT {
    int ntri;
    double tri[2][3][3];
    double area, wv;
};

__device__ void marching_full(const double (&V)[4][3], const double (&ph)[4], MT& o, bool want_tri,
                              unsigned* err) {
    o.ntri = 0; o.area = 0.0; o.wv = 0.0;
    int s[4], nz = 0;
    bool allp = true, alln = true, allge = true, allle = true;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        s[v] = ph[v] > kTinyD ? 1 : (ph[v] < -kTinyD ? -1 : 0);
        allp &= s[v] == 1; alln &= s[v] == -1; nz += s[v] == 0;
        allge &= s[v] >= 0; allle &= s[v] <= 0;
    }
    if (allp) { o.wv = tetvol<true>(V[0], V[1], V[2], V[3]); return; }
    if (alln) return;
    int fi = 0;
    if (nz > 0 && (allge || allle)) {
        if (nz == 1 || nz == 2) {
            o.ntri = -nz;  // a vertex or an edge: no triangle is used downstream
            int water;
            if (nz == 1) {
                water = s[0] == 0 ? s[1] == 1 : s[0] == 1;
            } else {
                if (s[0] == 0 && s[1] == 0) water = s[2] == 1;
                else if (s[1] == 0 && s[2] == 0) water = s[0] == 1;
                else if (s[2] == 0 && s[0] == 0) water = s[1] == 1;
                else if (s[0] == 0 && s[3] == 0) water = s[1] == 1;
                else water = s[0] == 1;
            }
            o.wv = water ? tetvol<true>(V[0], V[1], V[2], V[3]) : 0.0;
            return;
        }
        if (nz == 3) {  // a face: one triangle
            o.ntri = 1;
            int v = 0;
            while (s[v] == 0) ++v;
            int q = 0;
#pragma unroll
            for (int w = 0; w < 4; ++w)
                if (w != v) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) o.tri[0][q][c] = V[w][c];
                    ++q;
                }
            if (want_tri) o.area = tri_area(o.tri[0]);
            o.wv = s[v] == 1 ? tetvol<true>(V[0], V[1], V[2], V[3]) : 0.0;
            return;
        }
        // four zero vertices: FlagIndex stays 0
    } else {
#pragma unroll
        for (int v = 0; v < 4; ++v)
            if (s[v] == -1) fi |= 1 << v;
    }
    if (fi == 0) o.wv = tetvol<true>(V[0], V[1], V[2], V[3]);
    const int ef = c_edge_flags[fi];
    if (ef == 0) return;
    double E[6][3];
#pragma unroll
    for (int e = 0; e < 6; ++e) {
        E[e][0] = E[e][1] = E[e][2] = -9.9;
        if (!(ef >> e & 1)) continue;
        const int sv = c_edge[e][0], ev = c_edge[e][1];
        const double den = ph[ev] - ph[sv];
        const double sc = fabs(den) < kEpsSims * kEpsSims * kEpsSims ? 0.0 : ph[ev] / den;
#pragma unroll
        for (int c = 0; c < 3; ++c) E[e][c] = V[ev][c] + sc * (V[sv][c] - V[ev][c]);
    }
    for (int t = 0; t < 2; ++t) {
        if (c_tet_tris[fi][3 * t] < 0) break;
        o.ntri += 1;
        if (!want_tri) continue;
        for (int v = 0; v < 3; ++v) {
            const int e = c_tet_tris[fi][3 * t + v];
#pragma unroll
            for (int c = 0; c < 3; ++c) o.tri[t][v][c] = E[e][c];
        }
        o.area = o.area + tri_area(o.tri[t]);
    }
    o.wv = water_volume<true>(V, E, fi, err);
}

// DistancePointLine, src/TetrahedronMethods.F90:1356-1399, given the
// vectors and norms the caller already has: AP = P - A, BP = P - B,
// AB = B - A and their norms (BA = A - B is -AB exactly)
__device__ __forceinline__ double dist_point_line(const double* AP, const double* BP, const double* AB, double nAP,
                                                  double nBP, double nAB) {
    const double BA[3] = {-AB[0], -AB[1], -AB[2]};
    bool valid = true;
    if (nn_lt(nAB, kEpsSims)) valid = false;
    if (neg(dot3g(AB, AP))) valid = false;
    if (neg(dot3g(BA, BP))) valid = false;
    if (valid) {
        double c[3];
        cross3g(AP, BP, c);
        return norm2v(c) / nAB;
    }
    return dmin(nAP, nBP);
}

// What DistancePointTriangle computes from the triangle alone, evaluated
// once per triangle with the same operations: the edge vectors
// AB = B - A, BC = C - B, CA = A - C, their norms, and the projection
// step's normal nv = AB x (C - A) (C - A is -CA exactly) with nv . nv.
struct TriGeo {
    double AB[3], BC[3], CA[3];
    double nAB, nBC, nCA;
    double nv[3], nn;
};

__device__ void tri_geo(const double* T, TriGeo& g) {
    const double* A = T;
    const double* B = T + 3;
    const double* Cv = T + 6;
    sub3(B, A, g.AB); sub3(Cv, B, g.BC); sub3(A, Cv, g.CA);
    g.nAB = norm2v(g.AB); g.nBC = norm2v(g.BC); g.nCA = norm2v(g.CA);
    const double v[3] = {-g.CA[0], -g.CA[1], -g.CA[2]};
    cross3g(g.AB, v, g.nv);
    g.nn = dot3g(g.nv, g.nv);
}

// DistancePointTriangle + CheckProjectionPointOnATriangle3,
// src/TetrahedronMethods.F90:1008-1070,1593-1684.  Each norm the reference
// evaluates more than once on the same vector (|P - A| as a vertex distance
// and inside DistancePointLine, |B - A| twice per edge, |A - B| = |B - A| in
// the degenerate-triangle test) is evaluated once here, and the parts that
// depend on the triangle alone come from TriGeo: same inputs, same value.
// Kept from the reference: the projected point weights P1 by alpha (the
// weight of P3 in the standard barycentric form) and P3 by gamma.
__device__ double dist_point_triangle(const double* T, const TriGeo& g, const double* P) {
    const double* A = T;
    const double* B = T + 3;
    const double* Cv = T + 6;
    double PA[3], PB[3], PC[3];
    sub3(P, A, PA); sub3(P, B, PB); sub3(P, Cv, PC);
    const double nA = norm2v(PA), nB = norm2v(PB), nC = norm2v(PC);
    double m = dmin(dmin(nA, nB), nC);
    m = dmin(m, dist_point_line(PA, PB, g.AB, nA, nB, g.nAB));
    m = dmin(m, dist_point_line(PB, PC, g.BC, nB, nC, g.nBC));
    m = dmin(m, dist_point_line(PC, PA, g.CA, nC, nA, g.nCA));
    if (nn_le(g.nAB, kEpsSims) || nn_le(g.nCA, kEpsSims) || nn_le(g.nBC, kEpsSims)) return m;
    const double v[3] = {-g.CA[0], -g.CA[1], -g.CA[2]};
    double cu[3], cw[3];
    cross3g(g.AB, PA, cu); cross3g(PA, v, cw);
    const double alpha = dot3g(cu, g.nv) / g.nn;
    const double beta = dot3g(cw, g.nv) / g.nn;
    const double gamma = 1.0 - beta - alpha;
    if (pos(alpha) && lt1(alpha) && pos(beta) && lt1(beta) && pos(gamma) && lt1(gamma)) {
        double pp[3], dd[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) pp[c] = alpha * A[c] + beta * B[c] + gamma * Cv[c];
        sub3(P, pp, dd);
        m = dmin(m, norm2v(dd));
    }
    return m;
}

// the reference's running minimum d + exsign (da - d), exsign = (sign(1,
// d - da) + 1) / 2: 1 when da <= d (d - da >= +0), and then d + (da - d);
// 0 otherwise, and then d + 0 = d.  d, da >= +0.
__device__ __forceinline__ double run_min(double d, double da) {
    return nn_le(da, d) ? d + (da - d) : d;
}

// the reference's signed update of a running |value| by a distance dp
// (exsign2 = 1 when |value| >= dp): the new magnitude
__device__ __forceinline__ double mag_step(double a, double dp) {
    return nn_le(dp, a) ? a + (dp - a) : a;
}

// ------------------------------------------------------------ the lists

// cell vertex v at offset (dx, dy, dz): the reference's numbering
// v0 = 000, v1 = 100, v2 = 110, v3 = 010, v4 = 001, v5 = 101, v6 = 111, v7 = 011
__constant__ int c_cell_off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                     {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
__constant__ unsigned char c_vert_at[2][2][2] = {{{0, 4}, {3, 7}}, {{1, 5}, {2, 6}}};  // [dx][dy][dz]

// bits 1..6: the tetrahedra of the TriangulationCase-1 split containing vertex v
__host__ __device__ constexpr unsigned tets_of_vertex(int v) {
    constexpr int T[6][4] = {{0, 5, 1, 6}, {0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}};
    unsigned m = 0;
    for (int t = 0; t < 6; ++t)
        for (int q = 0; q < 4; ++q)
            if (T[t][q] == v) m |= 1u << (t + 1);
    return m;
}
__constant__ unsigned char c_vtets[8] = {tets_of_vertex(0), tets_of_vertex(1), tets_of_vertex(2),
                                         tets_of_vertex(3), tets_of_vertex(4), tets_of_vertex(5),
                                         tets_of_vertex(6), tets_of_vertex(7)};

// CellPnodeTetrahedronIdentification, src/TetrahedronMethods.F90:2124-2361:
// bit t (1..6) of *tets marks a phase-change tetrahedron, bit v of *verts a
// vertex of one
__device__ void cell_pnodes(const double (&P)[8], unsigned* verts, unsigned* tets) {
    *verts = 0; *tets = 0;
    bool allw = true, alla = true, anyz = false;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
        allw &= P[v] > kEpsSims; alla &= P[v] < -kEpsSims; anyz |= fabs(P[v]) < kEpsSims;
    }
    if (allw || alla) return;
    bool pc = anyz;
    if (!pc) {
        const double s0 = sgn1(P[0]);
#pragma unroll
        for (int v = 1; v < 8; ++v) pc |= s0 * P[v] < 0.0;
    }
    if (!pc) return;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
        double a = P[c_tets[t][0]];
        bool change = fabs(a) < kEpsSims, second = !(a <= kEpsSims);
        const double sg = sgn1(a);
#pragma unroll
        for (int q = 1; q < 4; ++q) {
            a = P[c_tets[t][q]];
            if (sg * a < 0.0 || fabs(a) < kEpsSims) {
                if (a <= kEpsSims) second = false;
                change = true;
            }
        }
        if (change && !second) {
            *tets |= 1u << (t + 1);
#pragma unroll
            for (int q = 0; q < 4; ++q) *verts |= 1u << c_tets[t][q];
        }
    }
}

__device__ __forceinline__ void node_ijk(const DevGrid& g, long long l, int* i, int* j, int* k) {
    *k = (int)(l / g.sk);
    const long long r = l - (long long)*k * g.sk;
    *j = (int)(r / g.sj);
    *i = (int)(r - (long long)*j * g.sj);
}

// the K tetrahedra with a vertex at node (i, j, k), in the order
// GetTetrahedraList appends them to the node's list
template <class F>
__device__ __forceinline__ void for_each_tet(const DevGrid& g, int i, int j, int k,
                                             const unsigned char* __restrict__ cellbits,
                                             const int* __restrict__ tetbase, F f) {
    for (int dz = 1; dz >= 0; --dz) {
        const int ck = k - dz;
        if (ck < 0 || ck > g.nk - 2) continue;
        for (int dy = 1; dy >= 0; --dy) {
            const int cj = j - dy;
            if (cj < 0 || cj > g.nj - 2) continue;
            for (int dx = 1; dx >= 0; --dx) {
                const int ci = i - dx;
                if (ci < 0 || ci > g.ni - 2) continue;
                const long long lc = gid(g, ci, cj, ck);
                const unsigned bits = cellbits[lc];
                unsigned m = bits & c_vtets[c_vert_at[dx][dy][dz]];
                if (!m) continue;
                const int base = tetbase[lc];
                while (m) {
                    const int t = __ffs(m) - 1;
                    m &= m - 1;
                    f(base + __popc(bits & ((1u << t) - 1u)));
                }
            }
        }
    }
}

// one K tetrahedron: its isosurface triangles (18 doubles) with their
// triangle-only distance terms (TriGeo), area and water volume of the
// linear reconstruction, its four pnode ids (0-based), and per triangle an
// FP32 bounding box (rounded outwards) and FP32 vertices, used only to skip
// distance evaluations that cannot change a running minimum
struct alignas(16) GeoTet {
    double tri[2][9];
    TriGeo tg[2];
    float box[2][6];  // lo x y z, hi x y z
    float trf[2][9];  // the vertices rounded to FP32 (upper bounds of the distance)
    double area, wv;
    int nis;
    int v[4];
    int pad;
};

// A distance evaluation is skipped only when a lower bound of the exact
// point-triangle distance -- the distance from the point to the triangle's
// bounding box -- exceeds the running minimum d by a margin.  Every candidate
// point of DistancePointTriangle (vertices, feet on the edges, the
// projection step's convex combination of the vertices) lies in the
// triangle, so the computed distance is at least the exact distance less a
// few ulps of the coordinates.  The bound is evaluated in FP32 (the FP64
// units are scarce) on a box rounded outwards: the point and d rounded to
// FP32 and the FP32 norm keep its error below 1e-6 of the sizes involved,
// and the margin is 1e-5 of them.  A skipped triangle therefore leaves
// d + exsign (da - d) = d exactly as the full evaluation would.
__device__ __forceinline__ bool beyond_box(const float* p, float pscale, const float* lo, const float* hi, float d) {
    const float dx = fmaxf(fmaxf(lo[0] - p[0], p[0] - hi[0]), 0.0f);
    const float dy = fmaxf(fmaxf(lo[1] - p[1], p[1] - hi[1]), 0.0f);
    const float dz = fmaxf(fmaxf(lo[2] - p[2], p[2] - hi[2]), 0.0f);
    const float lb = sqrtf(dx * dx + dy * dy + dz * dz);
    return lb > d + 1.0e-5f * (lb + d + pscale);
}

// -------------------------------------------------------------- kernels

// GetTetrahedraList, first loop (src/GetTetrahedraList.F90:205-284)
__global__ void k_geo_cells(DevGrid g, const double* __restrict__ phi, unsigned char* __restrict__ cellbits,
                            int* __restrict__ flags) {
    const long long ncell = (long long)(g.ni - 1) * (g.nj - 1) * (g.nk - 1);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(c % (g.ni - 1));
        const long long r = c / (g.ni - 1);
        const int j = (int)(r % (g.nj - 1));
        const int k = (int)(r / (g.nj - 1));
        double P[8];
#pragma unroll
        for (int v = 0; v < 8; ++v)
            P[v] = phi[gid(g, i + c_cell_off[v][0], j + c_cell_off[v][1], k + c_cell_off[v][2])];
        unsigned verts, tets;
        cell_pnodes(P, &verts, &tets);
        cellbits[gid(g, i, j, k)] = (unsigned char)tets;
#pragma unroll
        for (int v = 0; v < 8; ++v)
            if (verts >> v & 1) flags[gid(g, i + c_cell_off[v][0], j + c_cell_off[v][1], k + c_cell_off[v][2])] = 1;
    }
}

// block-wide exclusive scan of one value per thread; returns the prefix and
// the block total in *total
__device__ int block_exclusive_scan(int v, int* total) {
    __shared__ int ws[kThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < kThreads / 32 ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < kThreads / 32) ws[lane] = t;
    }
    __syncthreads();
    const int before = w ? ws[w - 1] : 0;
    *total = ws[kThreads / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// per-element count: mode 0 the pnode flag, mode 1 the number of K tetrahedra of the cell
template <int MODE>
__device__ __forceinline__ int scan_count(const void* src, long long l) {
    if (MODE == 0) return static_cast<const int*>(src)[l] ? 1 : 0;
    if (MODE == 2) return static_cast<const int*>(src)[l] < 0 ? 1 : 0;
    return __popc(static_cast<const unsigned char*>(src)[l]);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_scan_tiles(long long n, const void* __restrict__ src,
                                                         int* __restrict__ tile_sum) {
    const long long base = (long long)blockIdx.x * kTile + 4 * threadIdx.x;
    int s = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q)
        if (base + q < n) s += scan_count<MODE>(src, base + q);
    int tot;
    block_exclusive_scan(s, &tot);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

// exclusive scan of the tile sums in place (one block); total -> *total
__global__ void __launch_bounds__(kThreads) k_scan_top(int ntiles, int* __restrict__ tile_sum,
                                                       int* __restrict__ total) {
    int carry = 0;
    for (int b0 = 0; b0 < ntiles; b0 += kThreads) {
        const int b = b0 + threadIdx.x;
        const int v = b < ntiles ? tile_sum[b] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, &tot);
        if (b < ntiles) tile_sum[b] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total = carry;
}

// mode 0: ids[l] = pnode id + 1 (0: not a pnode), node_of[id] = l;
// mode 1: tetbase[l] = first K-tetrahedron id of cell l;
// mode 2: node_of[c] = the c-th node tagged -1
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_scan_apply(long long n, const void* __restrict__ src,
                                                         const int* __restrict__ tile_off, int* __restrict__ out,
                                                         long long* __restrict__ node_of) {
    const long long base = (long long)blockIdx.x * kTile + 4 * threadIdx.x;
    int c[4], s = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        c[q] = base + q < n ? scan_count<MODE>(src, base + q) : 0;
        s += c[q];
    }
    int tot;
    int off = tile_off[blockIdx.x] + block_exclusive_scan(s, &tot);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (base + q >= n) break;
        if (MODE == 0) {
            out[base + q] = c[q] ? off + 1 : 0;
            if (c[q]) node_of[off] = base + q;
        } else if (MODE == 1) {
            out[base + q] = off;
        } else if (c[q]) {
            node_of[off] = base + q;
        }
        off += c[q];
    }
}

// GetTetrahedraList third loop + the marching step of GetIsosurfaceAndDistances
// (src/GetIsosurfaceAndDistances.F90:80-162)
__global__ void k_geo_tets(DevGrid g, const double* __restrict__ phi, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z,
                           const unsigned char* __restrict__ cellbits, const int* __restrict__ tetbase,
                           const int* __restrict__ ids, GeoTet* __restrict__ tets, unsigned* err) {
    const long long n = (long long)g.ni * g.nj * g.nk;
    for (long long lc = blockIdx.x * (long long)blockDim.x + threadIdx.x; lc < n;
         lc += (long long)gridDim.x * blockDim.x) {
        const unsigned bits = cellbits[lc];
        if (!bits) continue;
        int i, j, k;
        node_ijk(g, lc, &i, &j, &k);
        int tid = tetbase[lc];
        for (int t = 0; t < 6; ++t) {
            if (!(bits >> (t + 1) & 1)) continue;
            double V[4][3], ph[4];
            GeoTet T;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int cv = c_tets[t][q];
                const long long l = gid(g, i + c_cell_off[cv][0], j + c_cell_off[cv][1], k + c_cell_off[cv][2]);
                V[q][0] = x[l]; V[q][1] = y[l]; V[q][2] = z[l];
                ph[q] = phi[l];
                T.v[q] = ids[l] - 1;
            }
            MT o;
            marching_full(V, ph, o, true, err);
            T.nis = o.ntri > 0 ? o.ntri : 0;
            T.area = o.area;
            T.wv = o.wv;
            T.pad = 0;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
#pragma unroll
                for (int c = 0; c < 9; ++c) T.tri[q][c] = q < T.nis ? o.tri[q][c / 3][c % 3] : 0.0;
                tri_geo(T.tri[q], T.tg[q]);
#pragma unroll
                for (int c = 0; c < 9; ++c) T.trf[q][c] = (float)T.tri[q][c];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const double a = T.tri[q][c], b = T.tri[q][3 + c], e = T.tri[q][6 + c];
                    T.box[q][c] = __double2float_rd(fmin(a, fmin(b, e)));
                    T.box[q][3 + c] = __double2float_ru(fmax(a, fmax(b, e)));
                }
            }
            tets[tid++] = T;
        }
    }
}

// nodes within +-4 of a pnode that are not pnodes are tagged -1
// (src/GetIsosurfaceAndDistances.F90:322-328); out starts as a copy of ids
__global__ void k_geo_mark(DevGrid g, int npn, const long long* __restrict__ node_of, const int* __restrict__ ids,
                           int* __restrict__ out) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npn; p += gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk(g, node_of[p], &i, &j, &k);
        for (int ks = max(k - 4, 0); ks <= min(k + 4, g.nk - 1); ++ks)
            for (int js = max(j - 4, 0); js <= min(j + 4, g.nj - 1); ++js)
                for (int is = max(i - 4, 0); is <= min(i + 4, g.ni - 1); ++is) {
                    const long long l = gid(g, is, js, ks);
                    if (ids[l] == 0) out[l] = -1;
                }
    }
}

__device__ __forceinline__ float dist3f(const float* a, const float* b) {
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

// a point in both precisions (the FP32 copy for the culling bounds)
struct Pt {
    double d[3];
    float f[3];
    float scale;
};
__device__ __forceinline__ Pt make_pt(double a, double b, double c) {
    Pt p;
    p.d[0] = a; p.d[1] = b; p.d[2] = c;
    p.f[0] = (float)a; p.f[1] = (float)b; p.f[2] = (float)c;
    p.scale = fmaxf(fabsf(p.f[0]), fmaxf(fabsf(p.f[1]), fabsf(p.f[2])));
    return p;
}

// a running value with its FP32 copy for the culling tests, converted
// only when the value changes (conversions run on the FP64 pipe)
struct Run {
    double d;
    float f;
};
__device__ __forceinline__ void set_run(Run& r, double v) {
    if (dbits(v) != dbits(r.d)) { r.d = v; r.f = (float)v; }
}

// the triangles of tetrahedron t against point P (running minimum d); a
// triangle whose bounding box lies beyond d is not evaluated
__device__ __forceinline__ void tet_min(const GeoTet* __restrict__ tets, int t, const Pt& P, Run& d) {
    const GeoTet& T = tets[t];
    const int nis = T.nis;
    if (nis > 0 && T.area > 0.0) {
        for (int q = 0; q < nis; ++q) {
            if (beyond_box(P.f, P.scale, T.box[q], T.box[q] + 3, d.f)) continue;
            set_run(d, run_min(d.d, dist_point_triangle(T.tri[q], T.tg[q], P.d)));
        }
    }
}

// per pnode: the bounding box of every triangle of its K tetrahedra
// (lo.w = 0: none of them has a triangle)
__global__ void k_geo_prad(DevGrid g, int npn, const long long* __restrict__ node_of,
                           const unsigned char* __restrict__ cellbits, const int* __restrict__ tetbase,
                           const GeoTet* __restrict__ tets, const double* __restrict__ x,
                           const double* __restrict__ y, const double* __restrict__ z, float4* __restrict__ pbox) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npn; p += gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk(g, node_of[p], &i, &j, &k);
        float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        float any = 0.0f;
        for_each_tet(g, i, j, k, cellbits, tetbase, [&](int t) {
            const GeoTet& T = tets[t];
            if (T.nis > 0 && T.area > 0.0)
                for (int q = 0; q < T.nis; ++q) {
                    any = 1.0f;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        lo[c] = fminf(lo[c], T.box[q][c]);
                        hi[c] = fmaxf(hi[c], T.box[q][3 + c]);
                    }
                }
        });
        pbox[2 * p] = make_float4(lo[0], lo[1], lo[2], any);
        pbox[2 * p + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    }
}

// true when pnode m's triangles all lie beyond d from P
__device__ __forceinline__ bool pnode_beyond(int m, const Pt& P, float d, const float4* __restrict__ pbox) {
    const float4 a = pbox[2 * m], b = pbox[2 * m + 1];
    if (a.w == 0.0f) return true;
    const float lo[3] = {a.x, a.y, a.z}, hi[3] = {b.x, b.y, b.z};
    return beyond_box(P.f, P.scale, lo, hi, d);
}

// the pnodes' signed distances (src/GetIsosurfaceAndDistances.F90:166-330)
__global__ void k_geo_sd(DevGrid g, int npn, const long long* __restrict__ node_of, const int* __restrict__ ids,
                         const unsigned char* __restrict__ cellbits, const int* __restrict__ tetbase,
                         const GeoTet* __restrict__ tets, const float4* __restrict__ prad,
                         const double* __restrict__ phi, const double* __restrict__ x,
                         const double* __restrict__ y, const double* __restrict__ z, double* __restrict__ sd_out) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npn; p += gridDim.x * blockDim.x) {
        const long long l0 = node_of[p];
        int i, j, k;
        node_ijk(g, l0, &i, &j, &k);
        const Pt P = make_pt(x[l0], y[l0], z[l0]);
        const double s = sgn1(phi[l0]);
        Run dp{10.0, 10.0f};
        double sd = 99.9;
        auto sd_step = [&]() {
            // sd = |sd| + exsign2 (dp - |sd|), then sign(one, phi) * sd
            sd = copysign(mag_step(fabs(sd), dp.d), s);
        };
        for (int ks = max(k - 4, 0); ks <= min(k + 4, g.nk - 1); ++ks)
            for (int js = max(j - 4, 0); js <= min(j + 4, g.nj - 1); ++js)
                for (int is = max(i - 4, 0); is <= min(i + 4, g.ni - 1); ++is) {
                    const int m = ids[gid(g, is, js, ks)] - 1;
                    if (m < 0) continue;
                    // every triangle of this pnode beyond dp: dp stays, the
                    // signed distance update still runs once per tetrahedron
                    if (pnode_beyond(m, P, dp.f, prad)) {
                        for_each_tet(g, is, js, ks, cellbits, tetbase, [&](int) { sd_step(); });
                        continue;
                    }
                    for_each_tet(g, is, js, ks, cellbits, tetbase, [&](int t) {
                        tet_min(tets, t, P, dp);
                        sd_step();
                    });
                }
        sd_out[p] = sd;
    }
}

// LocalVolumeVariation, src/TetrahedronMethods.F90:2390-2437
__device__ double local_dv(double eta, const double (&V)[4][3], const double (&ph)[4], double v0, unsigned* err) {
    double a[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) a[q] = ph[q] + eta;
    MT o;
    marching_full(V, a, o, false, err);
    return v0 - o.wv;
}

__device__ __forceinline__ void tet_vertices(const GeoTet& T, const long long* __restrict__ node_of,
                                             const double* __restrict__ x, const double* __restrict__ y,
                                             const double* __restrict__ z, double (&V)[4][3]) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const long long l = node_of[T.v[q]];
        V[q][0] = x[l]; V[q][1] = y[l]; V[q][2] = z[l];
    }
}

// PiecewiseConstantFunction + SecantMethodLocalCorrection,
// src/PiecewiseConstantFunction.F90:1-102, src/TetrahedronMethods.F90:2439-2588
__global__ void k_geo_secant(int ntet, const GeoTet* __restrict__ tets, const long long* __restrict__ node_of,
                             const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ z, const double* __restrict__ sd, double tol,
                             double* __restrict__ eta, unsigned* err) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntet; t += gridDim.x * blockDim.x) {
        const GeoTet T = tets[t];
        double V[4][3], ph[4];
        tet_vertices(T, node_of, x, y, z, V);
#pragma unroll
        for (int q = 0; q < 4; ++q) ph[q] = sd[T.v[q]];
        MT o;
        marching_full(V, ph, o, true, err);
        const double vol0 = T.wv, dv0 = vol0 - o.wv;
        double res = 0.0;
        if (!(fabs(dv0) < tol)) {
            double x0 = o.area > kEpsSims ? dv0 / o.area : 0.0;
            double x1 = T.area > kEpsSims ? dv0 / T.area : 0.0;
            double f0 = local_dv(x0, V, ph, vol0, err);
            double f1 = local_dv(x1, V, ph, vol0, err);
            if (fabs(f0) < tol || fabs(f1) < tol) {
                res = fabs(f1) < fabs(f0) ? x1 : x0;
            } else {
                bool conv = false;
                double x2 = 0.0;
                for (int it = 1; it <= 40; ++it) {
                    if (fabs(f1 - f0) < kEpsSims) break;
                    x2 = x1 - f1 * (x1 - x0) / (f1 - f0);
                    x0 = x1; x1 = x2; f0 = f1;
                    f1 = local_dv(x1, V, ph, vol0, err);
                    if (fabs(f1) < tol) { conv = true; break; }
                }
                if (fabs(f1) > dv0) x2 = 0.0;
                res = conv ? x2 : 0.0;
            }
        }
        eta[t] = res;
    }
}

// OrthogonalProjection, src/OrthogonalProjection.F90:1-49
__global__ void k_geo_xi(DevGrid g, int npn, const long long* __restrict__ node_of,
                         const unsigned char* __restrict__ cellbits, const int* __restrict__ tetbase,
                         const double* __restrict__ eta, double* __restrict__ xi) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npn; p += gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk(g, node_of[p], &i, &j, &k);
        int na = 0;
        for_each_tet(g, i, j, k, cellbits, tetbase, [&](int) { ++na; });
        const double dn = (double)na;
        double s = 0.0;
        for_each_tet(g, i, j, k, cellbits, tetbase, [&](int t) { s = s + eta[t] / dn; });
        xi[p] = s;
    }
}

// funcv's per-tetrahedron volume of phi* + C xi (src/NewtonRaphsonSolver.F90)
// and a per-block partial sum in fixed order
__global__ void __launch_bounds__(kThreads) k_geo_funcv(int ntet, const GeoTet* __restrict__ tets,
                                                        const long long* __restrict__ node_of,
                                                        const double* __restrict__ x, const double* __restrict__ y,
                                                        const double* __restrict__ z,
                                                        const double* __restrict__ sd,
                                                        const double* __restrict__ xi, double C,
                                                        double* __restrict__ part, unsigned* err) {
    __shared__ double red[kThreads];
    double acc = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntet; t += gridDim.x * blockDim.x) {
        const GeoTet T = tets[t];
        double V[4][3], a[4];
        tet_vertices(T, node_of, x, y, z, V);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double s = sd[T.v[q]], ca = C * xi[T.v[q]];
            a[q] = s + ca / 2.0 * fabs(sgn1(s) + sgn1(s + ca));
        }
        MT o;
        marching_full(V, a, o, false, err);
        acc += o.wv;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(kThreads) k_geo_sum(int n, const double* __restrict__ part,
                                                      double* __restrict__ out) {
    __shared__ double red[kThreads];
    double acc = 0.0;
    for (int b = threadIdx.x; b < n; b += kThreads) acc += part[b];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// NeighboursPhiCorrection on the pnodes (src/NeighboursPhiCorrection.F90:142-184)
__global__ void k_geo_pnode_phi(int npn, const long long* __restrict__ node_of, const double* __restrict__ sd,
                                const double* __restrict__ xi, double C, double* __restrict__ pc) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npn; p += gridDim.x * blockDim.x) {
        const double s = sd[p], xv = xi[p];
        const double pcf = fabs(sgn1(s) + sgn1(s + C * xv)) / 2.0;
        const double aux = pcf * C * xv;
        pc[node_of[p]] = s + aux;
    }
}

// NeighboursPhiCorrection on the -1 nodes (src/NeighboursPhiCorrection.F90:186-343).
//
// One warp per node.  The node's result is a sequential chain over the
// pnodes of its +-4 box, in the reference's order: per pnode a running
// minimum dp over the triangles of its K tetrahedra (reset to 10), and
// after each tetrahedron |v| <- |v| + exsign2 (dp - |v|).  Its last bits
// depend on that order, so the chain itself runs in order, uniformly on
// all lanes; what the lanes share out is the FP64 work inside it, the
// point-triangle distances.  Pnodes that can still change v (the same tests
// as the chain: the box of all their triangles, then the triangles' own
// boxes, against the current |v|) are queued with their tetrahedra and
// triangles; once the queue holds a lane-full of triangles, the lanes
// evaluate all of them, and the chain is replayed over the queued pnodes,
// each test made again with the v of that moment.  v only decreases, so a
// pnode skipped when queued would be skipped in the chain too; one queued
// but skipped in the replay, or a triangle culled there by the running
// minimum, only cost a wasted evaluation.  Every value the replay uses is
// the one the sequential chain computes.
constexpr int kQN = 16;    // queued pnodes
constexpr int kQT = 160;   // queued tetrahedra
constexpr int kQP = 96;    // queued triangles
constexpr int kQFlush = 32;

struct NeighQueue {
    int nn, nt, np;
    int nm[kQN];           // pnode ids
    int nstart[kQN + 1];   // first tetrahedron slot of each queued pnode
    int tet[kQT];          // tetrahedron ids, in order
    int tp[kQT + 1];       // first triangle slot of each tetrahedron slot
    int ptet[kQP];         // triangle slot -> tetrahedron id
    unsigned char pq[kQP]; // triangle slot -> triangle 0/1 of that tetrahedron
    double da[kQP];        // the distances
};

constexpr int kNeighWarps = 4;

__global__ void __launch_bounds__(32 * kNeighWarps) k_geo_neigh(
        DevGrid g, const int* __restrict__ ids, const unsigned char* __restrict__ cellbits,
        const int* __restrict__ tetbase, const GeoTet* __restrict__ tets, const float4* __restrict__ prad,
        const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
        double* __restrict__ pc, int nsec, const long long* __restrict__ second) {
    __shared__ NeighQueue qs[kNeighWarps];
    NeighQueue& Q = qs[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * kNeighWarps;
    for (int c = blockIdx.x * kNeighWarps + (threadIdx.x >> 5); c < nsec; c += nwarps) {
        const long long l0 = second[c];
        int i, j, k;
        node_ijk(g, l0, &i, &j, &k);
        const Pt P = make_pt(x[l0], y[l0], z[l0]);
        double v = pc[l0];
        float vf = (float)fabs(v);   // |v| in FP32 for the culling tests
        int nn = 0, nt = 0, np = 0;  // uniform copies of the queue sizes

        // the triangles of queued pnode slot n all beyond af (pnode box first)
        auto all_beyond = [&](int n, float af) -> bool {
            if (pnode_beyond(Q.nm[n], P, af, prad)) return true;
            for (int s2 = Q.nstart[n]; s2 < Q.nstart[n + 1]; ++s2)
                for (int p = Q.tp[s2]; p < Q.tp[s2 + 1]; ++p) {
                    const GeoTet& T = tets[Q.ptet[p]];
                    if (!beyond_box(P.f, P.scale, T.box[Q.pq[p]], T.box[Q.pq[p]] + 3, af)) return false;
                }
            return true;
        };
        auto flush = [&]() {
            __syncwarp();
            for (int p = lane; p < np; p += 32) {
                const GeoTet& T = tets[Q.ptet[p]];
                const int q = Q.pq[p];
                Q.da[p] = dist_point_triangle(T.tri[q], T.tg[q], P.d);
            }
            __syncwarp();
            for (int n = 0; n < nn; ++n) {
                if (all_beyond(n, vf)) continue;
                Run dp{10.0, 10.0f};
                for (int s2 = Q.nstart[n]; s2 < Q.nstart[n + 1]; ++s2) {
                    for (int p = Q.tp[s2]; p < Q.tp[s2 + 1]; ++p) {
                        const GeoTet& T = tets[Q.ptet[p]];
                        if (beyond_box(P.f, P.scale, T.box[Q.pq[p]], T.box[Q.pq[p]] + 3, dp.f)) continue;
                        set_run(dp, run_min(dp.d, Q.da[p]));
                    }
                    // |v| + exsign2 (dp - |v|), with the sign of v
                    const double av = fabs(v), nv2 = mag_step(av, dp.d);
                    if (dbits(nv2) != dbits(av)) vf = (float)nv2;
                    v = copysign(nv2, v);
                }
            }
            __syncwarp();
            nn = nt = np = 0;
        };

        for (int ks = max(k - 4, 0); ks <= min(k + 4, g.nk - 1); ++ks)
            for (int js = max(j - 4, 0); js <= min(j + 4, g.nj - 1); ++js)
                for (int is = max(i - 4, 0); is <= min(i + 4, g.ni - 1); ++is) {
                    const int m = ids[gid(g, is, js, ks)] - 1;
                    if (m < 0) continue;
                    if (pnode_beyond(m, P, vf, prad)) continue;
                    if (nn == kQN || nt > kQT - 24 || np > kQP - 48) flush();
                    // queue the pnode's tetrahedra and triangles (every lane
                    // writes the same values).  A triangle is left out when
                    // the chain will cull it for sure: ub bounds the
                    // running minimum from above (the reference's distance is
                    // at most the distance to each vertex, here in FP32
                    // with a margin, and whether an earlier triangle is
                    // evaluated or culled the minimum stays below it), and
                    // the cull test only gets stricter as the minimum falls.
                    Q.nm[nn] = m;
                    Q.nstart[nn] = nt;
                    float ub = 10.0f;
                    for_each_tet(g, is, js, ks, cellbits, tetbase, [&](int t) {
                        const GeoTet& T = tets[t];
                        const int ntri = (T.nis > 0 && T.area > 0.0) ? T.nis : 0;
                        Q.tet[nt] = t;
                        Q.tp[nt] = np;
                        for (int q = 0; q < ntri; ++q) {
                            if (!beyond_box(P.f, P.scale, T.box[q], T.box[q] + 3, ub)) {
                                Q.ptet[np] = t;
                                Q.pq[np] = (unsigned char)q;
                                ++np;
                            }
                            float u = fminf(dist3f(P.f, T.trf[q]), fminf(dist3f(P.f, T.trf[q] + 3),
                                                                           dist3f(P.f, T.trf[q] + 6)));
                            u = u + 1.0e-5f * (u + P.scale) + 1.0e-30f;
                            ub = fminf(ub, u);
                        }
                        ++nt;
                    });
                    Q.tp[nt] = np;
                    Q.nstart[nn + 1] = nt;
                    __syncwarp();
                    if (all_beyond(nn, vf)) {  // not near: drop it again
                        nt = Q.nstart[nn];
                        np = Q.tp[nt];
                        continue;
                    }
                    ++nn;
                    if (np >= kQFlush) flush();
                }
        if (nn) flush();
        if (lane == 0) pc[l0] = v;
    }
}

// levelsetmethod's phicorrected before the geometric step
// (src/levelsetmethod.F90:303-304): -9.9 where phi < -epsilon, 9.9 where
// phi > epsilon, the value in place elsewhere
__global__ void k_geo_seed(long long n, const double* __restrict__ phi, double* __restrict__ pc) {
    for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < n;
         l += (long long)gridDim.x * blockDim.x) {
        const double f = phi[l];
        if (f < -kEpsSims) pc[l] = -9.9;
        if (f > kEpsSims) pc[l] = 9.9;
    }
}

int grid_for(long long n, int bs = kThreads) {
    long long b = (n + bs - 1) / bs;
    return (int)(b < 1 ? 1 : (b > 152LL * 64 ? 152LL * 64 : b));
}

}  // namespace

// ------------------------------------------------------------ host driver

void launch_geo_seed(long long n, const double* phi, double* pc, cudaStream_t s) {
    ProfScope ps("k_geo_seed", s);
    k_geo_seed<<<grid_for(n), kThreads, 0, s>>>(n, phi, pc);
}

#define GEO_CU(call)                                   \
    do {                                               \
        cudaError_t e_ = (call);                       \
        if (e_ != cudaSuccess) return e_;              \
    } while (0)

cudaError_t geo_reinit(const DevGrid& g, const double* phi0, const double* x, const double* y, const double* z,
                       double target, int gmc, double tol, double* pc, int* tag, GeoAlloc alloc, void* actx,
                       unsigned* d_err, int* d_count, GeoInfo* info, cudaStream_t s) {
    const long long n = (long long)g.ni * g.nj * g.nk;
    const int ntiles = (int)((n + kTile - 1) / kTile);
    cudaError_t e = cudaSuccess;
    auto* cellbits = static_cast<unsigned char*>(alloc(actx, "geo_cellbits", (size_t)n, &e));
    GEO_CU(e);
    auto* ids = static_cast<int*>(alloc(actx, "geo_ids", 4 * (size_t)n, &e));
    GEO_CU(e);
    auto* tetbase = static_cast<int*>(alloc(actx, "geo_tetbase", 4 * (size_t)n, &e));
    GEO_CU(e);
    auto* tiles = static_cast<int*>(alloc(actx, "geo_tiles", 4 * (size_t)ntiles + 16, &e));
    GEO_CU(e);
    // 1. cells: K-tetrahedra bits and pnode flags (ids holds the flags first)
    GEO_CU(cudaMemsetAsync(cellbits, 0, (size_t)n, s));
    GEO_CU(cudaMemsetAsync(ids, 0, 4 * (size_t)n, s));
    {
        ProfScope ps("k_geo_cells", s);
        k_geo_cells<<<grid_for(n), kThreads, 0, s>>>(g, phi0, cellbits, ids);
        GEO_CU(cudaGetLastError());
    }
    // 2. pnode ids: the flags -> tag (scratch), scanned back into ids
    GEO_CU(cudaMemcpyAsync(tag, ids, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s));
    int counts[2] = {0, 0};
    {
        ProfScope ps("k_geo_scan", s);
        k_scan_tiles<0><<<ntiles, kThreads, 0, s>>>(n, tag, tiles);
        k_scan_top<<<1, kThreads, 0, s>>>(ntiles, tiles, d_count);
        GEO_CU(cudaGetLastError());
    }
    GEO_CU(cudaMemcpyAsync(&counts[0], d_count, sizeof(int), cudaMemcpyDeviceToHost, s));
    GEO_CU(cudaStreamSynchronize(s));
    const int npn = counts[0];
    auto* node_of = static_cast<long long*>(alloc(actx, "geo_node_of", 8 * (size_t)(npn + 1), &e));
    GEO_CU(e);
    {
        ProfScope ps("k_geo_scan", s);
        k_scan_apply<0><<<ntiles, kThreads, 0, s>>>(n, tag, tiles, ids, node_of);
        // 3. K-tetrahedra ids per cell
        k_scan_tiles<1><<<ntiles, kThreads, 0, s>>>(n, cellbits, tiles);
        k_scan_top<<<1, kThreads, 0, s>>>(ntiles, tiles, d_count + 1);
        k_scan_apply<1><<<ntiles, kThreads, 0, s>>>(n, cellbits, tiles, tetbase, nullptr);
        GEO_CU(cudaGetLastError());
    }
    GEO_CU(cudaMemcpyAsync(&counts[1], d_count + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    GEO_CU(cudaStreamSynchronize(s));
    const int ntet = counts[1];
    info->nnodes = npn;
    info->ntetrahedra = ntet;
    info->nsecond = 0;
    info->newton_iterations = 0;
    info->newton_converged = 0;
    info->C = 0.0;
    GEO_CU(cudaMemcpyAsync(tag, ids, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s));
    if (npn == 0) return cudaSuccess;
    auto* tets = static_cast<GeoTet*>(alloc(actx, "geo_tets", sizeof(GeoTet) * (size_t)(ntet + 1), &e));
    GEO_CU(e);
    auto* sd = static_cast<double*>(alloc(actx, "geo_sd", 8 * (size_t)npn, &e));
    GEO_CU(e);
    auto* xi = static_cast<double*>(alloc(actx, "geo_xi", 8 * (size_t)npn, &e));
    GEO_CU(e);
    auto* prad = static_cast<float4*>(alloc(actx, "geo_prad", 32 * (size_t)npn, &e));
    GEO_CU(e);
    {
        ProfScope ps("k_geo_tets", s);
        k_geo_tets<<<grid_for(n), kThreads, 0, s>>>(g, phi0, x, y, z, cellbits, tetbase, ids, tets, d_err);
        GEO_CU(cudaGetLastError());
    }
    {
        ProfScope ps("k_geo_mark", s);
        k_geo_mark<<<grid_for(npn), kThreads, 0, s>>>(g, npn, node_of, ids, tag);
        GEO_CU(cudaGetLastError());
    }
    {
        ProfScope ps("k_geo_prad", s);
        k_geo_prad<<<grid_for(npn), kThreads, 0, s>>>(g, npn, node_of, cellbits, tetbase, tets, x, y, z, prad);
        GEO_CU(cudaGetLastError());
    }
    {
        ProfScope ps("k_geo_sd", s);
        k_geo_sd<<<grid_for(npn), 128, 0, s>>>(g, npn, node_of, ids, cellbits, tetbase, tets, prad, phi0, x, y, z,
                                               sd);
        GEO_CU(cudaGetLastError());
    }
    GEO_CU(cudaMemsetAsync(xi, 0, 8 * (size_t)npn, s));
    double C = 0.0;
    if (gmc && ntet > 0) {
        auto* eta = static_cast<double*>(alloc(actx, "geo_eta", 8 * (size_t)ntet, &e));
        GEO_CU(e);
        const int nb = grid_for(ntet);
        auto* part = static_cast<double*>(alloc(actx, "geo_part", 8 * (size_t)nb + 64, &e));
        GEO_CU(e);
        {
            ProfScope ps("k_geo_secant", s);
            k_geo_secant<<<nb, kThreads, 0, s>>>(ntet, tets, node_of, x, y, z, sd, tol / 1000.0, eta, d_err);
            GEO_CU(cudaGetLastError());
        }
        {
            ProfScope ps("k_geo_xi", s);
            k_geo_xi<<<grid_for(npn), kThreads, 0, s>>>(g, npn, node_of, cellbits, tetbase, eta, xi);
            GEO_CU(cudaGetLastError());
        }
        double* d_sum = part + nb;
        cudaError_t fe = cudaSuccess;
        auto funcv = [&](double c) -> double {
            double tot = 0.0;
            if (fe != cudaSuccess) return 0.0;
            {
                ProfScope ps("k_geo_funcv", s);
                k_geo_funcv<<<nb, kThreads, 0, s>>>(ntet, tets, node_of, x, y, z, sd, xi, c, part, d_err);
                k_geo_sum<<<1, kThreads, 0, s>>>(nb, part, d_sum);
            }
            fe = cudaGetLastError();
            if (fe == cudaSuccess) fe = cudaMemcpyAsync(&tot, d_sum, sizeof(double), cudaMemcpyDeviceToHost, s);
            if (fe == cudaSuccess) fe = cudaStreamSynchronize(s);
            return target - tot;
        };
        int its = 0;
        bool conv = false;
        C = geo_newton(funcv, tol, &its, &conv);
        GEO_CU(fe);
        info->newton_iterations = its;
        info->newton_converged = conv ? 1 : 0;
        info->C = C;
    }
    {
        ProfScope ps("k_geo_pnode_phi", s);
        k_geo_pnode_phi<<<grid_for(npn), kThreads, 0, s>>>(npn, node_of, sd, xi, C, pc);
        GEO_CU(cudaGetLastError());
    }
    // the nodes tagged -1, listed in order
    {
        ProfScope ps("k_geo_scan", s);
        k_scan_tiles<2><<<ntiles, kThreads, 0, s>>>(n, tag, tiles);
        k_scan_top<<<1, kThreads, 0, s>>>(ntiles, tiles, d_count + 2);
        GEO_CU(cudaGetLastError());
    }
    int ns = 0;
    GEO_CU(cudaMemcpyAsync(&ns, d_count + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    GEO_CU(cudaStreamSynchronize(s));
    info->nsecond = ns;
    if (ns == 0) return cudaSuccess;
    auto* second = static_cast<long long*>(alloc(actx, "geo_second", 8 * (size_t)ns, &e));
    GEO_CU(e);
    {
        ProfScope ps("k_geo_scan", s);
        k_scan_apply<2><<<ntiles, kThreads, 0, s>>>(n, tag, tiles, nullptr, second);
        GEO_CU(cudaGetLastError());
    }
    {
        ProfScope ps("k_geo_neigh", s);
        k_geo_neigh<<<grid_for(ns, kNeighWarps), 32 * kNeighWarps, 0, s>>>(g, ids, cellbits, tetbase, tets, prad, x,
                                                                            y, z, pc, ns, second);
        GEO_CU(cudaGetLastError());
    }
    GEO_CU(cudaStreamSynchronize(s));
    return cudaSuccess;
}

}  // namespace lsm
