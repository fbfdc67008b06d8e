// lsm_volume_dev.cuh -- FP64 device functions of the reference's water
// volume: the 4x4 determinant, tetrahedron volume, marching tetrahedra with
// the reference's case tables, the Davies-Salmond hexahedron volume and the
// six-tetrahedra cell analysis.  Shared by the FP64 volume kernels and the
// batched path; a translation unit that needs the reference's rounding
// compiles it with --fmad=false.
#pragma once

#include <cuda_runtime.h>

#include "lsm_common.cuh"

namespace lsm {
namespace {

// M44Det, src/TetrahedronMethods.F90:1698-1720, specialised to a 4th column
// of ones (A(r,4) = 1 multiplies exactly)
__device__ __forceinline__ double det_ones(const double* a, const double* b, const double* c, const double* d) {
    // rows a, b, c, d; A(r,1:3) = row, A(r,4) = 1
    const double A11 = a[0], A12 = a[1], A13 = a[2];
    const double A21 = b[0], A22 = b[1], A23 = b[2];
    const double A31 = c[0], A32 = c[1], A33 = c[2];
    const double A41 = d[0], A42 = d[1], A43 = d[2];
    const double A14 = 1.0, A24 = 1.0, A34 = 1.0, A44 = 1.0;
    const double t1 = A11 * (A22 * (A33 * A44 - A34 * A43) + A23 * (A34 * A42 - A32 * A44) +
                             A24 * (A32 * A43 - A33 * A42));
    const double t2 = A12 * (A21 * (A33 * A44 - A34 * A43) + A23 * (A34 * A41 - A31 * A44) +
                             A24 * (A31 * A43 - A33 * A41));
    const double t3 = A13 * (A21 * (A32 * A44 - A34 * A42) + A22 * (A34 * A41 - A31 * A44) +
                             A24 * (A31 * A42 - A32 * A41));
    const double t4 = A14 * (A21 * (A32 * A43 - A33 * A42) + A22 * (A33 * A41 - A31 * A43) +
                             A23 * (A31 * A42 - A32 * A41));
    return t1 - t2 + t3 - t4;
}

// GetTetrahedronVolume, src/TetrahedronMethods.F90:666-688: |M44Det| / 6
__device__ __forceinline__ double tetvol_ref(const double* a, const double* b, const double* c, const double* d) {
    return 1.0 / 6.0 * fabs(det_ones(a, b, c, d));
}

// the same volume as |((b-a) x (c-a)) . (d-a)| / 6: 17 FP64 operations
// instead of ~40, used where the reference's rounding is not required
__device__ __forceinline__ double tetvol_fast(const double* a, const double* b, const double* c, const double* d) {
    const double u0 = b[0] - a[0], u1 = b[1] - a[1], u2 = b[2] - a[2];
    const double v0 = c[0] - a[0], v1 = c[1] - a[1], v2 = c[2] - a[2];
    const double w0 = d[0] - a[0], w1 = d[1] - a[1], w2 = d[2] - a[2];
    const double t = w0 * (u1 * v2 - u2 * v1) + w1 * (u2 * v0 - u0 * v2) + w2 * (u0 * v1 - u1 * v0);
    return fabs(t) * (1.0 / 6.0);
}

template <bool Ref>
__device__ __forceinline__ double tetvol(const double* a, const double* b, const double* c, const double* d) {
    return Ref ? tetvol_ref(a, b, c, d) : tetvol_fast(a, b, c, d);
}

__constant__ int c_edge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
__constant__ int c_edge_flags[16] = {0x00, 0x0d, 0x13, 0x1e, 0x26, 0x2b, 0x35, 0x38,
                                     0x38, 0x35, 0x2b, 0x26, 0x1e, 0x13, 0x0d, 0x00};
__constant__ int c_tets[6][4] = {{0, 5, 1, 6}, {0, 1, 2, 6}, {0, 2, 3, 6},
                                 {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}};

// GetWaterVolume, src/TetrahedronMethods.F90:710-954
template <bool Ref>
__device__ double water_volume(const double (&V)[4][3], const double (&E)[6][3], int fi, unsigned* err) {
    const double TV = tetvol<Ref>(V[0], V[1], V[2], V[3]);
    double AV, r = 0.0;
    switch (fi + 1) {
    case 2: case 15:
        AV = tetvol<Ref>(V[0], E[0], E[2], E[3]);
        r = (fi + 1 == 2) ? TV - AV : AV; break;
    case 3: case 14:
        AV = tetvol<Ref>(V[1], E[0], E[1], E[4]);
        r = (fi + 1 == 3) ? TV - AV : AV; break;
    case 4: case 13:
        AV = tetvol<Ref>(V[0], E[2], E[3], E[4]) + tetvol<Ref>(V[0], E[1], E[2], E[4]) + tetvol<Ref>(V[0], V[1], E[1], E[4]);
        r = (fi + 1 == 4) ? TV - AV : AV; break;
    case 5: case 12:
        AV = tetvol<Ref>(V[2], E[1], E[2], E[5]);
        r = (fi + 1 == 5) ? TV - AV : AV; break;
    case 6: case 11:
        AV = tetvol<Ref>(V[0], E[0], E[1], E[5]) + tetvol<Ref>(V[0], E[0], E[3], E[5]) + tetvol<Ref>(V[0], V[2], E[1], E[5]);
        r = (fi + 1 == 6) ? TV - AV : AV; break;
    case 7: case 10:
        AV = tetvol<Ref>(V[1], E[0], E[2], E[5]) + tetvol<Ref>(V[1], E[0], E[4], E[5]) + tetvol<Ref>(V[1], V[2], E[2], E[5]);
        r = (fi + 1 == 7) ? TV - AV : AV; break;
    case 8: case 9:
        AV = tetvol<Ref>(V[3], E[3], E[4], E[5]);
        r = (fi + 1 == 8) ? AV : TV - AV; break;
    default: r = 0.0;
    }
    if (r < -kEpsSims && err) atomicOr(err, (unsigned)kErrNegativeVolume);
    return r;
}

// MarchingTetrahedron (its water-volume output), src/TetrahedronMethods.F90:26-664
template <bool Ref>
__device__ double marching_tet(const double (&V)[4][3], const double (&ph)[4], unsigned* err) {
    int s[4], nz = 0;
    bool allp = true, alln = true, allge = true, allle = true;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        s[v] = ph[v] > kTinyD ? 1 : (ph[v] < -kTinyD ? -1 : 0);
        allp &= s[v] == 1; alln &= s[v] == -1; nz += s[v] == 0;
        allge &= s[v] >= 0; allle &= s[v] <= 0;
    }
    if (allp) return tetvol<Ref>(V[0], V[1], V[2], V[3]);
    if (alln) return 0.0;
    int fi = 0;
    if (nz > 0 && (allge || allle)) {
        int water = -1;  // -1: fall through (four zero vertices)
        if (nz == 1) {
            if (s[0] == 0) water = s[1] == 1;
            else if (s[1] == 0) water = s[0] == 1;
            else if (s[2] == 0) water = s[0] == 1;
            else water = s[0] == 1;
        } else if (nz == 2) {
            if (s[0] == 0 && s[1] == 0) water = s[2] == 1;
            else if (s[1] == 0 && s[2] == 0) water = s[0] == 1;
            else if (s[2] == 0 && s[0] == 0) water = s[1] == 1;
            else if (s[0] == 0 && s[3] == 0) water = s[1] == 1;
            else if (s[1] == 0 && s[3] == 0) water = s[0] == 1;
            else water = s[0] == 1;
        } else if (nz == 3) {
            for (int v = 0; v < 4; ++v)
                if (s[v] != 0) { water = s[v] == 1; break; }
        }
        if (water >= 0) return water ? tetvol<Ref>(V[0], V[1], V[2], V[3]) : 0.0;
    } else {
#pragma unroll
        for (int v = 0; v < 4; ++v)
            if (s[v] == -1) fi |= 1 << v;
    }
    double wv = 0.0;
    if (fi == 0) wv = tetvol<Ref>(V[0], V[1], V[2], V[3]);
    const int ef = c_edge_flags[fi];
    if (ef == 0) return wv;
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
    return water_volume<Ref>(V, E, fi, err);
}

__device__ __forceinline__ double dot3(const double* a, const double* b) {
    double s = 0.0;
    s = s + a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}
__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// HexahedronVolume (Davies & Salmond 1985), src/TetrahedronMethods.F90:1724-1793
__device__ double hex_volume(const double (&C)[8][3]) {
    double AC[3], AF[3], AH[3], BE[3], CH[3], DB[3], ED[3], FC[3], GA[3], GB[3], GC[3], GD[3], GE[3], GF[3],
        GH[3], HF[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        AC[c] = C[2][c] - C[0][c]; AF[c] = C[5][c] - C[0][c]; AH[c] = C[7][c] - C[0][c];
        BE[c] = C[4][c] - C[1][c]; CH[c] = C[7][c] - C[2][c]; DB[c] = C[1][c] - C[3][c];
        ED[c] = C[3][c] - C[4][c]; FC[c] = C[2][c] - C[5][c];
        GA[c] = C[0][c] - C[6][c]; GB[c] = C[1][c] - C[6][c]; GC[c] = C[2][c] - C[6][c];
        GD[c] = C[3][c] - C[6][c]; GE[c] = C[4][c] - C[6][c]; GF[c] = C[5][c] - C[6][c];
        GH[c] = C[7][c] - C[6][c]; HF[c] = C[5][c] - C[7][c];
    }
    double s1[3], s2[3], s3[3], x[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) { s1[c] = GA[c] + GB[c]; s2[c] = GA[c] + GE[c]; s3[c] = GA[c] + GD[c]; }
    double S;
    cross3(DB, AC, x); S = dot3(s1, x);
    cross3(BE, AF, x); S = S + dot3(s2, x);
    cross3(ED, AH, x); S = S + dot3(s3, x);
    cross3(HF, GE, x); S = S + dot3(GF, x);
    cross3(CH, GD, x); S = S + dot3(GH, x);
    cross3(FC, GB, x); S = S + dot3(GC, x);
    return -(1.0 / 12.0 * S);
}

// CellAnalysis with TriangulationCase 1, src/TetrahedronMethods.F90:1823-2121
template <bool Ref>
__device__ void cell_analysis(const double (&P)[8], const double (&C)[8][3], double* K, double* S,
                              unsigned* err) {
    double k = 0.0, s2 = 0.0;
    bool pcc = false;
#pragma unroll
    for (int v = 0; v < 8; ++v) pcc |= fabs(P[v]) < kEpsSims;
    if (!pcc) {
        const double sg = copysign(1.0, P[0]);
        for (int v = 1; v < 8; ++v)
            if (sg * P[v] < 0.0) { pcc = true; break; }
    }
    if (pcc) {
        for (int t = 0; t < 6; ++t) {
            bool pct = false, second = true;
            const double pa = P[c_tets[t][0]];
            if (pa <= kEpsSims) second = false;
            if (fabs(pa) < kEpsSims) pct = true;
            const double sg = copysign(1.0, pa);
            for (int v = 1; v < 4; ++v) {
                const double pb = P[c_tets[t][v]];
                if (sg * pb < 0.0 || fabs(pb) < kEpsSims) {
                    if (pb <= kEpsSims) second = false;
                    pct = true;
                }
            }
            double V[4][3], ph[4];
            for (int v = 0; v < 4; ++v) {
                const int cv = c_tets[t][v];
                V[v][0] = C[cv][0]; V[v][1] = C[cv][1]; V[v][2] = C[cv][2];
                ph[v] = P[cv];
            }
            if (pct) k = k + marching_tet<Ref>(V, ph, err);
            if (second && !pct) s2 = s2 + tetvol<Ref>(V[0], V[1], V[2], V[3]);
        }
    }
    *K = k; *S = s2;
}

}  // namespace
}  // namespace lsm
