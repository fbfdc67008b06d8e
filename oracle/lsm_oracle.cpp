/*
 * lsm_oracle.cpp -- TEST INFRASTRUCTURE ONLY.  CPU FP64 restatement of the
 * level-set transport routines of NS-LSM-Single-Phase, used as the parity
 * checker for the CUDA path and as the timed CPU baseline.  Nothing in the
 * product links or calls this file.
 *
 * Parity pinning: the reference is Fortran 90 + MPI and no Fortran compiler
 * exists in the build image, and the reference ships no tests, golden files
 * or recorded outputs.  This restatement is therefore pinned only by
 * analytic known-answer tests (tests/test_oracle_kat.py) and by hand-checked
 * vectors derived from the reference formulas: PARITY UNPINNED against
 * outputs of the reference itself.
 *
 * Rules followed so that the arithmetic is the reference's:
 *  - FP64 everywhere (rdf = selected_real_kind(p=7) is REAL(8),
 *    src/precision.F90:11);
 *  - Fortran left-to-right association of + - * /, parentheses kept;
 *  - x**2, x**two (real 2.0) become x*x; x**(-1) becomes 1/x;
 *  - compiled with -ffp-contract=off (gfortran on x86-64 emits no FMA);
 *  - constants that the Fortran folds at compile time (one/three, ...) are
 *    folded the same way (IEEE division of the literals).
 * Arrays are column-major with the grid's explicit bounds; vector fields are
 * (1:3, i, j, k) with the component fastest.
 *
 * Built twice from this one source (oracle/Makefile): serial
 * (liblsm_oracle.so, the checker) and with OpenMP over the outer loop of each
 * pass (liblsm_oracle_omp.so, the multi-core CPU timing baseline).
 */
#include "lsm_c.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = 3.141592653589793;      /* src/precision.F90:51 */
const double kEpsSims = DBL_EPSILON;       /* epsilon(one), src/precision.F90:62 */
const double kTiny = DBL_MIN;              /* tiny(eps_sims), src/TetrahedronMethods.F90:189 */

struct Grid {
    int il, iu, jl, ju, kl, ku, igp, jgp, kgp;
    long ni, nj, nk, n;
    double dc, de, dz;
    bool pb, pf, pl, pr, pd, pu; /* physical back(i1) front(im) left(j1) right(jm) down(k1) up(km) */
    /* non-ghost node range */
    int ia, ib, ja, jb, ka, kb;
    explicit Grid(const lsm_grid* g) {
        il = g->il; iu = g->iu; jl = g->jl; ju = g->ju; kl = g->kl; ku = g->ku;
        igp = g->igp; jgp = g->jgp; kgp = g->kgp;
        ni = iu - il + 1; nj = ju - jl + 1; nk = ku - kl + 1; n = ni * nj * nk;
        dc = g->dc; de = g->de; dz = g->dz;
        pb = g->physical_face[0] != 0; pf = g->physical_face[1] != 0;
        pl = g->physical_face[2] != 0; pr = g->physical_face[3] != 0;
        pd = g->physical_face[4] != 0; pu = g->physical_face[5] != 0;
        ia = il + igp; ib = iu - igp; ja = jl + jgp; jb = ju - jgp; ka = kl + kgp; kb = ku - kgp;
    }
    inline long id(int i, int j, int k) const {
        return (long)(i - il) + ni * ((long)(j - jl) + nj * (long)(k - kl));
    }
};

int check_grid(const lsm_grid* g) {
    if (!g) return LSM_ERR_NULL;
    if (g->igp < 0 || g->jgp < 0 || g->kgp < 0) return LSM_ERR_BAD_SHAPE;
    int ni = g->iu - g->il + 1 - 2 * g->igp, nj = g->ju - g->jl + 1 - 2 * g->jgp,
        nk = g->ku - g->kl + 1 - 2 * g->kgp;
    if (ni < 4 || nj < 4 || nk < 4) return LSM_ERR_BAD_SHAPE;
    for (int f = 0; f < 3; ++f) {
        int gp = f == 0 ? g->igp : (f == 1 ? g->jgp : g->kgp);
        /* a non-physical face reads two planes into the ghost region */
        if ((!g->physical_face[2 * f] || !g->physical_face[2 * f + 1]) && gp < 2) return LSM_ERR_BAD_SHAPE;
    }
    return LSM_OK;
}

/* ---------------------------------------------------------------- helpers */

/* GetWENO3Reconstruction, src/AdvectionMethods.F90:195-245 */
inline double weno3(double f0, double f1, double f2, double f3, double ws) {
    const double d0 = 2.0 / 3.0, d1 = 1.0 / 3.0, epsw = 0.000001;
    double fL, fC, fR;
    if (ws > 0.0) { fL = f0; fC = f1; fR = f2; }
    else          { fL = f3; fC = f2; fR = f1; }
    double b0 = (fC - fR) * (fC - fR);
    double b1 = (fL - fC) * (fL - fC);
    double t0 = b0 + epsw, t1 = b1 + epsw;
    double a0 = d0 / (t0 * t0);
    double a1 = d1 / (t1 * t1);
    double w0 = a0 / (a0 + a1);
    double w1 = a1 / (a0 + a1);
    double u0 = 0.5 * fC + 0.5 * fR;
    double u1 = -0.5 * fL + 1.5 * fC;
    return u0 * w0 + u1 * w1;
}

/* deltaf, src/global_lsm.F90:120-133 */
inline double deltaf(double v, double e) {
    if (std::fabs(v) > e) return 0.0;
    return 1.0 / (2.0 * e) * (1.0 + std::cos(kPi * v / e));
}

/* the reference's exchange: no-op on one rank, or the caller's callback */
struct Exch {
    lsm_exchange_fn fn; void* user; const lsm_grid* g;
    void operator()(double* f) const { if (fn) fn(user, f, g); }
};

} /* namespace */

extern "C" {

/* ------------------------------------------------------------------ A1 --- */
/* rhs_contra_j, src/rhs_contra_j.F90:2-53 (+ ucn_j = zero, levelsetmethod.F90:225) */
int oracle_rhs_contra_j(const lsm_grid* gg, const double* q, const double* csi, const double* eta,
                        const double* zet, const double* aj, double* ucn) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    std::memset(ucn, 0, sizeof(double) * 3 * g.n);
    int ista = g.pb ? g.ia : g.il, iend = g.pf ? g.ib : g.iu;
    int jsta = g.pl ? g.ja : g.jl, jend = g.pr ? g.jb : g.ju;
    int ksta = g.pd ? g.ka : g.kl, kend = g.pu ? g.kb : g.ku;
#pragma omp parallel for
    for (int k = ksta; k <= kend; ++k)
        for (int j = jsta; j <= jend; ++j)
            for (int i = ista; i <= iend; ++i) {
                long l = g.id(i, j, k);
                double tmp = 1.0 / aj[l];
                double u = q[4 * l + 1], v = q[4 * l + 2], w = q[4 * l + 3];
                ucn[3 * l + 0] = tmp * (csi[3 * l] * u + csi[3 * l + 1] * v + csi[3 * l + 2] * w);
                ucn[3 * l + 1] = tmp * (eta[3 * l] * u + eta[3 * l + 1] * v + eta[3 * l + 2] * w);
                ucn[3 * l + 2] = tmp * (zet[3 * l] * u + zet[3 * l + 1] * v + zet[3 * l + 2] * w);
            }
    return LSM_OK;
}

/* ------------------------------------------------------------------ A2 --- */
/* calc_RH_AD_WENO3, src/calc_RH_AD_WENO3.F90:86-403.  rh must arrive zeroed
   (ad_RKTVD3.F90:55); only the nodes of the loop are written. */
static void weno3_rhs(const Grid& g, const double* phi, const double* ucn, const int* mask, double* rh) {
    int i0 = g.ia + (g.pb ? 1 : 0), i1 = g.ib - (g.pf ? 1 : 0);
    int j0 = g.ja + (g.pl ? 1 : 0), j1 = g.jb - (g.pr ? 1 : 0);
    int k0 = g.ka + (g.pd ? 1 : 0), k1 = g.kb - (g.pu ? 1 : 0);
    const long si = 1, sj = g.ni, sk = g.ni * g.nj;
#pragma omp parallel for
    for (int k = k0; k <= k1; ++k)
        for (int j = j0; j <= j1; ++j)
            for (int i = i0; i <= i1; ++i) {
                long l = g.id(i, j, k);
                if (mask && mask[l] == 0) continue;
                bool mb = g.pb && i == i0, mf = g.pf && i == i1;
                bool ml = g.pl && j == j0, mr = g.pr && j == j1;
                bool md = g.pd && k == k0, mu = g.pu && k == k1;
                double L[3];
                const long st[3] = {si, sj, sk};
                const bool lo[3] = {mb, ml, md}, hi[3] = {mf, mr, mu};
                const double dd[3] = {g.dc, g.de, g.dz};
                for (int d = 0; d < 3; ++d) {
                    long s = st[d];
                    double U = ucn[3 * l + d];
                    /* + 1/2 face */
                    double ws = U, p0 = phi[l - s], p1 = phi[l], p2 = phi[l + s], p3;
                    if (hi[d]) { ws = 1.0; p3 = 0.0; } else p3 = phi[l + 2 * s];
                    double fp = weno3(p0, p1, p2, p3, ws);
                    /* - 1/2 face */
                    ws = U;
                    if (lo[d]) { ws = -1.0; p0 = 0.0; } else p0 = phi[l - 2 * s];
                    p1 = phi[l - s]; p2 = phi[l]; p3 = phi[l + s];
                    double fm = weno3(p0, p1, p2, p3, ws);
                    L[d] = U * (dd[d] * (fp - fm));
                }
                rh[l] = L[0] + L[1] + L[2];
            }
}

/* ------------------------------------------------------------------ A7 --- */
/* calc_RH_AD (first-order upwind, orderAD == 0), src/calc_RH_AD.F90:1-273.
   With orderAD == 0 `is_boundary` stays .true. everywhere. */
static void upwind_rhs(const Grid& g, const double* phi, const double* ucn, const int* mask, double* rh) {
    const long st[3] = {1, g.ni, g.ni * g.nj};
    const double dd[3] = {g.dc, g.de, g.dz};
    const bool plo[3] = {g.pb, g.pl, g.pd}, phi_[3] = {g.pf, g.pr, g.pu};
    const int lo[3] = {g.ia, g.ja, g.ka}, hi[3] = {g.ib, g.jb, g.kb};
    for (int d = 0; d < 3; ++d) {
        long s = st[d];
#pragma omp parallel for
        for (int k = g.ka; k <= g.kb; ++k)
            for (int j = g.ja; j <= g.jb; ++j)
                for (int i = g.ia; i <= g.ib; ++i) {
                    long l = g.id(i, j, k);
                    if (mask && mask[l] <= 0) continue;
                    int c = d == 0 ? i : (d == 1 ? j : k);
                    double U = ucn[3 * l + d];
                    double val;
                    if (plo[d] && c == lo[d]) {
                        val = dd[d] * U * (phi[l + s] - phi[l]);
                    } else if (phi_[d] && c == hi[d]) {
                        val = dd[d] * U * (phi[l] - phi[l - s]);
                    } else {
                        double ucon = 0.5 * U;
                        double up = ucon + std::fabs(ucon), um = ucon - std::fabs(ucon);
                        val = dd[d] * (up * (phi[l] - phi[l - s]) + um * (phi[l + s] - phi[l]));
                    }
                    rh[l] = d == 0 ? val : val + rh[l];
                }
    }
}

int oracle_calc_rh_ad_weno3(const lsm_grid* gg, const double* phi, const double* ucn, const int* mask,
                            double* rh) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    std::memset(rh, 0, sizeof(double) * g.n);
    weno3_rhs(g, phi, ucn, mask, rh);
    return LSM_OK;
}

int oracle_calc_rh_ad(const lsm_grid* gg, const double* phi, const double* ucn, const int* mask, double* rh) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    std::memset(rh, 0, sizeof(double) * g.n);
    upwind_rhs(g, phi, ucn, mask, rh);
    return LSM_OK;
}

/* ------------------------------------------------------------------ A5 --- */
/* bcond_lsm, src/bcond_lsm.F90:2-287 (no blanking: nblk == 0) */
static void bcond(const Grid& g, const lsm_params* p, double* phi) {
    const double a2 = 4.0 / 3.0, b2 = -1.0 / 3.0, a1 = 1.0, b1 = 0.0;
    const double BigPhi = p->BigPhi;
    auto ext = [&](double n1, double n2) {
        /* exsign = (one + sign(one, abs(phi2) - BigPhi)) / two */
        double exsign = (1.0 + std::copysign(1.0, std::fabs(n2) - BigPhi)) / 2.0;
        double itpa = a2 + exsign * (a1 - a2);
        double itpb = b2 + exsign * (b1 - b2);
        return itpa * n1 + itpb * n2;
    };
    const long sj = g.ni, sk = g.ni * g.nj;
    /* i faces: loops over j, k of the non-ghost range */
    for (int f = 0; f < 2; ++f) {
        bool phys = f == 0 ? g.pb : g.pf;
        int bt = p->btype_lsm[f];
        if (!phys) continue;
        int i = f == 0 ? g.ia : g.ib;
        long s = f == 0 ? 1 : -1;
        for (int k = g.ka; k <= g.kb; ++k)
            for (int j = g.ja; j <= g.jb; ++j) {
                long l = g.id(i, j, k);
                if (bt == 0) phi[l] = phi[l + s];
                else if (bt == 1) phi[l] = ext(phi[l + s], phi[l + 2 * s]);
                else if (bt == 2 && f == 1) phi[l] = 2.0 * phi[l + s] - 1.0 * phi[l + 2 * s];
            }
    }
    for (int f = 2; f < 4; ++f) {
        bool phys = f == 2 ? g.pl : g.pr;
        int bt = p->btype_lsm[f];
        if (!phys) continue;
        int j = f == 2 ? g.ja : g.jb;
        long s = f == 2 ? sj : -sj;
        for (int k = g.ka; k <= g.kb; ++k)
            for (int i = g.ia; i <= g.ib; ++i) {
                long l = g.id(i, j, k);
                if (bt == 0) phi[l] = phi[l + s];
                else if (bt == 1) phi[l] = ext(phi[l + s], phi[l + 2 * s]);
            }
    }
    for (int f = 4; f < 6; ++f) {
        bool phys = f == 4 ? g.pd : g.pu;
        int bt = p->btype_lsm[f];
        if (!phys) continue;
        int k = f == 4 ? g.ka : g.kb;
        long s = f == 4 ? sk : -sk;
        for (int j = g.ja; j <= g.jb; ++j)
            for (int i = g.ia; i <= g.ib; ++i) {
                long l = g.id(i, j, k);
                if (bt == 0) phi[l] = phi[l + s];
                else if (bt == 1) phi[l] = ext(phi[l + s], phi[l + 2 * s]);
            }
    }
}

int oracle_bcond_lsm(const lsm_grid* gg, const lsm_params* p, double* phi) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    bcond(g, p, phi);
    return LSM_OK;
}

/* ------------------------------------------------------------------ A4 --- */
/* ad_RKTVD3, src/ad_RKTVD3.F90:1-88 */
int oracle_ad_rktvd3_x(const lsm_grid* gg, const lsm_params* p, double* phi1, const double* phin,
                       const int* mask, const double* ucn, const double* aj, lsm_exchange_fn fn, void* user) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    Exch ex{fn, user, gg};
    const double c[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
    const double dt = p->delti_lsm;
    std::vector<double> rh(g.n);
    std::memcpy(phi1, phin, sizeof(double) * g.n);
    for (int rk = 0; rk < 3; ++rk) {
        std::fill(rh.begin(), rh.end(), 0.0);
        if (p->orderAD == 0) upwind_rhs(g, phi1, ucn, mask, rh.data());
        else weno3_rhs(g, phi1, ucn, mask, rh.data());
#pragma omp parallel for
        for (int k = g.ka; k <= g.kb; ++k)
            for (int j = g.ja; j <= g.jb; ++j)
                for (int i = g.ia; i <= g.ib; ++i) {
                    long l = g.id(i, j, k);
                    if (mask && mask[l] <= 0) continue;
                    phi1[l] = c[rk][0] * phin[l] + c[rk][1] * phi1[l] - c[rk][2] * aj[l] * dt * rh[l];
                }
        bcond(g, p, phi1);
        ex(phi1);
    }
    return LSM_OK;
}

int oracle_ad_rktvd3(const lsm_grid* gg, const lsm_params* p, double* phi1, const double* phin,
                     const int* mask, const double* ucn, const double* aj) {
    return oracle_ad_rktvd3_x(gg, p, phi1, phin, mask, ucn, aj, nullptr, nullptr);
}

/* ------------------------------------------------------------- R1 / R2 --- */
/* One-sided differences of calc_sign_ini.F90:42-176 / calc_RH_RN.F90:36-170
   (identical blocks): mas/menos along xi, eta, zeta, with the boundary
   planes of physical faces copying the single available difference. */
static void one_sided(const Grid& g, const double* f, std::vector<double>* D /* 6 arrays */) {
    const long st[3] = {1, g.ni, g.ni * g.nj};
    const double dd[3] = {g.dc, g.de, g.dz};
    const bool plo[3] = {g.pb, g.pl, g.pd}, phi_[3] = {g.pf, g.pr, g.pu};
    const int lo[3] = {g.ia, g.ja, g.ka}, hi[3] = {g.ib, g.jb, g.kb};
    for (int d = 0; d < 3; ++d) {
        long s = st[d];
        double* mas = D[2 * d].data();
        double* men = D[2 * d + 1].data();
#pragma omp parallel for
        for (int k = g.ka; k <= g.kb; ++k)
            for (int j = g.ja; j <= g.jb; ++j)
                for (int i = g.ia; i <= g.ib; ++i) {
                    long l = g.id(i, j, k);
                    int c = d == 0 ? i : (d == 1 ? j : k);
                    if (plo[d] && c == lo[d]) {
                        mas[l] = dd[d] * (f[l + s] - f[l]);
                        men[l] = mas[l];
                    } else if (phi_[d] && c == hi[d]) {
                        men[l] = dd[d] * (f[l] - f[l - s]);
                        mas[l] = men[l];
                    } else {
                        mas[l] = dd[d] * (f[l + s] - f[l]);
                        men[l] = dd[d] * (f[l] - f[l - s]);
                    }
                }
    }
}

/* Godunov |grad f|+ and |grad f|- from the contracted one-sided differences,
   calc_sign_ini.F90:204-242 / calc_RH_RN.F90:190-228 */
static inline void godunov(const double* csi, const double* eta, const double* zet, long l,
                           double cm, double cp, double em, double ep, double zm, double zp,
                           double* gplus, double* gminus) {
    double dxb = csi[3 * l] * cm + eta[3 * l] * em + zet[3 * l] * zm;
    double dxf = csi[3 * l] * cp + eta[3 * l] * ep + zet[3 * l] * zp;
    double dyb = csi[3 * l + 1] * cm + eta[3 * l + 1] * em + zet[3 * l + 1] * zm;
    double dyf = csi[3 * l + 1] * cp + eta[3 * l + 1] * ep + zet[3 * l + 1] * zp;
    double dzb = csi[3 * l + 2] * cm + eta[3 * l + 2] * em + zet[3 * l + 2] * zm;
    double dzf = csi[3 * l + 2] * cp + eta[3 * l + 2] * ep + zet[3 * l + 2] * zp;
    double aux;
    aux = dxb / 2.0; double dxbp = aux + std::fabs(aux), dxbm = aux - std::fabs(aux);
    aux = dxf / 2.0; double dxfp = aux + std::fabs(aux), dxfm = aux - std::fabs(aux);
    aux = dyb / 2.0; double dybp = aux + std::fabs(aux), dybm = aux - std::fabs(aux);
    aux = dyf / 2.0; double dyfp = aux + std::fabs(aux), dyfm = aux - std::fabs(aux);
    aux = dzb / 2.0; double dzbp = aux + std::fabs(aux), dzbm = aux - std::fabs(aux);
    aux = dzf / 2.0; double dzfp = aux + std::fabs(aux), dzfm = aux - std::fabs(aux);
    *gplus = std::sqrt(std::fmax(dxbp * dxbp, dxfm * dxfm) + std::fmax(dybp * dybp, dyfm * dyfm) +
                       std::fmax(dzbp * dzbp, dzfm * dzfm));
    *gminus = std::sqrt(std::fmax(dxbm * dxbm, dxfp * dxfp) + std::fmax(dybm * dybm, dyfp * dyfp) +
                        std::fmax(dzbm * dzbm, dzfp * dzfp));
}

/* calc_sign_ini, src/calc_sign_ini.F90:1-286 */
int oracle_calc_sign_ini(const lsm_grid* gg, const double* phi0, const double* csi, const double* eta,
                         const double* zet, double eps, int M_Sphi0, double* sgn, double* ng) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    std::vector<double> D[6];
    for (auto& v : D) v.assign(g.n, 0.0);
    one_sided(g, phi0, D);
#pragma omp parallel for
    for (int k = g.ka; k <= g.kb; ++k)
        for (int j = g.ja; j <= g.jb; ++j)
            for (int i = g.ia; i <= g.ib; ++i) {
                long l = g.id(i, j, k);
                double gp, gm;
                godunov(csi, eta, zet, l, D[1][l], D[0][l], D[3][l], D[2][l], D[5][l], D[4][l], &gp, &gm);
                double f = phi0[l];
                double nrm = f > 0.0 ? gp : (f < 0.0 ? gm : 1.0);
                double s;
                if (M_Sphi0 == 1) {
                    if (f >= eps) s = 1.0;
                    else if (f <= (-1.0) * eps) s = -1.0;
                    else s = f / eps - 1.0 / kPi * std::sin(kPi * f / eps);
                } else {
                    s = f / std::sqrt(f * f + (nrm * eps) * (nrm * eps));
                }
                sgn[l] = s;
                ng[l] = nrm;
            }
    return LSM_OK;
}

/* calc_RH_RN, src/calc_RH_RN.F90:1-244 */
static void rh_rn(const Grid& g, const double* d, const double* sgn, const double* csi, const double* eta,
                  const double* zet, double* rh, std::vector<double>* D) {
    one_sided(g, d, D);
#pragma omp parallel for
    for (int k = g.ka; k <= g.kb; ++k)
        for (int j = g.ja; j <= g.jb; ++j)
            for (int i = g.ia; i <= g.ib; ++i) {
                long l = g.id(i, j, k);
                double gp, gm;
                godunov(csi, eta, zet, l, D[1][l], D[0][l], D[3][l], D[2][l], D[5][l], D[4][l], &gp, &gm);
                double s = sgn[l];
                double nrm = s > 0.0 ? gp : (s < 0.0 ? gm : 1.0);
                rh[l] = s * (nrm - 1.0);
            }
}

int oracle_calc_rh_rn(const lsm_grid* gg, const double* d, const double* sgn, const double* csi,
                      const double* eta, const double* zet, double* rh) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    std::vector<double> D[6];
    for (auto& v : D) v.assign(g.n, 0.0);
    rh_rn(g, d, sgn, csi, eta, zet, rh, D);
    return LSM_OK;
}

/* ------------------------------------------------------------------ R3 --- */
/* calc_lambda_RN method 0, src/calc_lambda_RN.F90:42-63 */
static void lambda_rn(const Grid& g, double eps, const double* phi0, const double* ng, const double* d,
                      double dt, double* lam) {
    double volcell = 1.0 / g.dc * (1.0 / g.de) * (1.0 / g.dz);
#pragma omp parallel for
    for (int k = g.ka; k <= g.kb; ++k)
        for (int j = g.ja; j <= g.jb; ++j)
            for (int i = g.ia; i <= g.ib; ++i) {
                long l = g.id(i, j, k);
                double del = deltaf(phi0[l], eps);
                double Lop = del * (1.0 / dt * (d[l] - phi0[l]));
                double num = volcell * Lop;
                double den = volcell * (del * del) * ng[l];
                lam[l] = den == 0.0 ? 0.0 : -num / den;
            }
}

int oracle_calc_lambda_rn(const lsm_grid* gg, const lsm_params* p, const double* phi0, const double* ng,
                          const double* d, double dt, double* lam) {
    int st = check_grid(gg); if (st) return st;
    if (p->sussman_correction_method != 0) return LSM_ERR_UNSUPPORTED;
    Grid g(gg);
    lambda_rn(g, p->epslsm, phi0, ng, d, dt, lam);
    return LSM_OK;
}

/* ------------------------------------------------------------------ R0 --- */
/* reinitialization, src/reinitialization.F90:1-106 (act_obstacle_rn == 1) */
int oracle_reinitialization_x(const lsm_grid* gg, const lsm_params* p, const double* phi0, const double* csi,
                              const double* eta, const double* zet, double* out, lsm_exchange_fn fn,
                              void* user) {
    int st = check_grid(gg); if (st) return st;
    if (p->sussman_correction_method != 0) return LSM_ERR_UNSUPPORTED;
    Grid g(gg);
    Exch ex{fn, user, gg};
    const double dt = p->RNtimestep, eps = p->epslsm;
    std::vector<double> dn(phi0, phi0 + g.n), d(phi0, phi0 + g.n), rh(g.n, 0.0), sg(g.n, 0.0), ng(g.n, 0.0),
        lam(g.n, 0.0);
    std::vector<double> D[6];
    for (auto& v : D) v.assign(g.n, 0.0);
    oracle_calc_sign_ini(gg, phi0, csi, eta, zet, eps, p->M_Sphi0, sg.data(), ng.data());
    ex(sg.data()); ex(ng.data());
    for (int it = 0; it < p->RNitermax; ++it) {
        rh_rn(g, d.data(), sg.data(), csi, eta, zet, rh.data(), D);
#pragma omp parallel for
        for (int k = g.ka; k <= g.kb; ++k)
            for (int j = g.ja; j <= g.jb; ++j)
                for (int i = g.ia; i <= g.ib; ++i) {
                    long l = g.id(i, j, k);
                    d[l] = dn[l] - dt * rh[l];
                }
        ex(d.data());
        lambda_rn(g, eps, phi0, ng.data(), d.data(), dt, lam.data());
#pragma omp parallel for
        for (int k = g.ka; k <= g.kb; ++k)
            for (int j = g.ja; j <= g.jb; ++j)
                for (int i = g.ia; i <= g.ib; ++i) {
                    long l = g.id(i, j, k);
                    d[l] = d[l] + dt * lam[l] * deltaf(phi0[l], eps) * ng[l];
                }
        ex(d.data());
        dn = d;
    }
    std::memcpy(out, d.data(), sizeof(double) * g.n);
    return LSM_OK;
}

int oracle_reinitialization(const lsm_grid* gg, const lsm_params* p, const double* phi0, const double* csi,
                            const double* eta, const double* zet, double* out) {
    return oracle_reinitialization_x(gg, p, phi0, csi, eta, zet, out, nullptr, nullptr);
}

/* ------------------------------------------------------------------ N1 --- */
/* narrowband, src/narrowband.F90:2-19.  tol = 1.0E-5 is a default-kind
   (single precision) literal assigned to a REAL(8): the float value. */
int oracle_narrowband(const lsm_grid* gg, const lsm_params* p, const double* phin, int* nband) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    const double tol = (double)1.0E-5f;
    double thr = p->narrowcoef * p->epslsm + tol;
    for (long l = 0; l < g.n; ++l) nband[l] = (p->isnarrow == 0) ? 1 : (std::fabs(phin[l]) < thr ? 1 : 0);
    return LSM_OK;
}

/* ------------------------------------------------------------------ N3 --- */
/* get_gfm_list, src/get_gfm_list.F90:1-143 with the loop bounds of
   ghost_fluid_extrapolation.F90:263-277 and rsign, src/precision.F90:66-73 */
int oracle_get_gfm_list(const lsm_grid* gg, const lsm_params* p, const double* phi, int* count, int* list,
                        int ld) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    int i0 = g.ia + (g.pb ? 1 : 0), i1 = g.ib - (g.pf ? 1 : 0);
    int j0 = g.ja + (g.pl ? 1 : 0), j1 = g.jb - (g.pr ? 1 : 0);
    int k0 = g.ka + (g.pd ? 1 : 0), k1 = g.kb - (g.pu ? 1 : 0);
    std::vector<int> out;
    for (int k = k0; k <= k1; ++k)
        for (int j = j0; j <= j1; ++j)
            for (int i = i0; i <= i1; ++i) {
                double f = phi[g.id(i, j, k)];
                double rs = f > kEpsSims ? 1.0 : 0.0;
                if (rs > 0.5 || std::fabs(f) > p->BigPhi) continue;
                bool water = false;
                for (int kk = k - 1; kk <= k + 1 && !water; ++kk)
                    for (int jj = j - 1; jj <= j + 1 && !water; ++jj)
                        for (int ii = i - 1; ii <= i + 1 && !water; ++ii)
                            if (phi[g.id(ii, jj, kk)] > kEpsSims) water = true;
                if (!water) continue;
                out.push_back(i); out.push_back(j); out.push_back(k);
            }
    int c = (int)(out.size() / 3);
    *count = c;
    if (list) {
        if (ld < c) return LSM_ERR_CAPACITY;
        for (int n = 0; n < c; ++n) {
            list[n] = out[3 * n]; list[n + ld] = out[3 * n + 1]; list[n + 2 * (long)ld] = out[3 * n + 2];
        }
    }
    return LSM_OK;
}

} /* extern "C" */

/* --------------------------------------------------------------- V1 ------ */
namespace {

/* M44Det, src/TetrahedronMethods.F90:1698-1720 (A is 1-based in the comment) */
inline double m44det(const double A[4][4]) {
#define a(r, c) A[(r) - 1][(c) - 1]
    double t1 = a(1, 1) * (a(2, 2) * (a(3, 3) * a(4, 4) - a(3, 4) * a(4, 3)) +
                           a(2, 3) * (a(3, 4) * a(4, 2) - a(3, 2) * a(4, 4)) +
                           a(2, 4) * (a(3, 2) * a(4, 3) - a(3, 3) * a(4, 2)));
    double t2 = a(1, 2) * (a(2, 1) * (a(3, 3) * a(4, 4) - a(3, 4) * a(4, 3)) +
                           a(2, 3) * (a(3, 4) * a(4, 1) - a(3, 1) * a(4, 4)) +
                           a(2, 4) * (a(3, 1) * a(4, 3) - a(3, 3) * a(4, 1)));
    double t3 = a(1, 3) * (a(2, 1) * (a(3, 2) * a(4, 4) - a(3, 4) * a(4, 2)) +
                           a(2, 2) * (a(3, 4) * a(4, 1) - a(3, 1) * a(4, 4)) +
                           a(2, 4) * (a(3, 1) * a(4, 2) - a(3, 2) * a(4, 1)));
    double t4 = a(1, 4) * (a(2, 1) * (a(3, 2) * a(4, 3) - a(3, 3) * a(4, 2)) +
                           a(2, 2) * (a(3, 3) * a(4, 1) - a(3, 1) * a(4, 3)) +
                           a(2, 3) * (a(3, 1) * a(4, 2) - a(3, 2) * a(4, 1)));
#undef a
    return t1 - t2 + t3 - t4;
}

/* GetTetrahedronVolume, src/TetrahedronMethods.F90:666-688 */
inline double tet_volume(const double* v0, const double* v1, const double* v2, const double* v3) {
    double A[4][4] = {{v0[0], v0[1], v0[2], 1.0}, {v1[0], v1[1], v1[2], 1.0},
                      {v2[0], v2[1], v2[2], 1.0}, {v3[0], v3[1], v3[2], 1.0}};
    return 1.0 / 6.0 * std::fabs(m44det(A));
}

const int kEdge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
const int kEdgeFlags[16] = {0x00, 0x0d, 0x13, 0x1e, 0x26, 0x2b, 0x35, 0x38,
                            0x38, 0x35, 0x2b, 0x26, 0x1e, 0x13, 0x0d, 0x00};

/* GetWaterVolume, src/TetrahedronMethods.F90:710-954 (E is 0-based: E[e] = edge e+1) */
double water_volume(const double V[4][3], const double E[6][3], int fi, int* err) {
    double TV = tet_volume(V[0], V[1], V[2], V[3]);
    double AV, r = 0.0;
    switch (fi + 1) {
    case 2: case 15:
        AV = tet_volume(V[0], E[0], E[2], E[3]);
        r = (fi + 1 == 2) ? TV - AV : AV; break;
    case 3: case 14:
        AV = tet_volume(V[1], E[0], E[1], E[4]);
        r = (fi + 1 == 3) ? TV - AV : AV; break;
    case 4: case 13:
        AV = tet_volume(V[0], E[2], E[3], E[4]) + tet_volume(V[0], E[1], E[2], E[4]) +
             tet_volume(V[0], V[1], E[1], E[4]);
        r = (fi + 1 == 4) ? TV - AV : AV; break;
    case 5: case 12:
        AV = tet_volume(V[2], E[1], E[2], E[5]);
        r = (fi + 1 == 5) ? TV - AV : AV; break;
    case 6: case 11:
        AV = tet_volume(V[0], E[0], E[1], E[5]) + tet_volume(V[0], E[0], E[3], E[5]) +
             tet_volume(V[0], V[2], E[1], E[5]);
        r = (fi + 1 == 6) ? TV - AV : AV; break;
    case 7: case 10:
        AV = tet_volume(V[1], E[0], E[2], E[5]) + tet_volume(V[1], E[0], E[4], E[5]) +
             tet_volume(V[1], V[2], E[2], E[5]);
        r = (fi + 1 == 7) ? TV - AV : AV; break;
    case 8: case 9:
        AV = tet_volume(V[3], E[3], E[4], E[5]);
        r = (fi + 1 == 8) ? AV : TV - AV; break;
    default: r = 0.0;
    }
    if (r < -kEpsSims) *err = 1;
    return r;
}

/* MarchingTetrahedron (volume output only), src/TetrahedronMethods.F90:26-664 */
double marching_tet(const double V[4][3], const double ph[4], int* err) {
    int s[4];
    for (int v = 0; v < 4; ++v) s[v] = ph[v] > kTiny ? 1 : (ph[v] < -kTiny ? -1 : 0);
    bool allp = true, alln = true, anyz = false, allge = true, allle = true;
    int nz = 0;
    for (int v = 0; v < 4; ++v) {
        allp &= s[v] == 1; alln &= s[v] == -1; anyz |= s[v] == 0; nz += s[v] == 0;
        allge &= s[v] >= 0; allle &= s[v] <= 0;
    }
    if (allp) return tet_volume(V[0], V[1], V[2], V[3]);
    if (alln) return 0.0;
    int fi = 0;
    if (anyz && (allge || allle)) {
        double full = 0.0;
        switch (nz) {
        case 1:
            if (s[0] == 0) return s[1] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[1] == 0) return s[0] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[2] == 0) return s[0] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[3] == 0) return s[0] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            break;
        case 2:
            if (s[0] == 0 && s[1] == 0) return s[2] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[1] == 0 && s[2] == 0) return s[0] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[2] == 0 && s[0] == 0) return s[1] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[0] == 0 && s[3] == 0) return s[1] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[1] == 0 && s[3] == 0) return s[0] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            if (s[2] == 0 && s[3] == 0) return s[0] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            break;
        case 3:
            for (int v = 0; v < 4; ++v)
                if (s[v] == 1 || s[v] == -1) return s[v] == 1 ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0;
            break;
        default: break; /* four zero vertices: FlagIndex stays 0 below */
        }
        (void)full;
    } else {
        for (int v = 0; v < 4; ++v)
            if (s[v] == -1) fi |= 1 << v;
    }
    double wv = 0.0;
    if (fi == 0) wv = tet_volume(V[0], V[1], V[2], V[3]);
    if (fi == 15) wv = 0.0;
    int ef = kEdgeFlags[fi];
    if (ef == 0) return wv;
    double E[6][3];
    for (int e = 0; e < 6; ++e) E[e][0] = E[e][1] = E[e][2] = -9.9;
    for (int e = 0; e < 6; ++e) {
        if (!(ef >> e & 1)) continue;
        int sv = kEdge[e][0], ev = kEdge[e][1];
        double den = ph[ev] - ph[sv];
        double sc = std::fabs(den) < kEpsSims * kEpsSims * kEpsSims ? 0.0 : ph[ev] / den;
        for (int c = 0; c < 3; ++c) E[e][c] = V[ev][c] + sc * (V[sv][c] - V[ev][c]);
    }
    return water_volume(V, E, fi, err);
}

/* HexahedronVolume (Davies & Salmond 1985), src/TetrahedronMethods.F90:1724-1793 */
inline double dot3(const double* a, const double* b) {
    double s = 0.0;
    s = s + a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}
inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
double hex_volume(const double C[8][3]) {
    const double *A = C[0], *B = C[1], *Cc = C[2], *D = C[3], *E = C[4], *F = C[5], *G = C[6], *H = C[7];
    double AC[3], AF[3], AH[3], BE[3], CH[3], DB[3], ED[3], FC[3], GA[3], GB[3], GC[3], GD[3], GE[3], GF[3],
        GH[3], HF[3];
    for (int c = 0; c < 3; ++c) {
        AC[c] = Cc[c] - A[c]; AF[c] = F[c] - A[c]; AH[c] = H[c] - A[c]; BE[c] = E[c] - B[c];
        CH[c] = H[c] - Cc[c]; DB[c] = B[c] - D[c]; ED[c] = D[c] - E[c]; FC[c] = Cc[c] - F[c];
        GA[c] = A[c] - G[c]; GB[c] = B[c] - G[c]; GC[c] = Cc[c] - G[c]; GD[c] = D[c] - G[c];
        GE[c] = E[c] - G[c]; GF[c] = F[c] - G[c]; GH[c] = H[c] - G[c]; HF[c] = F[c] - H[c];
    }
    double s1[3], s2[3], s3[3], x[3];
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

const int kTets[6][4] = {{0, 5, 1, 6}, {0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}};

/* CellAnalysis (TriangulationCase 1), src/TetrahedronMethods.F90:1823-2121 */
void cell_analysis(const double ph[8], const double C[8][3], double* K, double* S, int* err) {
    *K = 0.0; *S = 0.0;
    bool pcc = false;
    for (int v = 0; v < 8; ++v) if (std::fabs(ph[v]) < kEpsSims) pcc = true;
    if (!pcc) {
        double sg = std::copysign(1.0, ph[0]);
        for (int v = 1; v < 8; ++v) if (sg * ph[v] < 0.0) { pcc = true; break; }
    }
    if (!pcc) return;
    for (int t = 0; t < 6; ++t) {
        bool pct = false, second = true;
        double pa = ph[kTets[t][0]];
        if (pa <= kEpsSims) second = false;
        if (std::fabs(pa) < kEpsSims) pct = true;
        double sg = std::copysign(1.0, pa);
        for (int v = 1; v < 4; ++v) {
            double pb = ph[kTets[t][v]];
            if (sg * pb < 0.0 || std::fabs(pb) < kEpsSims) {
                if (pb <= kEpsSims) second = false;
                pct = true;
            }
        }
        double V[4][3], P[4];
        for (int v = 0; v < 4; ++v) {
            for (int c = 0; c < 3; ++c) V[v][c] = C[kTets[t][v]][c];
            P[v] = ph[kTets[t][v]];
        }
        if (pct) *K = *K + marching_tet(V, P, err);
        if (second && !pct) *S = *S + tet_volume(V[0], V[1], V[2], V[3]);
    }
}

/* One cell of TotalWaterVolume.F90:241-290: returns the three parts. */
void cell_volume(const Grid& g, const double* phi, const double* x, const double* y, const double* z, int i,
                 int j, int k, double* K, double* S, double* B, int* err) {
    static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    double C[8][3], P[8];
    for (int v = 0; v < 8; ++v) {
        long l = g.id(i + off[v][0], j + off[v][1], k + off[v][2]);
        C[v][0] = x[l]; C[v][1] = y[l]; C[v][2] = z[l]; P[v] = phi[l];
    }
    *K = *S = *B = 0.0;
    bool allw = true, alla = true;
    for (int v = 0; v < 8; ++v) { allw &= P[v] > kEpsSims; alla &= P[v] < -kEpsSims; }
    if (allw) { *B = hex_volume(C); return; }
    if (alla) return;
    cell_analysis(P, C, K, S, err);
}

struct CellRange { int i0, i1, j0, j1, k0, k1, ista, iend, jsta, jend, ksta, kend; };
CellRange cell_range(const Grid& g) {
    CellRange r;
    r.i0 = g.ia; r.j0 = g.ja; r.k0 = g.ka;
    r.i1 = g.ib - (g.pf ? 1 : 0); r.j1 = g.jb - (g.pr ? 1 : 0); r.k1 = g.kb - (g.pu ? 1 : 0);
    r.ista = g.pb ? g.ia : g.il; r.jsta = g.pl ? g.ja : g.jl; r.ksta = g.pd ? g.ka : g.kl;
    r.iend = g.pf ? g.ib : g.iu; r.jend = g.pr ? g.jb : g.ju; r.kend = g.pu ? g.kb : g.ku;
    return r;
}

} /* namespace */

extern "C" {

/* TotalWaterVolume, src/TotalWaterVolume.F90:1-297 (TriangulationCase 1,
   nblk == 0).  Sequential k, j, i sums as in the reference. */
int oracle_total_water_volume(const lsm_grid* gg, const double* phi, const double* x, const double* y,
                              const double* z, double* vols, int* adv) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    CellRange r = cell_range(g);
    if (adv) std::memset(adv, 0, sizeof(int) * g.n);
    double VK = 0.0, V2 = 0.0, VB = 0.0;
    int err = 0;
    for (int k = r.k0; k <= r.k1; ++k)
        for (int j = r.j0; j <= r.j1; ++j)
            for (int i = r.i0; i <= r.i1; ++i) {
                int km = std::max(k - 1, r.ksta), kp = std::min(k + 1, r.kend);
                int jm = std::max(j - 1, r.jsta), jp = std::min(j + 1, r.jend);
                int im = std::max(i - 1, r.ista), ip = std::min(i + 1, r.iend);
                if (adv) {
                    double f = phi[g.id(i, j, k)];
                    double sg = std::copysign(1.0, f);
                    bool pc = std::fabs(f) < kEpsSims;
                    for (int ks = km; ks <= kp && !pc; ++ks)
                        for (int js = jm; js <= jp && !pc; ++js)
                            for (int is = im; is <= ip && !pc; ++is) {
                                double h = phi[g.id(is, js, ks)];
                                if (sg * h < 0.0 || std::fabs(h) < kEpsSims) pc = true;
                            }
                    if (pc)
                        for (int ks = km; ks <= kp; ++ks)
                            for (int js = jm; js <= jp; ++js)
                                for (int is = im; is <= ip; ++is) adv[g.id(is, js, ks)] = 1;
                }
                double K, S, B;
                cell_volume(g, phi, x, y, z, i, j, k, &K, &S, &B, &err);
                VK = VK + K; V2 = V2 + S; VB = VB + B;
            }
    vols[0] = VK; vols[1] = V2; vols[2] = VB; vols[3] = VK + V2 + VB;
    return err ? LSM_ERR_NEGATIVE_VOLUME : LSM_OK;
}

/* Multi-threaded volume (timing baseline only: per-thread partial sums). */
int oracle_total_water_volume_par(const lsm_grid* gg, const double* phi, const double* x, const double* y,
                                  const double* z, double* vols) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    CellRange r = cell_range(g);
    double VK = 0.0, V2 = 0.0, VB = 0.0;
    int err = 0;
#pragma omp parallel for reduction(+ : VK, V2, VB) reduction(| : err)
    for (int k = r.k0; k <= r.k1; ++k)
        for (int j = r.j0; j <= r.j1; ++j)
            for (int i = r.i0; i <= r.i1; ++i) {
                double K, S, B;
                int e = 0;
                cell_volume(g, phi, x, y, z, i, j, k, &K, &S, &B, &e);
                VK += K; V2 += S; VB += B; err |= e;
            }
    vols[0] = VK; vols[1] = V2; vols[2] = VB; vols[3] = VK + V2 + VB;
    return err ? LSM_ERR_NEGATIVE_VOLUME : LSM_OK;
}

/* per-cell diagnostic: cellvol(i,j,k) = (K + S) + B of cell (i,j,k) */
int oracle_cell_water_volumes(const lsm_grid* gg, const double* phi, const double* x, const double* y,
                              const double* z, double* cv) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    CellRange r = cell_range(g);
    std::memset(cv, 0, sizeof(double) * g.n);
    int err = 0;
    for (int k = r.k0; k <= r.k1; ++k)
        for (int j = r.j0; j <= r.j1; ++j)
            for (int i = r.i0; i <= r.i1; ++i) {
                double K, S, B;
                cell_volume(g, phi, x, y, z, i, j, k, &K, &S, &B, &err);
                cv[g.id(i, j, k)] = K + S + B;
            }
    return err ? LSM_ERR_NEGATIVE_VOLUME : LSM_OK;
}

/* ------------------------------------------------------------------ M0 --- */
/* mg_metrics on the fine grid of one rank, src/mg_metrics.F90:44-264:
   central differences inside, one-sided on the physical faces, then
   aj = 1/det and csi/eta/zet = aj * cofactors. */
int oracle_mg_metrics(const lsm_grid* gg, const double* x, const double* y, const double* z, double* csi,
                      double* eta, double* zet, double* aj) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    if (g.igp || g.jgp || g.kgp || !(g.pb && g.pf && g.pl && g.pr && g.pd && g.pu)) return LSM_ERR_UNSUPPORTED;
    const long st3[3] = {1, g.ni, g.ni * g.nj};
    const double dd[3] = {g.dc, g.de, g.dz};
    const int lo[3] = {g.ia, g.ja, g.ka}, hi[3] = {g.ib, g.jb, g.kb};
    std::vector<double> dx[3], dy[3], dzv[3];
    for (int d = 0; d < 3; ++d) { dx[d].assign(g.n, 0.0); dy[d].assign(g.n, 0.0); dzv[d].assign(g.n, 0.0); }
    for (int d = 0; d < 3; ++d) {
        long s = st3[d];
        double dum1 = dd[d], dum = 0.5 * dd[d];
        for (int k = g.ka; k <= g.kb; ++k)
            for (int j = g.ja; j <= g.jb; ++j)
                for (int i = g.ia; i <= g.ib; ++i) {
                    long l = g.id(i, j, k);
                    int c = d == 0 ? i : (d == 1 ? j : k);
                    if (c == lo[d]) {
                        dx[d][l] = dum1 * (x[l + s] - x[l]); dy[d][l] = dum1 * (y[l + s] - y[l]);
                        dzv[d][l] = dum1 * (z[l + s] - z[l]);
                    } else if (c == hi[d]) {
                        dx[d][l] = dum1 * (x[l] - x[l - s]); dy[d][l] = dum1 * (y[l] - y[l - s]);
                        dzv[d][l] = dum1 * (z[l] - z[l - s]);
                    } else {
                        dx[d][l] = dum * (x[l + s] - x[l - s]); dy[d][l] = dum * (y[l + s] - y[l - s]);
                        dzv[d][l] = dum * (z[l + s] - z[l - s]);
                    }
                }
    }
    for (long l = 0; l < g.n; ++l) {
        double xc = dx[0][l], yc = dy[0][l], zc = dzv[0][l];
        double xe = dx[1][l], ye = dy[1][l], ze = dzv[1][l];
        double xz = dx[2][l], yz = dy[2][l], zz = dzv[2][l];
        double gj = xc * (ye * zz - yz * ze) + xe * (yz * zc - yc * zz) + xz * (yc * ze - ye * zc);
        double a = 1.0 / gj;
        aj[l] = a;
        csi[3 * l + 0] = a * (ye * zz - yz * ze);
        csi[3 * l + 1] = a * (xz * ze - xe * zz);
        csi[3 * l + 2] = a * (xe * yz - xz * ye);
        eta[3 * l + 0] = a * (yz * zc - yc * zz);
        eta[3 * l + 1] = a * (xc * zz - xz * zc);
        eta[3 * l + 2] = a * (xz * yc - xc * yz);
        zet[3 * l + 0] = a * (yc * ze - ye * zc);
        zet[3 * l + 1] = a * (xe * zc - xc * ze);
        zet[3 * l + 2] = a * (xc * ye - xe * yc);
    }
    return LSM_OK;
}

/* ------------------------------------------------------------------ L0 --- */
/* The reference's live reinitialisation: reinitialisation_test2
   (src/reinitialisation_test2.F90:1-221) with calc_NormGrad_d
   (src/calc_NormGrad_d.F90:1-2448) and the AdvectionMethods helpers
   GetENO2Reconstruction (src/AdvectionMethods.F90:63-191), BiasedDerivative
   (:248-302), GetSignPhi0 (:576-587), ENO2Boundary (:654-707) and
   GetLambdaMassCorrection (src/global_lsm.F90:200-219). */
} /* extern "C" */
namespace {

/* GetENO2Reconstruction, src/AdvectionMethods.F90:63-191 */
double eno2(double f0, double fLL, double fL, double fC, double fR, double fRR, bool lo, bool hi) {
    double a, b, Mf, dp, dm;
    if (lo) {
        a = fR - (2.0 * fC) + fL;
        b = fRR - (2.0 * fR) + fC;
        Mf = a;
        if (std::fabs(b) < std::fabs(a)) Mf = b;
        dp = fR - fC - 0.5 * Mf;
        a = fR - (2.0 * fC) + fL;
        Mf = a;
        dm = fC - fL + 0.5 * Mf;
    } else if (hi) {
        a = fR - (2.0 * fC) + fL;
        Mf = a;
        dp = fR - fC - 0.5 * Mf;
        a = fR - (2.0 * fC) + fL;
        b = fC - (2.0 * fL) + fLL;
        Mf = a;
        if (std::fabs(b) < std::fabs(a)) Mf = b;
        dm = fC - fL + 0.5 * Mf;
    } else {
        a = fR - (2.0 * fC) + fL;
        b = fRR - (2.0 * fR) + fC;
        Mf = a;
        if (std::fabs(b) < std::fabs(a)) Mf = b;
        dp = fR - fC - 0.5 * Mf;
        a = fR - (2.0 * fC) + fL;
        b = fC - (2.0 * fL) + fLL;
        Mf = a;
        if (std::fabs(b) < std::fabs(a)) Mf = b;
        dm = fC - fL + 0.5 * Mf;
    }
    const double sg = std::fabs(f0) > kEpsSims ? (f0 >= 0.0 ? 1.0 : -1.0) : 0.0;
    if (sg * (fR - fC) < 0.0 && sg * (fC - fL) < -sg * (fR - fC)) return dp;
    if (sg * (fC - fL) > 0.0 && sg * (fR - fC) > -sg * (fC - fL)) return dm;
    return 0.5 * (dp + dm);
}

/* ENO2Boundary, src/AdvectionMethods.F90:654-707 */
double eno2_boundary(double f0, double f1, double f2, int bias) {
    const double as = (double)bias;
    const double D1 = as * (f1 - f0), D2 = as * (f2 - f1), D3 = as * (f2 - f0) / 2.0;
    if (std::fabs(D1 - D2) < kEpsSims) return D1;
    if (std::fabs(D1) < std::fabs(D2)) return (2.0 * D1 + D2) / 3.0;
    if (std::fabs(D2) < std::fabs(D1)) return (D1 + 2.0 * D2) / 3.0;
    if (std::fabs(D1) == std::fabs(D2)) return (4.0 * D1 + D2) / 5.0;
    if (std::fabs(D1) < std::fabs(D3) && std::fabs(D2) < std::fabs(D3)) return (3.0 * D1 + 6.0 * D2 - D3) / 7.0;
    if (std::fabs(D1) >= std::fabs(D3) && std::fabs(D2) >= std::fabs(D3)) return D3;
    return D1;
}

/* BiasedDerivative, src/AdvectionMethods.F90:248-302 (orders 1, 2, 3) */
double biased(double f0, double f1, double f2, double f3, int order, int bias, bool enobc) {
    const double as = (double)bias;
    if (order == 1) return as * (-1.0 * f0 + 1.0 * f1);
    if (order == 2) {
        if (enobc) return eno2_boundary(f0, f1, f2, bias);
        return as * (-(3.0 * f0) + 4.0 * f1 - 1.0 * f2) / 2.0;
    }
    return as * (-(11.0 * f0) + 18.0 * f1 - 9.0 * f2 + 2.0 * f3) / 6.0;
}

/* GetSignPhi0, src/AdvectionMethods.F90:576-587 */
inline double sign_phi0(double phi0, double eps) {
    if (std::fabs(phi0) > eps) return phi0 >= 0.0 ? 1.0 : -1.0;
    return phi0 / eps - 1.0 / kPi * std::sin((kPi * phi0) / eps);
}

/* GetLambdaMassCorrection, src/global_lsm.F90:200-219 */
inline double lambda_mass(double phi, double s, double ng, double eps) {
    const double d = deltaf(phi, eps);
    const double num = -d * s * (1.0 - ng);
    const double den = (d * d) * ng;
    return std::fabs(den) < kEpsSims ? 0.0 : num / den;
}

} /* namespace */
extern "C" {

/* calc_NormGrad_d, src/calc_NormGrad_d.F90:1-2448: |grad phi_RN| by ENO2 in
   each direction, one-sided BiasedDerivative along a direction whose face is
   physical at the node, zero on ghost nodes.  The blocks of the reference
   (interior, 6 faces, 12 edges, 8 corners) reduce to a per-direction choice;
   the two i-face blocks (src/calc_NormGrad_d.F90:186-376) never assign phi0,
   so their ENO2 stencil choice uses phizero at the last node of the
   interior loop (iRN_end, jRN_end, kRN_end), which is kept here. */
int oracle_calc_normgrad_d(const lsm_grid* gg, const lsm_params* p, const double* phi, const double* phizero,
                           const double* csi, const double* eta, const double* zet, double* ng) {
    int st = check_grid(gg); if (st) return st;
    if (p->OrderReinitialisationBoundaries < 1 || p->OrderReinitialisationBoundaries > 3) return LSM_ERR_BAD_PARAM;
    Grid g(gg);
    const int order = p->OrderReinitialisationBoundaries;
    const bool enobc = p->ENOBCReinitialisation != 0;
    /* interior-loop range (src/calc_NormGrad_d.F90:41-56) */
    const int is = g.ia + (g.pb ? 1 : 0), ie = g.ib - (g.pf ? 1 : 0);
    const int js = g.ja + (g.pl ? 1 : 0), je = g.jb - (g.pr ? 1 : 0);
    const int ks = g.ka + (g.pd ? 1 : 0), ke = g.kb - (g.pu ? 1 : 0);
    const double stale = phizero[g.id(ie, je, ke)];
    const long st3[3] = {1, g.ni, g.ni * g.nj};
    const double dd[3] = {g.dc, g.de, g.dz};
    std::fill(ng, ng + g.n, 0.0);
#pragma omp parallel for
    for (int k = g.ka; k <= g.kb; ++k)
        for (int j = g.ja; j <= g.jb; ++j)
            for (int i = g.ia; i <= g.ib; ++i) {
                const long l = g.id(i, j, k);
                const int c[3] = {i, j, k};
                const int lo[3] = {g.ia, g.ja, g.ka}, hi[3] = {g.ib, g.jb, g.kb};
                const int sta[3] = {is, js, ks}, end[3] = {ie, je, ke};
                const bool plo[3] = {g.pb, g.pl, g.pd}, phi_[3] = {g.pf, g.pr, g.pu};
                const bool iface = (g.pb && i == g.ia) || (g.pf && i == g.ib);
                const bool jface = (g.pl && j == g.ja) || (g.pr && j == g.jb);
                const bool kface = (g.pd && k == g.ka) || (g.pu && k == g.kb);
                const double phi0 = (iface && !jface && !kface) ? stale : phizero[l];
                double d[3];
                for (int m = 0; m < 3; ++m) {
                    const long s = st3[m];
                    if (plo[m] && c[m] == lo[m]) {
                        d[m] = dd[m] * biased(phi[l], phi[l + s], phi[l + 2 * s], phi[l + 3 * s], order, 1, enobc);
                    } else if (phi_[m] && c[m] == hi[m]) {
                        d[m] = dd[m] * biased(phi[l], phi[l - s], phi[l - 2 * s], phi[l - 3 * s], order, -1, enobc);
                    } else {
                        const bool lob = plo[m] && c[m] == sta[m], hib = phi_[m] && c[m] == end[m];
                        const double fLL = lob ? 0.0 : phi[l - 2 * s], fRR = hib ? 0.0 : phi[l + 2 * s];
                        d[m] = dd[m] * eno2(phi0, fLL, phi[l - s], phi[l], phi[l + s], fRR, lob, hib);
                    }
                }
                const double dx = csi[3 * l + 0] * d[0] + eta[3 * l + 0] * d[1] + zet[3 * l + 0] * d[2];
                const double dy = csi[3 * l + 1] * d[0] + eta[3 * l + 1] * d[1] + zet[3 * l + 1] * d[2];
                const double dz = csi[3 * l + 2] * d[0] + eta[3 * l + 2] * d[1] + zet[3 * l + 2] * d[2];
                ng[l] = std::sqrt(dx * dx + dy * dy + dz * dz);
            }
    return LSM_OK;
}

/* reinitialisation_test2, src/reinitialisation_test2.F90:1-221 (non-hybrid) */
int oracle_reinitialisation_test2(const lsm_grid* gg, const lsm_params* p, const double* phizero,
                                  const double* csi, const double* eta, const double* zet, double* out,
                                  int* iterations) {
    int st = check_grid(gg); if (st) return st;
    Grid g(gg);
    const double eps = p->epslsm, epsr = p->epsReinitialisation, dt = p->RNtimestep;
    const double C[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
    std::vector<double> sg(g.n), dn(g.n), dn1(phizero, phizero + g.n), ng(g.n, 0.0), ngc(g.n, 0.0);
    for (long l = 0; l < g.n; ++l) sg[l] = sign_phi0(phizero[l], eps);
    st = oracle_calc_normgrad_d(gg, p, dn1.data(), phizero, csi, eta, zet, ng.data());
    if (st) return st;
    int done = 0;
    for (int it = 1; it <= p->RNitermax; ++it) {
        const double mx = *std::max_element(ng.begin(), ng.end()), mn = *std::min_element(ng.begin(), ng.end());
        if (std::fabs(mx - 1.0) < epsr && std::fabs(mn - 1.0) < epsr) break;
        dn = dn1;
        oracle_calc_normgrad_d(gg, p, dn.data(), phizero, csi, eta, zet, ngc.data());
        for (int rk = 0; rk < 3; ++rk) {
            oracle_calc_normgrad_d(gg, p, dn1.data(), phizero, csi, eta, zet, ng.data());
#pragma omp parallel for
            for (int k = g.ka; k <= g.kb; ++k)
                for (int j = g.ja; j <= g.jb; ++j)
                    for (int i = g.ia; i <= g.ib; ++i) {
                        const long l = g.id(i, j, k);
                        if (ngc[l] - 1.0 > epsr) {
                            double rhs = sg[l] * (ng[l] - 1.0);
                            const double lam = lambda_mass(dn1[l], sg[l], ng[l], eps);
                            const double aux = deltaf(dn1[l], eps) * ng[l];
                            rhs = rhs - lam * aux;
                            dn1[l] = C[rk][0] * dn[l] + C[rk][1] * dn1[l] - C[rk][2] * dt * rhs;
                        }
                    }
        }
        done = it;
    }
    if (iterations) *iterations = done;
    std::memcpy(out, dn1.data(), sizeof(double) * g.n);
    return LSM_OK;
}

} /* extern "C" */

/* ====================================== geometric reinitialisation ====== */
/* The hybrid path's reinitialisation, src/geometric_reinitialisation.F90:1-94,
   restated with the reference's own data structures (lists built by the
   three loops of GetTetrahedraList) so that it checks the GPU version, which
   enumerates the same lists implicitly. */
namespace {

/* NORM2 of a 3-vector as gfortran expands the intrinsic: a scaled sum of
   squares (skip zeros; rescale when a larger magnitude appears) and
   sqrt(sum) * scale. */
inline double norm2v(const double* a) {
    double scale = 1.0, r = 0.0;
    for (int c = 0; c < 3; ++c) {
        if (a[c] != 0.0) {
            const double ax = std::fabs(a[c]);
            if (scale < ax) {
                const double v = scale / ax;
                r = 1.0 + r * v * v;
                scale = ax;
            } else {
                const double v = ax / scale;
                r = r + v * v;
            }
        }
    }
    return std::sqrt(r) * scale;
}
inline void sub3(const double* a, const double* b, double* c) {
    c[0] = a[0] - b[0]; c[1] = a[1] - b[1]; c[2] = a[2] - b[2];
}
inline double fsign1(double x) { return std::copysign(1.0, x); } /* sign(one, x) */

/* GetTriangleArea, src/TetrahedronMethods.F90:691-707 */
double tri_area(const double T[3][3]) {
    double u[3], v[3], c[3];
    sub3(T[1], T[0], u); sub3(T[2], T[0], v); cross3(u, v, c);
    return 0.5 * norm2v(c);
}

/* TetrahedronTriangles, src/TetrahedronMethods.F90:86-104 (edge numbers 0..5) */
const int kTetTris[16][6] = {{-1, -1, -1, -1, -1, -1}, {0, 3, 2, -1, -1, -1}, {0, 1, 4, -1, -1, -1},
                             {1, 4, 2, 2, 4, 3},       {1, 2, 5, -1, -1, -1}, {0, 3, 5, 0, 5, 1},
                             {0, 2, 5, 0, 5, 4},       {5, 4, 3, -1, -1, -1}, {3, 4, 5, -1, -1, -1},
                             {4, 5, 0, 5, 2, 0},       {1, 5, 0, 5, 3, 0},    {5, 2, 1, -1, -1, -1},
                             {3, 4, 2, 2, 4, 1},       {4, 1, 0, -1, -1, -1}, {2, 3, 0, -1, -1, -1},
                             {-1, -1, -1, -1, -1, -1}};

struct MTOut { int ntri; double tri[2][3][3]; double area, wv; };

/* MarchingTetrahedron with all its outputs, src/TetrahedronMethods.F90:26-664 */
void marching_tet_full(const double V[4][3], const double ph[4], MTOut* o, int* err) {
    o->ntri = 0; o->area = 0.0; o->wv = 0.0;
    std::memset(o->tri, 0, sizeof(o->tri));
    int s[4], nz = 0;
    bool allp = true, alln = true, allge = true, allle = true;
    for (int v = 0; v < 4; ++v) {
        s[v] = ph[v] > kTiny ? 1 : (ph[v] < -kTiny ? -1 : 0);
        allp &= s[v] == 1; alln &= s[v] == -1; nz += s[v] == 0;
        allge &= s[v] >= 0; allle &= s[v] <= 0;
    }
    if (allp) { o->wv = tet_volume(V[0], V[1], V[2], V[3]); return; }
    if (alln) return;
    int fi = 0;
    auto put = [&](int a, int b, int c) {
        for (int q = 0; q < 3; ++q) { o->tri[0][0][q] = V[a][q]; o->tri[0][1][q] = V[b][q]; o->tri[0][2][q] = V[c][q]; }
    };
    auto vol_if = [&](bool water) { o->wv = water ? tet_volume(V[0], V[1], V[2], V[3]) : 0.0; };
    if (nz > 0 && (allge || allle)) {
        if (nz == 1) { /* one zero vertex: a point "isosurface", ntriangles = -1 */
            o->ntri = -1;
            if (s[0] == 0) { put(0, 0, 0); vol_if(s[1] == 1); return; }
            if (s[1] == 0) { put(1, 1, 1); vol_if(s[0] == 1); return; }
            if (s[2] == 0) { put(2, 2, 2); vol_if(s[0] == 1); return; }
            put(3, 3, 3); vol_if(s[0] == 1); return;
        }
        if (nz == 2) { /* an edge, ntriangles = -2 */
            o->ntri = -2;
            if (s[0] == 0 && s[1] == 0) { put(0, 1, 1); vol_if(s[2] == 1); return; }
            if (s[1] == 0 && s[2] == 0) { put(1, 2, 2); vol_if(s[0] == 1); return; }
            if (s[2] == 0 && s[0] == 0) { put(2, 0, 0); vol_if(s[1] == 1); return; }
            if (s[0] == 0 && s[3] == 0) { put(0, 3, 3); vol_if(s[1] == 1); return; }
            if (s[1] == 0 && s[3] == 0) { put(1, 3, 3); vol_if(s[0] == 1); return; }
            put(2, 3, 3); vol_if(s[0] == 1); return;
        }
        if (nz == 3) { /* a face, one triangle */
            o->ntri = 1;
            const int f[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
            for (int v = 0; v < 4; ++v)
                if (s[v] != 0) {
                    put(f[v][0], f[v][1], f[v][2]);
                    o->area = tri_area(o->tri[0]);
                    vol_if(s[v] == 1);
                    return;
                }
        }
        /* four zero vertices: FlagIndex stays 0 */
    } else {
        for (int v = 0; v < 4; ++v)
            if (s[v] == -1) fi |= 1 << v;
    }
    if (fi == 0) o->wv = tet_volume(V[0], V[1], V[2], V[3]);
    if (fi == 15) o->wv = 0.0;
    const int ef = kEdgeFlags[fi];
    if (ef == 0) return;
    double E[6][3];
    for (int e = 0; e < 6; ++e) E[e][0] = E[e][1] = E[e][2] = -9.9;
    for (int e = 0; e < 6; ++e) {
        if (!(ef >> e & 1)) continue;
        const int sv = kEdge[e][0], ev = kEdge[e][1];
        const double den = ph[ev] - ph[sv];
        const double sc = std::fabs(den) < kEpsSims * kEpsSims * kEpsSims ? 0.0 : ph[ev] / den;
        for (int c = 0; c < 3; ++c) E[e][c] = V[ev][c] + sc * (V[sv][c] - V[ev][c]);
    }
    for (int t = 0; t < 2; ++t) {
        if (kTetTris[fi][3 * t] < 0) break;
        o->ntri += 1;
        for (int v = 0; v < 3; ++v)
            for (int c = 0; c < 3; ++c) o->tri[t][v][c] = E[kTetTris[fi][3 * t + v]][c];
        o->area = o->area + tri_area(o->tri[t]);
    }
    if (fi == 0) o->wv = tet_volume(V[0], V[1], V[2], V[3]);
    else if (fi == 15) o->wv = 0.0;
    else o->wv = water_volume(V, E, fi, err);
}

/* DistancePointLine, src/TetrahedronMethods.F90:1356-1399 */
double dist_point_line(const double* A, const double* B, const double* P) {
    double AB[3], AP[3], BA[3], BP[3];
    sub3(B, A, AB); sub3(P, A, AP); sub3(A, B, BA); sub3(P, B, BP);
    bool valid = true;
    if (norm2v(AB) < kEpsSims) valid = false;
    if (dot3(AB, AP) < 0.0) valid = false;
    if (dot3(BA, BP) < 0.0) valid = false;
    if (valid) {
        double c[3];
        cross3(AP, BP, c);
        return norm2v(c) / norm2v(AB);
    }
    const double a = norm2v(AP), b = norm2v(BP);
    return b < a ? b : a;
}

/* CheckProjectionPointOnATriangle3, src/TetrahedronMethods.F90:1593-1684.
   Kept from the reference: alpha (the weight of P3 in the standard
   barycentric form) multiplies P1 and gamma multiplies P3. */
bool projection3(const double T[3][3], const double* P, double* pd) {
    double d[3];
    sub3(T[0], T[1], d); if (norm2v(d) <= kEpsSims) return false;
    sub3(T[0], T[2], d); if (norm2v(d) <= kEpsSims) return false;
    sub3(T[1], T[2], d); if (norm2v(d) <= kEpsSims) return false;
    double u[3], v[3], w[3], nv[3], cu[3], cw[3];
    sub3(T[1], T[0], u); sub3(T[2], T[0], v); sub3(P, T[0], w);
    cross3(u, v, nv);
    cross3(u, w, cu); cross3(w, v, cw);
    const double nn = dot3(nv, nv);
    const double alpha = dot3(cu, nv) / nn;
    const double beta = dot3(cw, nv) / nn;
    const double gamma = 1.0 - beta - alpha;
    double pp[3], dd[3];
    for (int c = 0; c < 3; ++c) pp[c] = alpha * T[0][c] + beta * T[1][c] + gamma * T[2][c];
    sub3(P, pp, dd);
    const double dist = norm2v(dd);
    const bool inside = alpha > 0.0 && alpha < 1.0 && beta > 0.0 && beta < 1.0 && gamma > 0.0 && gamma < 1.0;
    *pd = inside ? dist : 999.9;
    return inside;
}

/* DistancePointTriangle, src/TetrahedronMethods.F90:1008-1070 */
double dist_point_triangle(const double T[3][3], const double* P) {
    double d[3];
    sub3(P, T[0], d); double m = norm2v(d);
    sub3(P, T[1], d); m = std::min(m, norm2v(d));
    sub3(P, T[2], d); m = std::min(m, norm2v(d));
    m = std::min(m, dist_point_line(T[0], T[1], P));
    m = std::min(m, dist_point_line(T[1], T[2], P));
    m = std::min(m, dist_point_line(T[2], T[0], P));
    double pd;
    if (projection3(T, P, &pd)) m = std::min(m, pd);
    return m;
}

/* the reference's running minimum: d + exsign (da - d), exsign = 1 when da <= d */
inline double run_min(double d, double da) {
    const double ex = (fsign1(d - da) + 1.0) / 2.0;
    return d + ex * (da - d);
}

const int kCellOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
const int kCellTets[6][4] = {{0, 5, 1, 6}, {0, 1, 2, 6}, {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}, {0, 4, 5, 6}};

/* CellPnodeTetrahedronIdentification, src/TetrahedronMethods.F90:2124-2361
   (TriangulationCase 1): bit t (1..6) of *tets marks a phase-change
   tetrahedron, bit v (0..7) of *verts a vertex of one. */
void cell_pnodes(const double P[8], int* verts, int* tets) {
    *verts = 0; *tets = 0;
    bool allw = true, alla = true, anyz = false;
    for (int v = 0; v < 8; ++v) {
        allw &= P[v] > kEpsSims; alla &= P[v] < -kEpsSims; anyz |= std::fabs(P[v]) < kEpsSims;
    }
    if (allw || alla) return;
    bool pc = anyz;
    if (!pc) {
        const double s0 = fsign1(P[0]);
        for (int v = 1; v < 8 && !pc; ++v) pc = s0 * P[v] < 0.0;
    }
    if (!pc) return;
    for (int t = 0; t < 6; ++t) {
        double a = P[kCellTets[t][0]];
        bool change = std::fabs(a) < kEpsSims, second = !(a <= kEpsSims);
        const double sg = fsign1(a);
        for (int q = 1; q < 4; ++q) {
            a = P[kCellTets[t][q]];
            if (sg * a < 0.0 || std::fabs(a) < kEpsSims) {
                if (a <= kEpsSims) second = false;
                change = true;
            }
        }
        if (change && !second) {
            *tets |= 1 << (t + 1);
            for (int q = 0; q < 4; ++q) *verts |= 1 << kCellTets[t][q];
        }
    }
}

struct GPNode { int i, j, k; double x, y, z, phi, sd, xi; int nasoc; int asoc[24]; };
struct GKTet { int v[4]; int nis; double tri[2][3][3]; double area, wv, etaK; };

struct Geo {
    const Grid& g;
    std::vector<GPNode> nodes;
    std::vector<GKTet> tets;
    explicit Geo(const Grid& gg) : g(gg) {}

    void vertices(const GKTet& t, double V[4][3]) const {
        for (int q = 0; q < 4; ++q) {
            const GPNode& n = nodes[t.v[q]];
            V[q][0] = n.x; V[q][1] = n.y; V[q][2] = n.z;
        }
    }
    /* the distance loop body shared by GetIsosurfaceAndDistances and
       NeighboursPhiCorrection: triangles of tetrahedron t against point P */
    double tet_min(const GKTet& t, const double* P, double d) const {
        if (t.nis > 0 && t.area > 0.0) {
            d = run_min(d, dist_point_triangle(t.tri[0], P));
            if (t.nis > 1) d = run_min(d, dist_point_triangle(t.tri[1], P));
        }
        return d;
    }
};

/* LocalVolumeVariation, src/TetrahedronMethods.F90:2390-2437 */
double local_dv(double eta, const double V[4][3], const double ph[4], double v0, int* err) {
    double a[4];
    for (int q = 0; q < 4; ++q) a[q] = ph[q] + eta;
    MTOut o;
    marching_tet_full(V, a, &o, err);
    return v0 - o.wv;
}

/* SecantMethodLocalCorrection, src/TetrahedronMethods.F90:2439-2588 */
double secant_eta(const double V[4][3], double vol0, double area0, const double ph[4], double tol, int maxit,
                  bool* conv, int* err) {
    *conv = false;
    MTOut o;
    marching_tet_full(V, ph, &o, err);
    const double dv0 = vol0 - o.wv;
    if (std::fabs(dv0) < tol) { *conv = true; return 0.0; }
    double x0 = o.area > kEpsSims ? dv0 / o.area : 0.0;
    double x1 = area0 > kEpsSims ? dv0 / area0 : 0.0;
    double f0 = local_dv(x0, V, ph, vol0, err);
    double f1 = local_dv(x1, V, ph, vol0, err);
    if (std::fabs(f0) < tol || std::fabs(f1) < tol) {
        *conv = true;
        return std::fabs(f1) < std::fabs(f0) ? x1 : x0;
    }
    double x2 = 0.0; /* unset in the reference when the loop exits at once (then not converged) */
    for (int it = 1; it <= maxit; ++it) {
        if (std::fabs(f1 - f0) < kEpsSims) break;
        x2 = x1 - f1 * (x1 - x0) / (f1 - f0);
        x0 = x1; x1 = x2; f0 = f1;
        f1 = local_dv(x1, V, ph, vol0, err);
        if (std::fabs(f1) < tol) { *conv = true; break; }
    }
    if (std::fabs(f1) > dv0) x2 = 0.0;
    return x2;
}

/* funcv, src/NewtonRaphsonSolver.F90: target - K-tetrahedra volume of
   phi* + C xi (a node's correction is dropped where it changes the sign) */
double geo_funcv(const Geo& G, double target, double C, int* err) {
    double tot = 0.0;
    for (const GKTet& t : G.tets) {
        double V[4][3], a[4];
        G.vertices(t, V);
        for (int q = 0; q < 4; ++q) {
            const GPNode& n = G.nodes[t.v[q]];
            const double sd = n.sd, ca = C * n.xi;
            a[q] = sd + ca / 2.0 * std::fabs(fsign1(sd) + fsign1(sd + ca));
        }
        MTOut o;
        marching_tet_full(V, a, &o, err);
        tot = tot + o.wv;
    }
    return target - tot;
}

/* NewtonRaphson + newt/fdjac/fmin/lnsrch/ludcmp/lubksb for one unknown,
   src/NewtonRaphsonSolver.F90 (Numerical Recipes' globally convergent
   Newton).  The PARAMETERs written as default-real literals (1.e-12, 1.e-7,
   1.e-4, .1) are single precision promoted to REAL(8).  Returns C. */
template <class F>
double newton_1d(F funcv, double tol, int* its_out, bool* converged) {
    const int MAXITS = 20;
    const double TOLF = (double)1.e-12f, TOLMIN = (double)1.e-12f, TOLX = (double)1.e-12f, STPMX = 100.0;
    const double ALF = (double)1.e-4f, TOLXL = (double)1.e-7f, P1 = (double)0.1f;
    const double EPS = std::sqrt(kEpsSims);
    double x = 0.0;            /* C_initial_guest */
    bool check = false;        /* not set by newt on its zero-Jacobian return */
    int its = 1;
    double fvec = funcv(x);
    double f = 0.5 * (0.0 + fvec * fvec);
    auto finish = [&](bool conv_path) {
        (void)conv_path;
        *its_out = its;
        *converged = its < MAXITS && !check;
        return *converged ? x : 0.0;
    };
    if (std::fabs(fvec) < 0.01 * TOLF && std::fabs(fvec) < tol) { check = false; return finish(true); }
    const double stpmax = STPMX * std::max(std::sqrt(0.0 + x * x), 1.0);
    for (its = 1; its <= MAXITS; ++its) {
        /* fdjac */
        const double temp = x;
        double h = EPS * std::fabs(temp);
        if (h < kEpsSims) h = EPS;
        x = temp + h;
        h = x - temp;
        const double fh = funcv(x);
        x = temp;
        double fjac = (fh - fvec) / h;
        if (std::fabs(0.0 + fjac) < tol) return finish(false); /* zero Jacobian */
        fvec = funcv(x);
        const double gr = 0.0 + fjac * fvec;
        const double xold = x, fold = f;
        double p = -fvec;
        /* ludcmp / lubksb, n = 1 */
        if (fjac == 0.0) fjac = 1.0e-20;
        p = p / fjac;
        /* lnsrch */
        check = false;
        const double sum = std::sqrt(0.0 + p * p);
        if (sum > stpmax) p = p * stpmax / sum;
        const double slope = 0.0 + gr * p;
        const double test = std::fabs(p) / std::max(std::fabs(xold), 1.0);
        const double alamin = TOLXL / test;
        double alam = 1.0, alam2 = 2.0, f2 = 2.0, tmplam = 0.0;
        for (;;) {
            x = xold + alam * p;
            fvec = funcv(x);
            f = 0.5 * (0.0 + fvec * fvec);
            if (alam < alamin) { x = xold; check = true; break; }
            if (f <= fold + ALF * alam * slope) break;
            if (alam == 1.0) {
                tmplam = -slope / (2.0 * (f - fold - slope));
            } else {
                const double rhs1 = f - fold - alam * slope, rhs2 = f2 - fold - alam2 * slope;
                const double a = (rhs1 / (alam * alam) - rhs2 / (alam2 * alam2)) / (alam - alam2);
                const double b = (-alam2 * rhs1 / (alam * alam) + alam * rhs2 / (alam2 * alam2)) / (alam - alam2);
                if (a == 0.0) {
                    tmplam = -slope / (2.0 * b);
                } else {
                    const double disc = b * b - 3.0 * a * slope;
                    if (disc < 0.0) tmplam = 0.5 * alam;
                    else if (b <= 0.0) tmplam = (-b + std::sqrt(disc)) / (3.0 * a);
                    else tmplam = -slope / (b + std::sqrt(disc));
                }
                if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
            }
            alam2 = alam; f2 = f;
            alam = std::max(tmplam, P1 * alam);
        }
        if (std::fabs(fvec) < TOLF && std::fabs(fvec) < tol) { check = false; return finish(true); }
        if (check) {
            const double den = std::max(f, 0.5 * 1);
            const double t2 = std::fabs(gr) * std::max(std::fabs(x), 1.0) / den;
            check = t2 < TOLMIN; /* spurious convergence: check stays set */
            return finish(false);
        }
        const double t3 = std::fabs(x - xold) / std::max(std::fabs(x), 1.0);
        if (t3 < TOLX && std::fabs(fvec) < tol) return finish(true);
    }
    return finish(false); /* its = MAXITS + 1 */
}

double geo_newton(const Geo& G, double target, double tol, int* its_out, bool* converged, int* err) {
    return newton_1d([&](double c) { return geo_funcv(G, target, c, err); }, tol, its_out, converged);
}

} /* namespace */

extern "C" {

/* The Newton solve alone, on a caller's function f(ud, C) = target - volume(C)
   (test entry: the product's solver is checked against this one). */
int oracle_newton_1d(double (*f)(void*, double), void* ud, double tol, int* its, int* conv, double* C) {
    bool c = false;
    *C = newton_1d([&](double x) { return f(ud, x); }, tol, its, &c);
    *conv = c ? 1 : 0;
    return LSM_OK;
}

/* geometric_reinitialisation, src/geometric_reinitialisation.F90:1-94
   (TriangulationCase 1, one rank, no ghost planes, no blanking).
   info (nullable): [nnodes, ntetrahedra, nsecond, newton its, converged]. */
int oracle_geometric_reinitialisation(const lsm_grid* gg, const lsm_params* p, const double* phi0, const double* x,
                                      const double* y, const double* z, double total_water_volume, double* pc,
                                      int* ids, int* info_i, double* info_c) {
    int st = check_grid(gg); if (st) return st;
    if (gg->igp || gg->jgp || gg->kgp) return LSM_ERR_UNSUPPORTED;
    for (int f = 0; f < 6; ++f) if (!gg->physical_face[f]) return LSM_ERR_UNSUPPORTED;
    Grid g(gg);
    Geo G(g);
    int err = 0;
    std::memset(ids, 0, sizeof(int) * g.n);
    /* GetTetrahedraList, first loop: cells, pnode flags and K-tetrahedra bits */
    std::vector<int> cellbits(g.n, 0);
    for (int k = g.kl; k < g.ku; ++k)
        for (int j = g.jl; j < g.ju; ++j)
            for (int i = g.il; i < g.iu; ++i) {
                double P[8];
                for (int v = 0; v < 8; ++v) P[v] = phi0[g.id(i + kCellOff[v][0], j + kCellOff[v][1], k + kCellOff[v][2])];
                int verts, tets;
                cell_pnodes(P, &verts, &tets);
                for (int v = 0; v < 8; ++v)
                    if (verts >> v & 1) ids[g.id(i + kCellOff[v][0], j + kCellOff[v][1], k + kCellOff[v][2])] = 1;
                cellbits[g.id(i, j, k)] = tets;
            }
    /* second loop: number the pnodes in k, j, i order */
    for (int k = g.kl; k <= g.ku; ++k)
        for (int j = g.jl; j <= g.ju; ++j)
            for (int i = g.il; i <= g.iu; ++i) {
                const long l = g.id(i, j, k);
                if (ids[l] > 0) {
                    GPNode n{};
                    n.i = i; n.j = j; n.k = k;
                    n.x = x[l]; n.y = y[l]; n.z = z[l]; n.phi = phi0[l];
                    n.sd = 99.9; n.xi = 0.0; n.nasoc = 0;
                    G.nodes.push_back(n);
                    ids[l] = (int)G.nodes.size();
                }
            }
    /* third loop: the K tetrahedra and each pnode's list of them */
    for (int k = g.kl; k < g.ku; ++k)
        for (int j = g.jl; j < g.ju; ++j)
            for (int i = g.il; i < g.iu; ++i) {
                const int bits = cellbits[g.id(i, j, k)];
                if (!bits) continue;
                int nid[8];
                for (int v = 0; v < 8; ++v) nid[v] = ids[g.id(i + kCellOff[v][0], j + kCellOff[v][1], k + kCellOff[v][2])];
                for (int t = 0; t < 6; ++t) {
                    if (!(bits >> (t + 1) & 1)) continue;
                    GKTet T{};
                    for (int q = 0; q < 4; ++q) T.v[q] = nid[kCellTets[t][q]] - 1;
                    const int tid = (int)G.tets.size();
                    G.tets.push_back(T);
                    for (int q = 0; q < 4; ++q) {
                        GPNode& n = G.nodes[T.v[q]];
                        n.asoc[n.nasoc++] = tid;
                    }
                }
            }
    /* GetIsosurfaceAndDistances: marching tetrahedra on the K tetrahedra */
    const long ntet = (long)G.tets.size(), npn = (long)G.nodes.size();
#pragma omp parallel for schedule(static) reduction(| : err)
    for (long it = 0; it < ntet; ++it) {
        GKTet& t = G.tets[it];
        double V[4][3], ph[4];
        G.vertices(t, V);
        for (int q = 0; q < 4; ++q) ph[q] = G.nodes[t.v[q]].phi;
        MTOut o;
        marching_tet_full(V, ph, &o, &err);
        t.area = o.area; t.wv = o.wv;
        t.nis = o.ntri > 0 ? o.ntri : 0;
        std::memcpy(t.tri, o.tri, sizeof(t.tri));
    }
    /* ... the pnodes' distances over the +-4 box ... (the reference tags the
       box's non-pnodes -1 inside the same loop; the tags change no test of
       the loop, which only asks for ids > 0, so they are a pass of their
       own here and the distance loop reads ids only) */
#pragma omp parallel for schedule(dynamic, 16)
    for (long ip = 0; ip < npn; ++ip) {
        GPNode& n = G.nodes[ip];
        const double P[3] = {n.x, n.y, n.z};
        double dp = 10.0;
        for (int ks = std::max(n.k - 4, g.kl); ks <= std::min(n.k + 4, g.ku); ++ks)
            for (int js = std::max(n.j - 4, g.jl); js <= std::min(n.j + 4, g.ju); ++js)
                for (int is = std::max(n.i - 4, g.il); is <= std::min(n.i + 4, g.iu); ++is) {
                    const long l = g.id(is, js, ks);
                    if (ids[l] > 0) {
                        const GPNode& m = G.nodes[ids[l] - 1];
                        for (int a = 0; a < m.nasoc; ++a) {
                            dp = G.tet_min(G.tets[m.asoc[a]], P, dp);
                            const double asd = std::fabs(n.sd);
                            const double ex2 = (fsign1(asd - dp) + 1.0) / 2.0;
                            n.sd = asd + ex2 * (dp - asd);
                            n.sd = fsign1(n.phi) * n.sd;
                        }
                    }
                }
    }
    /* ... and the -1 tags */
    for (const GPNode& n : G.nodes)
        for (int ks = std::max(n.k - 4, g.kl); ks <= std::min(n.k + 4, g.ku); ++ks)
            for (int js = std::max(n.j - 4, g.jl); js <= std::min(n.j + 4, g.ju); ++js)
                for (int is = std::max(n.i - 4, g.il); is <= std::min(n.i + 4, g.iu); ++is) {
                    const long l = g.id(is, js, ks);
                    if (ids[l] <= 0) ids[l] = -1;
                }
    /* GlobalMassCorrection: per-tetrahedron eta (secant), xi, Newton's C */
    double Cc = 0.0;
    int its = 0;
    bool conv = false;
    if (p->GlobalMassCorrection) {
        const double tol = p->ConvergenceToleranceGeomReini / 1000.0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : err)
        for (long it = 0; it < ntet; ++it) {
            GKTet& t = G.tets[it];
            double V[4][3], ph[4];
            G.vertices(t, V);
            for (int q = 0; q < 4; ++q) ph[q] = G.nodes[t.v[q]].sd;
            bool c = false;
            const double e = secant_eta(V, t.wv, t.area, ph, tol, 40, &c, &err);
            t.etaK = c ? e : 0.0;
        }
        for (GPNode& n : G.nodes)
            for (int a = 0; a < n.nasoc; ++a) n.xi = n.xi + G.tets[n.asoc[a]].etaK / (double)n.nasoc;
        Cc = geo_newton(G, total_water_volume, p->ConvergenceToleranceGeomReini, &its, &conv, &err);
    }
    /* NeighboursPhiCorrection: pnodes ... */
    for (GPNode& n : G.nodes) {
        const double pcf = std::fabs(fsign1(n.sd) + fsign1(n.sd + Cc * n.xi)) / 2.0;
        const double aux = pcf * Cc * n.xi;
        n.phi = n.sd + aux;
        pc[g.id(n.i, n.j, n.k)] = n.phi;
    }
    /* ... and the -1 nodes (each reads and writes its own value only) */
    int nsecond = 0;
#pragma omp parallel for collapse(2) schedule(dynamic, 4) reduction(+ : nsecond)
    for (int k = g.kl; k <= g.ku; ++k)
        for (int j = g.jl; j <= g.ju; ++j)
            for (int i = g.il; i <= g.iu; ++i) {
                const long l0 = g.id(i, j, k);
                if (ids[l0] >= 0) continue;
                ++nsecond;
                const int km = std::max(k - 4, g.kl), kp = std::min(k + 4, g.ku);
                const int jm = std::max(j - 4, g.jl), jp = std::min(j + 4, g.ju);
                const int im = std::max(i - 4, g.il), ip = std::min(i + 4, g.iu);
                const double P[3] = {x[l0], y[l0], z[l0]};
                for (int ks = km; ks <= kp; ++ks)
                    for (int js = jm; js <= jp; ++js)
                        for (int is = im; is <= ip; ++is) {
                            const long l = g.id(is, js, ks);
                            if (ids[l] <= 0) continue;
                            const GPNode& m = G.nodes[ids[l] - 1];
                            double dp = 10.0;
                            for (int a = 0; a < m.nasoc; ++a) {
                                dp = G.tet_min(G.tets[m.asoc[a]], P, dp);
                                const double apc = std::fabs(pc[l0]);
                                const double ex2 = (fsign1(apc - dp) + 1.0) / 2.0;
                                const double aux = apc + ex2 * (dp - apc);
                                pc[l0] = fsign1(pc[l0]) * aux;
                            }
                        }
            }
    if (info_i) {
        info_i[0] = (int)G.nodes.size(); info_i[1] = (int)G.tets.size(); info_i[2] = nsecond;
        info_i[3] = its; info_i[4] = conv ? 1 : 0;
    }
    if (info_c) *info_c = Cc;
    return err ? LSM_ERR_NEGATIVE_VOLUME : LSM_OK;
}


/* ------------------------------------------------------------------ A0 --- */
/* levelsetmethod, src/levelsetmethod.F90:1-372: the hybrid branch
   (geometric reinitialisation, advection on the AdvectionNodes band) or the
   Sussman-Fatemi branch with `reinitialization` (reinit_scheme 0) or the
   live `reinitialisation_test2` (reinit_scheme 1). */
int oracle_levelsetmethod_x(const lsm_grid* gg, const lsm_params* p, const double* q, const double* csi,
                            const double* eta, const double* zet, const double* aj, double* phi,
                            const double* phin, const double* x, const double* y, const double* z, int iter,
                            double* vols, lsm_exchange_fn fn, void* user) {
    int st = check_grid(gg); if (st) return st;
    if (p->reinit_scheme < 0 || p->reinit_scheme > 1 || p->sussman_correction_method != 0)
        return LSM_ERR_UNSUPPORTED;
    const bool hybrid = p->call_reinitialisation && p->hybrid_reinitialisation;
    Grid g(gg);
    Exch ex{fn, user, gg};
    std::vector<int> adv(g.n);
    double v[4];
    st = oracle_total_water_volume(gg, phi, x, y, z, v, adv.data());
    if (st) return st;
    if (vols) std::memcpy(vols, v, sizeof(v));
    /* AdvectionNodes = 1 unless (reinit .and. hybrid), levelsetmethod.F90:218-219 */
    if (!hybrid) std::fill(adv.begin(), adv.end(), 1);
    std::vector<double> pc(g.n, 0.0); /* phicorrected = zero, :147 */
    if (p->call_levelsetmethod) {
        std::memcpy(pc.data(), phin, sizeof(double) * g.n);
        std::vector<double> ucn(3 * g.n);
        oracle_rhs_contra_j(gg, q, csi, eta, zet, aj, ucn.data());
        for (int it = 0; it < p->numiter_lsm; ++it) {
            oracle_ad_rktvd3_x(gg, p, phi, pc.data(), adv.data(), ucn.data(), aj, fn, user);
            std::memcpy(pc.data(), phi, sizeof(double) * g.n);
        }
    }
    /* ConvergenceVolume, :245-264 */
    double conv = v[3];
    if (p->GlobalMassCorrection) {
        double w[4];
        st = oracle_total_water_volume(gg, phi, x, y, z, w, nullptr);
        if (st) return st;
        conv = v[3] - (w[0] + w[1]);
    }
    if (p->call_reinitialisation && p->RNfreq > 0 && iter % p->RNfreq == 0) {
        if (p->hybrid_reinitialisation) {
            /* :300-309: +-9.9 off the interface, then the geometric reinitialisation */
            for (long l = 0; l < g.n; ++l) {
                if (phi[l] < -kEpsSims) pc[l] = -9.9;
                if (phi[l] > kEpsSims) pc[l] = 9.9;
            }
            std::vector<int> ids(g.n);
            st = oracle_geometric_reinitialisation(gg, p, phi, x, y, z, conv, pc.data(), ids.data(), nullptr,
                                                   nullptr);
            if (st) return st;
        } else if (p->reinit_scheme == 1) oracle_reinitialisation_test2(gg, p, phi, csi, eta, zet, pc.data(), nullptr);
        else oracle_reinitialization_x(gg, p, phi, csi, eta, zet, pc.data(), fn, user);
        bcond(g, p, pc.data());
        std::memcpy(phi, pc.data(), sizeof(double) * g.n);
        ex(phi);
    }
    return LSM_OK;
}

int oracle_levelsetmethod(const lsm_grid* gg, const lsm_params* p, const double* q, const double* csi,
                          const double* eta, const double* zet, const double* aj, double* phi,
                          const double* phin, const double* x, const double* y, const double* z, int iter,
                          double* vols) {
    return oracle_levelsetmethod_x(gg, p, q, csi, eta, zet, aj, phi, phin, x, y, z, iter, vols, nullptr,
                                   nullptr);
}

/* number of OpenMP threads this build uses (1 for the serial build) */
int oracle_num_threads(void) {
#ifdef _OPENMP
    int n = 1;
#pragma omp parallel
    {
#pragma omp single
        n = omp_get_num_threads();
    }
    return n;
#else
    return 1;
#endif
}

} /* extern "C" */
