/* euler_oracle.c -- CPU oracle of the Eulerian grid hydrocode (TEST ONLY).
 * See euler_oracle.h.  Line references are to hydrocodes/euler/hydro_cpu.cpp
 * of the reference; the operation order of every expression is the
 * reference's (bit-exact pinning against the reference compiled here). */
#include "euler_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NF 16 /* per-cell fields of the grid */
#define ND 14 /* fields of the right-hand side */
static const char* FIELD_NAMES[NF] = {"r",   "mu",  "mv", "mw", "E",  "Sxx", "Syy", "Szz",
                                      "Sxy", "Sxz", "Syz", "D", "af", "rc",  "vib", "Pmax"};
static const char* RHS_NAMES[ND] = {"r", "mu", "mv", "mw", "E", "Sxx", "Syy", "Szz",
                                    "Sxy", "Sxz", "Syz", "D", "rc", "vib"};
enum { F_R, F_MU, F_MV, F_MW, F_E, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ, F_D, F_AF, F_RC, F_VIB, F_PMAX };
enum { D_R, D_MU, D_MV, D_MW, D_E, D_SXX, D_SYY, D_SZZ, D_SXY, D_SXZ, D_SYZ, D_D, D_RC, D_VIB };

struct eorc_grid {
    int nx, ny, nz, n;
    double dx;
    double* f[NF];
    double* d[ND];
    orc_material mat;
    eorc_params p;
    double *ref_r0, *ref_p0; /* hydrostatic reference (set_ref), NULL when off */
    long visc_iters;         /* conjugate-gradient iterations of the implicit viscosity */
};

static inline double dmax2(double a, double b) { return a < b ? b : a; } /* std::max */
static inline double dmin2(double a, double b) { return b < a ? b : a; } /* std::min */
static inline int imax2(int a, int b) { return a < b ? b : a; }
static inline int imin2(int a, int b) { return b < a ? b : a; }

void eorc_params_default(eorc_params* p) { /* hydro_cpu.cpp:17-36, 222 */
    memset(p, 0, sizeof *p);
    p->p_coh = 1.0e6;
    p->damp = 1.0;
    p->y_i0 = 1.0e7;
    p->mu_i = 1.2;
    p->mu_d = 0.6;
    p->y_m = 2.5e9;
    p->c_reg = 0.1;
    p->af_sat = 1.0;
}

eorc_grid* eorc_create(int nx, int ny, int nz, double dx) {
    eorc_grid* g = (eorc_grid*)calloc(1, sizeof *g);
    g->nx = nx; g->ny = ny; g->nz = nz; g->n = nx * ny * nz; g->dx = dx;
    for (int q = 0; q < NF; q++) g->f[q] = (double*)calloc((size_t)(g->n > 0 ? g->n : 1), sizeof(double));
    for (int q = 0; q < ND; q++) g->d[q] = (double*)calloc((size_t)(g->n > 0 ? g->n : 1), sizeof(double));
    g->mat = orc_mat_ideal(1.4);
    eorc_params_default(&g->p);
    return g;
}

void eorc_destroy(eorc_grid* g) {
    if (!g) return;
    free(g->ref_r0);
    free(g->ref_p0);
    for (int q = 0; q < NF; q++) free(g->f[q]);
    for (int q = 0; q < ND; q++) free(g->d[q]);
    free(g);
}

void eorc_set_material(eorc_grid* g, const orc_material* m) { g->mat = *m; }
void eorc_set_params(eorc_grid* g, const eorc_params* p) { g->p = *p; }

double* eorc_field(eorc_grid* g, const char* name) {
    for (int q = 0; q < NF; q++)
        if (!strcmp(name, FIELD_NAMES[q])) return g->f[q];
    return NULL;
}

double* eorc_rhs(eorc_grid* g, const char* name) {
    for (int q = 0; q < ND; q++)
        if (!strcmp(name, RHS_NAMES[q])) return g->d[q];
    return NULL;
}

static inline int idx(const eorc_grid* g, int i, int j, int k) { return (i * g->ny + j) * g->nz + k; }

/* hydro_cpu.cpp:38 */
static inline void eos_pc(const orc_material* m, double rho, double e, double* p, double* cs) {
    *p = orc_pressure(m, rho, e);
    if (*p < 0) *p = 0;
    *cs = orc_sound_speed(m, rho, e);
}

/* hydro_cpu.cpp:94 */
static inline double eint(const eorc_grid* g, int c) {
    const double* r = g->f[F_R];
    double ke = 0.5 * (g->f[F_MU][c] * g->f[F_MU][c] + g->f[F_MV][c] * g->f[F_MV][c] +
                       g->f[F_MW][c] * g->f[F_MW][c]) / r[c];
    return (g->f[F_E][c] - ke) / r[c];
}

double eorc_pcell(const eorc_grid* g, int c) { /* hydro_cpu.cpp:95 */
    double p, cs;
    eos_pc(&g->mat, g->f[F_R][c], eint(g, c), &p, &cs);
    return p;
}

typedef struct { double r, mn, mt1, mt2, E; } F5;

/* Exact rarefaction into vacuum sampled at the face, hydro_cpu.cpp:43-53. */
static F5 vac_flux(const orc_material* m, double rM, double vnM, double t1M, double t2M, double eM, int side) {
    double pM, cM;
    eos_pc(m, rM, eM, &pM, &cM);
    double g = rM * cM * cM / dmax2(pM, 1e-30);
    if (g < 1.01) g = 1.01;
    if (g > 1e5) g = 1e5;
    double s = (double)side, vn = s * vnM;
    if (vn - cM >= 0) {
        double E = rM * eM + 0.5 * rM * (vnM * vnM + t1M * t1M + t2M * t2M);
        F5 o = {rM * vnM, rM * vnM * vnM + pM, rM * vnM * t1M, rM * vnM * t2M, (E + pM) * vnM};
        return o;
    }
    if (vn + 2 * cM / (g - 1) <= 0) {
        F5 z = {0, 0, 0, 0, 0};
        return z;
    }
    double u0 = 2.0 / (g + 1) * (cM + 0.5 * (g - 1) * vn), c0 = u0;
    double r0 = rM * pow(c0 / cM, 2.0 / (g - 1)), p0 = pM * pow(r0 / rM, g), e0 = p0 / ((g - 1) * r0), un0 = s * u0;
    double E0 = r0 * e0 + 0.5 * r0 * (un0 * un0 + t1M * t1M + t2M * t2M);
    F5 o = {r0 * un0, r0 * un0 * un0 + p0, r0 * un0 * t1M, r0 * un0 * t2M, (E0 + p0) * un0};
    return o;
}

static inline F5 flux_of(double r, double vn, double t1, double t2, double p, double E) {
    F5 o = {r * vn, r * vn * vn + p, r * vn * t1, r * vn * t2, (E + p) * vn};
    return o;
}

static inline F5 hllc_star(double r, double vn, double t1, double t2, double p, double E, double S, double Ss, F5 Fk) {
    double f = r * (S - vn) / (S - Ss);
    F5 Us = {f, f * Ss, f * t1, f * t2, f * (E / r + (Ss - vn) * (Ss + p / (r * (S - vn))))};
    F5 U = {r, r * vn, r * t1, r * t2, E};
    F5 o = {Fk.r + S * (Us.r - U.r), Fk.mn + S * (Us.mn - U.mn), Fk.mt1 + S * (Us.mt1 - U.mt1),
            Fk.mt2 + S * (Us.mt2 - U.mt2), Fk.E + S * (Us.E - U.E)};
    return o;
}

/* HLLC face flux, hydro_cpu.cpp:54-74. */
static F5 hllc(const eorc_grid* gr, double rL, double vnL, double t1L, double t2L, double eL, double rR, double vnR,
               double t1R, double t2R, double eR) {
    const orc_material* m = &gr->mat;
    const double rho_vac = gr->p.rho_vac;
    if (rho_vac > 0) {
        int vL = rL < rho_vac, vR = rR < rho_vac;
        if (vL && vR) {
            F5 z = {0, 0, 0, 0, 0};
            return z;
        }
        if (vR) return vac_flux(m, rL, vnL, t1L, t2L, eL, +1);
        if (vL) return vac_flux(m, rR, vnR, t1R, t2R, eR, -1);
    }
    double pL, cL, pR, cR;
    eos_pc(m, rL, eL, &pL, &cL);
    eos_pc(m, rR, eR, &pR, &cR);
    double SL = dmin2(vnL - cL, vnR - cR), SR = dmax2(vnL + cL, vnR + cR);
    double Ss = (pR - pL + rL * vnL * (SL - vnL) - rR * vnR * (SR - vnR)) / (rL * (SL - vnL) - rR * (SR - vnR));
    double EL = rL * eL + 0.5 * rL * (vnL * vnL + t1L * t1L + t2L * t2L),
           ER = rR * eR + 0.5 * rR * (vnR * vnR + t1R * t1R + t2R * t2R);
    if (SL >= 0) return flux_of(rL, vnL, t1L, t2L, pL, EL);
    if (SR <= 0) return flux_of(rR, vnR, t1R, t2R, pR, ER);
    if (Ss >= 0) return hllc_star(rL, vnL, t1L, t2L, pL, EL, SL, Ss, flux_of(rL, vnL, t1L, t2L, pL, EL));
    return hllc_star(rR, vnR, t1R, t2R, pR, ER, SR, Ss, flux_of(rR, vnR, t1R, t2R, pR, ER));
}

/* HLLC with the face pressures given (well-balanced z-sweep), hydro_cpu.cpp:75-88. */
static F5 hllc_p(const eorc_grid* gr, double rL, double vnL, double t1L, double t2L, double eL, double pL, double rR,
                 double vnR, double t1R, double t2R, double eR, double pR) {
    const orc_material* m = &gr->mat;
    double cL = orc_sound_speed(m, rL, eL), cR = orc_sound_speed(m, rR, eR);
    if (pL < 0) pL = 0;
    if (pR < 0) pR = 0;
    double SL = dmin2(vnL - cL, vnR - cR), SR = dmax2(vnL + cL, vnR + cR);
    double Ss = (pR - pL + rL * vnL * (SL - vnL) - rR * vnR * (SR - vnR)) / (rL * (SL - vnL) - rR * (SR - vnR));
    double EL = rL * eL + 0.5 * rL * (vnL * vnL + t1L * t1L + t2L * t2L),
           ER = rR * eR + 0.5 * rR * (vnR * vnR + t1R * t1R + t2R * t2R);
    if (SL >= 0) return flux_of(rL, vnL, t1L, t2L, pL, EL);
    if (SR <= 0) return flux_of(rR, vnR, t1R, t2R, pR, ER);
    if (Ss >= 0) return hllc_star(rL, vnL, t1L, t2L, pL, EL, SL, Ss, flux_of(rL, vnL, t1L, t2L, pL, EL));
    return hllc_star(rR, vnR, t1R, t2R, pR, ER, SR, Ss, flux_of(rR, vnR, t1R, t2R, pR, ER));
}

static inline double mm(double a, double b) { /* hydro_cpu.cpp:89 */
    return (a * b <= 0) ? 0.0 : (fabs(a) < fabs(b) ? a : b);
}

static inline void prim(const eorc_grid* g, int c, double* W) { /* hydro_cpu.cpp:101 */
    W[0] = g->f[F_R][c];
    W[1] = g->f[F_MU][c] / W[0];
    W[2] = g->f[F_MV][c] / W[0];
    W[3] = g->f[F_MW][c] / W[0];
    W[4] = eint(g, c);
}

static inline int sweep_cell(const eorc_grid* g, int dir, int p, int a, int b) {
    return dir == 0 ? idx(g, p, a, b) : (dir == 1 ? idx(g, a, p, b) : idx(g, a, b, p));
}

/* One direction of the unsplit MUSCL + HLLC update, hydro_cpu.cpp:103-134
 * (the plain, not well-balanced, form). */
static void sweep(const eorc_grid* g, int dir, double* Fr, double* Fmn, double* Ft1, double* Ft2, double* FE,
                  double* Frc) {
    double** d = ((eorc_grid*)g)->d;
    const double* r = g->f[F_R];
    const double* rc = g->f[F_RC];
    const double invdx = 1.0 / g->dx;
    const int nL = dir == 0 ? g->nx : (dir == 1 ? g->ny : g->nz), nA = dir == 0 ? g->ny : g->nx,
              nB = dir == 2 ? g->ny : g->nz;
    const int in = dir == 0 ? 1 : (dir == 1 ? 2 : 3), it1 = dir == 0 ? 2 : 1, it2 = dir == 2 ? 2 : 3;
    const int axi = g->p.axisym && dir == 0;
    for (int a = 0; a < nA; a++)
        for (int b = 0; b < nB; b++) {
            for (int f = 0; f <= nL; f++) {
                int iL = imax2(0, f - 1), iR = imin2(nL - 1, f), iLL = imax2(0, f - 2), iRR = imin2(nL - 1, f + 1);
                double A[5], B[5], AA[5], BB[5], L[5], R[5];
                prim(g, sweep_cell(g, dir, iL, a, b), A);
                prim(g, sweep_cell(g, dir, iR, a, b), B);
                prim(g, sweep_cell(g, dir, iLL, a, b), AA);
                prim(g, sweep_cell(g, dir, iRR, a, b), BB);
                for (int q = 0; q < 5; q++) {
                    L[q] = A[q] + 0.5 * mm(A[q] - AA[q], B[q] - A[q]);
                    R[q] = B[q] - 0.5 * mm(B[q] - A[q], BB[q] - B[q]);
                }
                if (L[0] < 1e-9) L[0] = A[0];
                if (R[0] < 1e-9) R[0] = B[0];
                if (L[4] < 0) L[4] = A[4];
                if (R[4] < 0) R[4] = B[4];
                F5 fl;
                if (dir == 2 && g->ref_r0) { /* well-balanced: the pressure deviation from the reference */
                    int cLL = sweep_cell(g, dir, iLL, a, b), cL = sweep_cell(g, dir, iL, a, b),
                        cR = sweep_cell(g, dir, iR, a, b), cRR = sweep_cell(g, dir, iRR, a, b);
                    double dLL = eorc_pcell(g, cLL) - g->ref_p0[cLL], dL = eorc_pcell(g, cL) - g->ref_p0[cL],
                           dR = eorc_pcell(g, cR) - g->ref_p0[cR], dRR = eorc_pcell(g, cRR) - g->ref_p0[cRR];
                    double dLf = dL + 0.5 * mm(dL - dLL, dR - dL), dRf = dR - 0.5 * mm(dR - dL, dRR - dR);
                    double p0f = orc_pressure(&g->mat, 0.5 * (g->ref_r0[cL] + g->ref_r0[cR]), 0.0);
                    if (p0f < 0) p0f = 0;
                    fl = hllc_p(g, L[0], L[in], L[it1], L[it2], L[4], p0f + dLf, R[0], R[in], R[it1], R[it2], R[4],
                                p0f + dRf);
                } else {
                    fl = hllc(g, L[0], L[in], L[it1], L[it2], L[4], R[0], R[in], R[it1], R[it2], R[4]);
                }
                Fr[f] = fl.r; Fmn[f] = fl.mn; Ft1[f] = fl.mt1; Ft2[f] = fl.mt2; FE[f] = fl.E;
                int cl = sweep_cell(g, dir, iL, a, b), cr = sweep_cell(g, dir, iR, a, b);
                Frc[f] = fl.r * (fl.r >= 0.0 ? rc[cl] / r[cl] : rc[cr] / r[cr]);
            }
            for (int p = 0; p < nL; p++) {
                int c = sweep_cell(g, dir, p, a, b);
                double w0, w1, inv;
                if (axi) {
                    w0 = p * g->dx;
                    w1 = (p + 1) * g->dx;
                    inv = 1.0 / (((p + 0.5) * g->dx) * g->dx);
                } else {
                    w0 = w1 = 1.0;
                    inv = invdx;
                }
                d[D_R][c] += -(w1 * Fr[p + 1] - w0 * Fr[p]) * inv;
                d[D_E][c] += -(w1 * FE[p + 1] - w0 * FE[p]) * inv;
                d[D_RC][c] += -(w1 * Frc[p + 1] - w0 * Frc[p]) * inv;
                double dmn = -(w1 * Fmn[p + 1] - w0 * Fmn[p]) * inv, dt1 = -(w1 * Ft1[p + 1] - w0 * Ft1[p]) * inv,
                       dt2 = -(w1 * Ft2[p + 1] - w0 * Ft2[p]) * inv;
                if (axi) dmn += eorc_pcell(g, c) / ((p + 0.5) * g->dx);
                if (dir == 0) {
                    d[D_MU][c] += dmn; d[D_MV][c] += dt1; d[D_MW][c] += dt2;
                } else if (dir == 1) {
                    d[D_MV][c] += dmn; d[D_MU][c] += dt1; d[D_MW][c] += dt2;
                } else {
                    d[D_MW][c] += dmn; d[D_MU][c] += dt1; d[D_MV][c] += dt2;
                }
            }
        }
}

/* Upwind advection v . grad S of one cell, hydro_cpu.cpp:175-178. */
static inline double adv(const eorc_grid* g, const double* S, int c, int i, int j, int k, int xm, int xp, int ym,
                         int yp, int zm, int zp, double u, double v, double w) {
    double ax = u > 0 ? (S[c] - S[xm]) / ((i > 0) ? g->dx : 1e30) : (S[xp] - S[c]) / ((i < g->nx - 1) ? g->dx : 1e30);
    double ay = v > 0 ? (S[c] - S[ym]) / ((j > 0) ? g->dx : 1e30) : (S[yp] - S[c]) / ((j < g->ny - 1) ? g->dx : 1e30);
    double az = w > 0 ? (S[c] - S[zm]) / ((k > 0) ? g->dx : 1e30) : (S[zp] - S[c]) / ((k < g->nz - 1) ? g->dx : 1e30);
    return u * ax + v * ay + w * az;
}

/* Right-hand side of the conserved and material fields, hydro_cpu.cpp:98-214. */
void eorc_lop(eorc_grid* g) {
    const int n = g->n;
    double** d = g->d;
    for (int q = 0; q < ND; q++) memset(d[q], 0, sizeof(double) * (size_t)(n > 0 ? n : 1));
    int nmax = imax2(g->nx, imax2(g->ny, g->nz)) + 1;
    double* buf = (double*)malloc(sizeof(double) * 6 * (size_t)nmax);
    for (int dir = 0; dir < 3; dir++)
        sweep(g, dir, buf, buf + nmax, buf + 2 * nmax, buf + 3 * nmax, buf + 4 * nmax, buf + 5 * nmax);
    free(buf);
    const double GZ = g->p.gz, RHO_CFL = g->p.rho_cfl, ETA_AF = g->p.eta_af;
    const double* r = g->f[F_R];
    const double* mu = g->f[F_MU];
    const double* mv = g->f[F_MV];
    const double* mw = g->f[F_MW];
    if (GZ != 0.0) {
        if (!g->ref_r0) { /* hydro_cpu.cpp:137-138 (plain gravity body force) */
            for (int c = 0; c < n; c++) {
                d[D_MW][c] += -GZ * r[c];
                d[D_E][c] += -GZ * g->f[F_MW][c];
            }
        } else { /* hydro_cpu.cpp:139-143 (well-balanced source against the reference) */
            const double invdx = 1.0 / g->dx;
            const double* R0 = g->ref_r0;
            for (int i = 0; i < g->nx; i++)
                for (int j = 0; j < g->ny; j++)
                    for (int k = 0; k < g->nz; k++) {
                        int c = idx(g, i, j, k);
                        double r0t = 0.5 * (R0[c] + R0[idx(g, i, j, imin2(g->nz - 1, k + 1))]),
                               r0b = 0.5 * (R0[idx(g, i, j, imax2(0, k - 1))] + R0[c]);
                        double p0t = orc_pressure(&g->mat, r0t, 0.0);
                        if (p0t < 0) p0t = 0;
                        double p0b = orc_pressure(&g->mat, r0b, 0.0);
                        if (p0b < 0) p0b = 0;
                        d[D_MW][c] += -GZ * (r[c] - R0[c]) + (p0t - p0b) * invdx;
                        d[D_E][c] += -GZ * g->f[F_MW][c];
                    }
        }
    }
    const double G = g->mat.G;
    if (G <= 0) return;
    const double *Sxx = g->f[F_SXX], *Syy = g->f[F_SYY], *Szz = g->f[F_SZZ], *Sxy = g->f[F_SXY],
                 *Sxz = g->f[F_SXZ], *Syz = g->f[F_SYZ];
#define VX(cc) (mu[cc] / r[cc])
#define VY(cc) (mv[cc] / r[cc])
#define VZ(cc) (mw[cc] / r[cc])
#define VOIDC(cc) (RHO_CFL > 0 && r[cc] < RHO_CFL)
    for (int i = 0; i < g->nx; i++)
        for (int j = 0; j < g->ny; j++)
            for (int k = 0; k < g->nz; k++) {
                int c = idx(g, i, j, k);
                if (RHO_CFL > 0 && r[c] < RHO_CFL) continue;
                int xm = idx(g, imax2(0, i - 1), j, k), xp = idx(g, imin2(g->nx - 1, i + 1), j, k),
                    ym = idx(g, i, imax2(0, j - 1), k), yp = idx(g, i, imin2(g->ny - 1, j + 1), k),
                    zm = idx(g, i, j, imax2(0, k - 1)), zp = idx(g, i, j, imin2(g->nz - 1, k + 1));
                double hx = ((i > 0 && i < g->nx - 1) ? 2.0 : 1.0) * g->dx,
                       hy = ((j > 0 && j < g->ny - 1) ? 2.0 : 1.0) * g->dx,
                       hz = ((k > 0 && k < g->nz - 1) ? 2.0 : 1.0) * g->dx;
                /* void neighbours take the centre velocity (traction-free surface) */
#define VXW(cc) (VOIDC(cc) ? mu[c] / r[c] : mu[cc] / r[cc])
#define VYW(cc) (VOIDC(cc) ? mv[c] / r[c] : mv[cc] / r[cc])
#define VZW(cc) (VOIDC(cc) ? mw[c] / r[c] : mw[cc] / r[cc])
                double Lxx = (VXW(xp) - VXW(xm)) / hx, Lxy = (VXW(yp) - VXW(ym)) / hy, Lxz = (VXW(zp) - VXW(zm)) / hz;
                double Lyx = (VYW(xp) - VYW(xm)) / hx, Lyy = (VYW(yp) - VYW(ym)) / hy, Lyz = (VYW(zp) - VYW(zm)) / hz;
                double Lzx = (VZW(xp) - VZW(xm)) / hx, Lzy = (VZW(yp) - VZW(ym)) / hy, Lzz = (VZW(zp) - VZW(zm)) / hz;
                double rcyl = (i + 0.5) * g->dx;
                double eyy = g->p.axisym ? (VX(c) / rcyl) : Lyy;
                double exx = Lxx, ezz = Lzz, exy = 0.5 * (Lxy + Lyx), exz = 0.5 * (Lxz + Lzx), eyz = 0.5 * (Lyz + Lzy),
                       tr = (exx + eyy + ezz) / 3.0;
                double Wxy = 0.5 * (Lxy - Lyx), Wxz = 0.5 * (Lxz - Lzx), Wyz = 0.5 * (Lyz - Lzy);
                double sxx = Sxx[c], syy = Syy[c], szz = Szz[c], sxy = Sxy[c], sxz = Sxz[c], syz = Syz[c];
                double Sm[3][3] = {{sxx, sxy, sxz}, {sxy, syy, syz}, {sxz, syz, szz}},
                       Wm[3][3] = {{0, Wxy, Wxz}, {-Wxy, 0, Wyz}, {-Wxz, -Wyz, 0}}, Jm[3][3];
                for (int aa = 0; aa < 3; aa++)
                    for (int bb = 0; bb < 3; bb++) {
                        double s = 0;
                        for (int cc = 0; cc < 3; cc++) s += Sm[aa][cc] * Wm[cc][bb] - Wm[aa][cc] * Sm[cc][bb];
                        Jm[aa][bb] = s;
                    }
                double u = VX(c), v = VY(c), w = VZ(c);
#define ADV(S) adv(g, S, c, i, j, k, xm, xp, ym, yp, zm, zp, u, v, w)
                d[D_SXX][c] += 2 * G * (exx - tr) + Jm[0][0] - ADV(Sxx);
                d[D_SYY][c] += 2 * G * (eyy - tr) + Jm[1][1] - ADV(Syy);
                d[D_SZZ][c] += 2 * G * (ezz - tr) + Jm[2][2] - ADV(Szz);
                d[D_SXY][c] += 2 * G * exy + Jm[0][1] - ADV(Sxy);
                d[D_SXZ][c] += 2 * G * exz + Jm[0][2] - ADV(Sxz);
                d[D_SYZ][c] += 2 * G * eyz + Jm[1][2] - ADV(Syz);
                d[D_D][c] += -ADV(g->f[F_D]);
                d[D_VIB][c] += -ADV(g->f[F_VIB]);
#undef ADV
                double dSxx_x = (Sxx[xp] - Sxx[xm]) / hx, dSxy_y = (Sxy[yp] - Sxy[ym]) / hy,
                       dSxz_z = (Sxz[zp] - Sxz[zm]) / hz;
                double dSxy_x = (Sxy[xp] - Sxy[xm]) / hx, dSyy_y = (Syy[yp] - Syy[ym]) / hy,
                       dSyz_z = (Syz[zp] - Syz[zm]) / hz;
                double dSxz_x = (Sxz[xp] - Sxz[xm]) / hx, dSyz_y = (Syz[yp] - Syz[ym]) / hy,
                       dSzz_z = (Szz[zp] - Szz[zm]) / hz;
                d[D_MU][c] += dSxx_x + dSxy_y + dSxz_z;
                d[D_MV][c] += dSxy_x + dSyy_y + dSyz_z;
                d[D_MW][c] += dSxz_x + dSyz_y + dSzz_z;
                if (g->p.axisym) {
                    d[D_MU][c] += (Sxx[c] - Syy[c]) / rcyl;
                    d[D_MW][c] += Sxz[c] / rcyl;
                }
                if (g->f[F_AF][c] > 0 && ETA_AF > 0 && !g->p.visc_imp) { /* explicit AF viscosity */
                    double eta = g->f[F_AF][c] * ETA_AF, id2 = 1.0 / (g->dx * g->dx);
                    d[D_MU][c] += eta * (VX(xp) + VX(xm) + VX(yp) + VX(ym) + VX(zp) + VX(zm) - 6 * VX(c)) * id2;
                    d[D_MV][c] += eta * (VY(xp) + VY(xm) + VY(yp) + VY(ym) + VY(zp) + VY(zm) - 6 * VY(c)) * id2;
                    d[D_MW][c] += eta * (VZ(xp) + VZ(xm) + VZ(yp) + VZ(ym) + VZ(zp) + VZ(zm) - 6 * VZ(c)) * id2;
                    if (g->p.axisym) {
                        d[D_MU][c] += eta * (Lxx / rcyl - VX(c) / (rcyl * rcyl));
                        d[D_MW][c] += eta * (Lzx / rcyl);
                    }
                }
#define SVX(cc) (Sxx[cc] * VX(cc) + Sxy[cc] * VY(cc) + Sxz[cc] * VZ(cc))
#define SVY(cc) (Sxy[cc] * VX(cc) + Syy[cc] * VY(cc) + Syz[cc] * VZ(cc))
#define SVZ(cc) (Sxz[cc] * VX(cc) + Syz[cc] * VY(cc) + Szz[cc] * VZ(cc))
                d[D_E][c] += (SVX(xp) - SVX(xm)) / hx + (SVY(yp) - SVY(ym)) / hy + (SVZ(zp) - SVZ(zm)) / hz;
                if (g->p.axisym) d[D_E][c] += SVX(c) / rcyl;
#undef SVX
#undef SVY
#undef SVZ
#undef VXW
#undef VYW
#undef VZW
            }
#undef VX
#undef VY
#undef VZ
#undef VOIDC
}

/* Radial return to the yield surface, hydro_cpu.cpp:229-252. */
void eorc_vonmises(eorc_grid* g, int reg) {
    const eorc_params* P_ = &g->p;
    const double Y0 = g->mat.Y;
    if (Y0 <= 0 && !P_->rock) return;
    double *Sxx = g->f[F_SXX], *Syy = g->f[F_SYY], *Szz = g->f[F_SZZ], *Sxy = g->f[F_SXY], *Sxz = g->f[F_SXZ],
           *Syz = g->f[F_SYZ];
    const double* r = g->f[F_R];
    const double* D = g->f[F_D];
    const double* af = g->f[F_AF];
    double* vib = g->f[F_VIB];
    for (int c = 0; c < g->n; c++) {
        double Y;
        if (P_->rock) {
            double P = dmax2(eorc_pcell(g, c), 0.0);
            double Peff = P;
            if (P_->af_prel && vib[c] > 0) {
                double p2, cs2;
                eos_pc(&g->mat, r[c], eint(g, c), &p2, &cs2);
                Peff = dmax2(P - r[c] * cs2 * vib[c], 0.0);
            }
            double Yi = P_->y_i0 + P_->mu_i * Peff / (1.0 + P_->mu_i * Peff / dmax2(P_->y_m - P_->y_i0, 1.0));
            double Yd = dmin2(P_->y_d0 + P_->mu_d * Peff, P_->y_m);
            double Yb = (1.0 - D[c]) * Yi + D[c] * Yd;
            Y = P_->af_prel ? Yb : Yb * (1.0 - af[c]);
            if (P_->y_bingham > 0 && af[c] > 1e-3) {
                double Yf = dmin2(P_->y_bingham, Yb);
                if (Y < Yf) Y = Yf;
            }
        } else {
            Y = (1.0 - D[c]) * (1.0 - af[c]) * Y0;
        }
        double sxx = Sxx[c], syy = Syy[c], szz = Szz[c], sxy = Sxy[c], sxz = Sxz[c], syz = Syz[c];
        double J2 = 0.5 * (sxx * sxx + syy * syy + szz * szz) + sxy * sxy + sxz * sxz + syz * syz;
        double vm = sqrt(3.0 * J2);
        if (vm > Y) {
            double f = (vm > 0 ? Y / vm : 0.0);
            Sxx[c] *= f; Syy[c] *= f; Szz[c] *= f; Sxy[c] *= f; Sxz[c] *= f; Syz[c] *= f;
            if (P_->af_reg && reg && g->mat.G > 0 && (P_->rho_cfl <= 0 || r[c] > P_->rho_cfl)) {
                double dW = (vm * vm - Y * Y) / (6.0 * g->mat.G);
                vib[c] = sqrt(vib[c] * vib[c] + 2.0 * P_->c_reg * dW / r[c]);
                g->f[F_E][c] -= P_->c_reg * dW;
            }
        }
    }
}

/* Tensile damage growth from the weakest-flaw activation strain,
 * hydro_cpu.cpp:253-258. */
void eorc_grow_damage(eorc_grid* g, double dt) {
    const double Em = g->mat.Emod, wk = g->mat.wk, wm = g->mat.wm;
    if (Em <= 0 || wk <= 0) return;
    const double dx = g->dx, eps_act = pow(1.0 / (wk * dx * dx * dx), 1.0 / wm);
    double* D = g->f[F_D];
    const double* r = g->f[F_R];
    for (int c = 0; c < g->n; c++) {
        if (D[c] >= 1.0) continue;
        double P = eorc_pcell(g, c);
        double sigmax = dmax2(-P + g->f[F_SXX][c], dmax2(-P + g->f[F_SYY][c], -P + g->f[F_SZZ][c]));
        if (sigmax > 0.0 && sigmax / Em > eps_act) {
            double cg = 0.4 * sqrt(Em / dmax2(r[c], 1e-30)), Rs = 0.5 * dx;
            double d13 = pow(D[c], 1.0 / 3.0) + (cg / Rs) * dt;
            D[c] = dmin2(1.0, d13 * d13 * d13);
        }
    }
}

/* Shock-activated acoustic fluidization, hydro_cpu.cpp:390-410. */
void eorc_update_af(eorc_grid* g, double dt) {
    const eorc_params* P_ = &g->p;
    if (P_->c_act <= 0 || P_->tdec <= 0) return;
    const double dec = exp(-dt / P_->tdec);
    double *r = g->f[F_R], *vib = g->f[F_VIB], *Pmax = g->f[F_PMAX], *af = g->f[F_AF];
    for (int c = 0; c < g->n; c++) {
        double P = eorc_pcell(g, c);
        double cs = orc_sound_speed(&g->mat, r[c], eint(g, c));
        if (P > Pmax[c]) {
            double dP = P - Pmax[c];
            Pmax[c] = P;
            if (dP > P_->p_act) {
                double sp = P_->af_seeddp
                                ? dP / (dmax2(r[c], 1e-30) * dmax2(cs, 1e-30))
                                : sqrt(g->f[F_MU][c] * g->f[F_MU][c] + g->f[F_MV][c] * g->f[F_MV][c] +
                                       g->f[F_MW][c] * g->f[F_MW][c]) / dmax2(r[c], 1e-30);
                vib[c] = dmax2(vib[c], P_->c_act * sp);
            }
        }
        double v0 = vib[c];
        vib[c] *= dec;
        double pov = dmax2(P, P_->p_coh);
        if (P_->af_reg) {
            if (r[c] > dmax2(P_->rho_cfl, 1e-12)) g->f[F_E][c] += 0.5 * r[c] * (v0 * v0 - vib[c] * vib[c]);
            double vcap = P_->af_sat * pov / (dmax2(r[c], 1e-30) * dmax2(cs, 1e-30));
            if (vib[c] > vcap) vib[c] = vcap;
        }
        double pvib = r[c] * cs * vib[c];
        af[c] = pvib / (pvib + pov);
    }
}

/* Largest signal speed |v| + sqrt(c^2 + 4G/(3 rho)), hydro_cpu.cpp:378-380. */
double eorc_maxspeed(const eorc_grid* g) {
    double s = 1e-30;
    const double G = g->mat.G;
    const double* r = g->f[F_R];
    for (int c = 0; c < g->n; c++) {
        if (r[c] < g->p.rho_cfl) continue;
        double p, cs;
        eos_pc(&g->mat, r[c], eint(g, c), &p, &cs);
        double cel = sqrt(cs * cs + (G > 0 ? (4.0 / 3.0) * G / r[c] : 0.0));
        double v = sqrt(g->f[F_MU][c] * g->f[F_MU][c] + g->f[F_MV][c] * g->f[F_MV][c] +
                        g->f[F_MW][c] * g->f[F_MW][c]) / r[c];
        s = dmax2(s, v + cel);
    }
    return s;
}

/* Near-void cells lose their momentum and, with a reference state, are reset
 * to the reference density (or the ambient VOID_AMB) with no energy, stress or
 * tracer; with VOID_CONS the excess over the ambient density first moves to
 * the densest face neighbour above RHO_CFL (volume-weighted in cylindrical
 * geometry), cell by cell in index order, hydro_cpu.cpp:272-290. */
static void void_cells(eorc_grid* g) {
    if (g->p.rho_cfl <= 0) return;
    double* r = g->f[F_R];
    for (int c = 0; c < g->n; c++)
        if (r[c] < g->p.rho_cfl) {
            g->f[F_MU][c] = g->f[F_MV][c] = g->f[F_MW][c] = 0;
            if (g->ref_r0) {
                if (g->p.void_cons) {
                    double amb = (g->p.void_amb > 0 ? g->p.void_amb : 0.27), exc = r[c] - amb;
                    if (exc > 0) {
                        int i = c / (g->ny * g->nz), j = (c / g->nz) % g->ny, k = c % g->nz, nb = -1;
                        double rbest = g->p.rho_cfl;
                        int ci[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j, k - 1}, {i, j, k + 1}, {i, j - 1, k}, {i, j + 1, k}};
                        int ncand = g->ny > 1 ? 6 : 4;
                        for (int q = 0; q < ncand; q++) {
                            int ii = ci[q][0], jj = ci[q][1], kk = ci[q][2];
                            if (ii < 0 || ii >= g->nx || jj < 0 || jj >= g->ny || kk < 0 || kk >= g->nz) continue;
                            int cc = idx(g, ii, jj, kk);
                            if (r[cc] > rbest) {
                                rbest = r[cc];
                                nb = cc;
                            }
                        }
                        if (nb >= 0) {
                            double w = 1.0;
                            if (g->p.axisym) {
                                int inb = nb / (g->ny * g->nz);
                                w = (i + 0.5) / (inb + 0.5);
                            }
                            r[nb] += exc * w;
                        }
                    }
                }
                r[c] = (g->p.void_amb > 0 ? g->p.void_amb : g->ref_r0[c]);
                g->f[F_E][c] = 0;
                g->f[F_SXX][c] = g->f[F_SYY][c] = g->f[F_SZZ][c] = g->f[F_SXY][c] = g->f[F_SXZ][c] = g->f[F_SYZ][c] = 0;
                g->f[F_RC][c] = 0;
            }
        }
}

void eorc_set_ref(eorc_grid* g) { /* hydro_cpu.cpp:259-261 */
    if (!g->ref_r0) g->ref_r0 = (double*)calloc((size_t)(g->n > 0 ? g->n : 1), sizeof(double));
    if (!g->ref_p0) g->ref_p0 = (double*)calloc((size_t)(g->n > 0 ? g->n : 1), sizeof(double));
    for (int c = 0; c < g->n; c++) {
        g->ref_r0[c] = g->f[F_R][c];
        g->ref_p0[c] = eorc_pcell(g, c);
    }
}

void eorc_clear_ref(eorc_grid* g) {
    free(g->ref_r0);
    free(g->ref_p0);
    g->ref_r0 = g->ref_p0 = NULL;
}

/* ---- implicit fluidization viscosity, hydro_cpu.cpp:286-377 ----
 * Backward Euler for d(rho v)/dt = div(eta grad v) with eta = af * ETA_AF in
 * fluidized cells (af > 1e-3, rho above RHO_CFL): a finite-volume operator
 * with face-harmonic eta (a face with a non-fluidized side carries no flux),
 * face-area weights and the -v/r^2 diagonal of the r and hoop components in
 * cylindrical geometry; each component solved by Jacobi-preconditioned
 * conjugate gradients to a relative residual of 1e-8 (at most 800
 * iterations); the kinetic energy removed comes back as heat, spread in
 * proportion to each face's dissipation and scaled so that total energy is
 * conserved. */
typedef struct {
    int nx, ny, nz, n, axisym;
    const double *cfx, *cfy, *cfz, *dsum, *dax;
} visc_op;

static double visc_diag(const visc_op* A, int c, int wdax) { return A->dsum[c] + (wdax ? A->dax[c] : 0.0); }

/* y = A x (hydro_cpu.cpp:321-331). */
static void visc_apply(const visc_op* A, const double* x, double* y, int wdax) {
    const int nx = A->nx, ny = A->ny, nz = A->nz;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int c = (i * ny + j) * nz + k;
                double s = visc_diag(A, c, wdax) * x[c];
                if (i < nx - 1) s -= A->cfx[c] * x[c + ny * nz];
                if (i > 0) s -= A->cfx[c - ny * nz] * x[c - ny * nz];
                if (ny > 1) {
                    if (j < ny - 1) s -= A->cfy[c] * x[c + nz];
                    if (j > 0) s -= A->cfy[c - nz] * x[c - nz];
                }
                if (k < nz - 1) s -= A->cfz[c] * x[c + 1];
                if (k > 0) s -= A->cfz[c - 1] * x[c - 1];
                y[c] = s;
            }
}

/* Jacobi-preconditioned CG from the initial guess in x (hydro_cpu.cpp:332-351);
 * every sum runs over the cells in index order. */
static void visc_cg(const visc_op* A, double* x, const double* b, int wdax, double* rr, double* zz, double* pp,
                    double* qq, long* iters) {
    const int n = A->n;
    double bn = 0;
    for (int c = 0; c < n; c++) bn += b[c] * b[c];
    if (bn <= 0) {
        for (int c = 0; c < n; c++) x[c] = 0;
        return;
    }
    visc_apply(A, x, qq, wdax);
    double rn = 0;
    for (int c = 0; c < n; c++) {
        rr[c] = b[c] - qq[c];
        rn += rr[c] * rr[c];
    }
    const double tol2 = 1e-16 * bn;
    double rz = 0;
    for (int c = 0; c < n; c++) {
        zz[c] = rr[c] / visc_diag(A, c, wdax);
        pp[c] = zz[c];
        rz += rr[c] * zz[c];
    }
    for (int it = 0; it < 800 && rn > tol2; it++) {
        visc_apply(A, pp, qq, wdax);
        double pq = 0;
        for (int c = 0; c < n; c++) pq += pp[c] * qq[c];
        if (pq <= 0) break;
        const double al = rz / pq;
        rn = 0;
        for (int c = 0; c < n; c++) {
            x[c] += al * pp[c];
            rr[c] -= al * qq[c];
            rn += rr[c] * rr[c];
        }
        (*iters)++;
        if (rn <= tol2) break;
        double rz2 = 0;
        for (int c = 0; c < n; c++) {
            zz[c] = rr[c] / visc_diag(A, c, wdax);
            rz2 += rr[c] * zz[c];
        }
        const double be = rz2 / rz;
        rz = rz2;
        for (int c = 0; c < n; c++) pp[c] = zz[c] + be * pp[c];
    }
}

static double harmonic(double a, double b) { return (a > 0 && b > 0) ? 2.0 * a * b / (a + b) : 0.0; }

void eorc_implicit_visc(eorc_grid* g, double dt) {
    if (!g->p.visc_imp || g->p.eta_af <= 0) return;
    const int nx = g->nx, ny = g->ny, nz = g->nz, n = g->n, ax = g->p.axisym;
    const double dx = g->dx, rmin = dmax2(g->p.rho_cfl, 1e-12);
    double** f = g->f;
    double* eta = (double*)calloc((size_t)n, sizeof(double));
    int any = 0;
    for (int c = 0; c < n; c++)
        if (f[F_R][c] > rmin && f[F_AF][c] > 1e-3) {
            eta[c] = f[F_AF][c] * g->p.eta_af;
            any = 1;
        }
    if (!any) {
        free(eta);
        return;
    }
    enum { VC, CFX, CFY, CFZ, DSUM, DAX, RR, ZZ, PP, QQ, U1, V1, W1, BB, HR, NBUF };
    double* w[NBUF];
    for (int q = 0; q < NBUF; q++) w[q] = (double*)calloc((size_t)n, sizeof(double));
    double *Vc = w[VC], *cfx = w[CFX], *cfy = w[CFY], *cfz = w[CFZ], *dsum = w[DSUM], *dax = w[DAX];
    const int sx = ny * nz, sy = nz;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int c = idx(g, i, j, k);
                const double rc = (i + 0.5) * dx, wV = ax ? rc : dx;
                Vc[c] = wV * dx * dx;
                dsum[c] = f[F_R][c] * Vc[c];
                if (i < nx - 1) cfx[c] = dt * (ax ? (i + 1) * dx : dx) * harmonic(eta[c], eta[c + sx]);
                if (ny > 1 && j < ny - 1) cfy[c] = dt * dx * harmonic(eta[c], eta[c + sy]);
                if (k < nz - 1) cfz[c] = dt * wV * harmonic(eta[c], eta[c + 1]);
                if (ax) dax[c] = dt * eta[c] * Vc[c] / (rc * rc);
            }
    /* each face coefficient enters the diagonal of both its cells, in the
     * reference's scatter order (hydro_cpu.cpp:315-319) */
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int c = idx(g, i, j, k);
                if (i < nx - 1) { dsum[c] += cfx[c]; dsum[c + sx] += cfx[c]; }
                if (ny > 1 && j < ny - 1) { dsum[c] += cfy[c]; dsum[c + sy] += cfy[c]; }
                if (k < nz - 1) { dsum[c] += cfz[c]; dsum[c + 1] += cfz[c]; }
            }
    const visc_op A = {nx, ny, nz, n, ax, cfx, cfy, cfz, dsum, dax};
    const int mom[3] = {F_MU, F_MV, F_MW}, xq[3] = {U1, V1, W1};
    for (int m = 0; m < 3; m++) { /* u and the hoop component carry -v/r^2; w does not */
        double *x = w[xq[m]], *b = w[BB];
        for (int c = 0; c < n; c++) {
            x[c] = f[mom[m]][c] / f[F_R][c];
            b[c] = Vc[c] * f[mom[m]][c];
        }
        visc_cg(&A, x, b, m < 2 ? ax : 0, w[RR], w[ZZ], w[PP], w[QQ], &g->visc_iters);
    }
    const double *u1 = w[U1], *v1 = w[V1], *w1 = w[W1];
    double* hr = w[HR];
    double totold = 0, totnew = 0, htot = 0;
#define FACE_HEAT(cn, cf)                                                              \
    do {                                                                               \
        const double du = u1[c] - u1[cn], dv = v1[c] - v1[cn], dw = w1[c] - w1[cn];    \
        const double h = (cf) * (du * du + dv * dv + dw * dw);                         \
        hr[c] += 0.5 * h;                                                              \
        hr[cn] += 0.5 * h;                                                             \
        htot += h;                                                                     \
    } while (0)
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const int c = idx(g, i, j, k);
                const double r = f[F_R][c];
                const double keo = 0.5 * (f[F_MU][c] * f[F_MU][c] + f[F_MV][c] * f[F_MV][c] + f[F_MW][c] * f[F_MW][c]) / r;
                const double ken = 0.5 * r * (u1[c] * u1[c] + v1[c] * v1[c] + w1[c] * w1[c]);
                totold += keo * Vc[c];
                totnew += ken * Vc[c];
                if (i < nx - 1 && cfx[c] > 0) FACE_HEAT(c + sx, cfx[c]);
                if (ny > 1 && j < ny - 1 && cfy[c] > 0) FACE_HEAT(c + sy, cfy[c]);
                if (k < nz - 1 && cfz[c] > 0) FACE_HEAT(c + 1, cfz[c]);
                if (ax && dax[c] > 0) {
                    const double h = dax[c] * (u1[c] * u1[c] + v1[c] * v1[c]);
                    hr[c] += h;
                    htot += h;
                }
            }
#undef FACE_HEAT
    const double loss = totold - totnew, sc = (loss > 0 && htot > 0) ? loss / htot : 0.0;
    for (int c = 0; c < n; c++) {
        const double r = f[F_R][c];
        const double keo = 0.5 * (f[F_MU][c] * f[F_MU][c] + f[F_MV][c] * f[F_MV][c] + f[F_MW][c] * f[F_MW][c]) / r;
        f[F_MU][c] = r * u1[c];
        f[F_MV][c] = r * v1[c];
        f[F_MW][c] = r * w1[c];
        const double ken = 0.5 * (f[F_MU][c] * f[F_MU][c] + f[F_MV][c] * f[F_MV][c] + f[F_MW][c] * f[F_MW][c]) / r;
        double q = sc * hr[c] / Vc[c];
        if (g->p.af_reg && q > 0) { /* C_REG of the dissipation regenerates vibrations */
            f[F_VIB][c] = sqrt(f[F_VIB][c] * f[F_VIB][c] + 2.0 * g->p.c_reg * q / r);
            q *= (1.0 - g->p.c_reg);
        }
        f[F_E][c] += (ken - keo) + q;
    }
    for (int q = 0; q < NBUF; q++) free(w[q]);
    free(eta);
}

long eorc_visc_iters(const eorc_grid* g) { return g->visc_iters; }

static const int RK_FIELDS[ND] = {F_R, F_MU, F_MV, F_MW, F_E, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ, F_D, F_RC, F_VIB};

/* Two-stage Runge-Kutta step, hydro_cpu.cpp:411-425. */
void eorc_step_rk2(eorc_grid* g, double dt) {
    const int n = g->n;
    eorc_update_af(g, dt);
    eorc_grid* g1 = eorc_create(g->nx, g->ny, g->nz, g->dx);
    g1->mat = g->mat;
    g1->p = g->p;
    g1->ref_r0 = g->ref_r0; /* shared, not owned */
    g1->ref_p0 = g->ref_p0;
    for (int q = 0; q < NF; q++) memcpy(g1->f[q], g->f[q], sizeof(double) * (size_t)n);
    eorc_lop(g);
    for (int q = 0; q < ND; q++) {
        const double* x = g->f[RK_FIELDS[q]];
        const double* dq = g->d[q];
        double* y = g1->f[RK_FIELDS[q]];
        for (int c = 0; c < n; c++) y[c] = x[c] + dt * dq[c];
    }
    void_cells(g1);
    eorc_vonmises(g1, 0);
    eorc_lop(g1);
    for (int q = 0; q < ND; q++) {
        double* x = g->f[RK_FIELDS[q]];
        const double* y = g1->f[RK_FIELDS[q]];
        const double* dq = g1->d[q];
        for (int c = 0; c < n; c++) x[c] = 0.5 * (x[c] + y[c] + dt * dq[c]);
    }
    for (int q = 0; q < ND; q++) memcpy(g->d[q], g1->d[q], sizeof(double) * (size_t)n);
    g1->ref_r0 = g1->ref_p0 = NULL;
    eorc_destroy(g1);
    eorc_implicit_visc(g, dt);
    eorc_grow_damage(g, dt);
    eorc_vonmises(g, 1);
    if (g->p.damp < 1.0)
        for (int c = 0; c < n; c++) {
            g->f[F_MU][c] *= g->p.damp;
            g->f[F_MV][c] *= g->p.damp;
            g->f[F_MW][c] *= g->p.damp;
        }
    void_cells(g);
}

int eorc_run(eorc_grid* g, double cfl, double t_end, int max_steps, double* t_out) {
    double t = 0;
    int s = 0;
    while (t < t_end && (max_steps < 0 || s < max_steps)) {
        double dt = cfl * g->dx / eorc_maxspeed(g);
        if (t + dt > t_end) dt = t_end - t;
        eorc_step_rk2(g, dt);
        t += dt;
        s++;
    }
    if (t_out) *t_out = t;
    return s;
}
