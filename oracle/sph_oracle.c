/*
 * sph_oracle.c -- CPU oracle for the SPH step loop (TEST INFRASTRUCTURE ONLY).
 *
 * Restates hydrocodes/sph/sph.hpp and hydrocodes/common/eos.hpp in plain C with
 * structure-of-arrays storage.  Every expression keeps the reference's
 * floating-point operation order (build with -ffp-contract=off) so the result
 * is bit-identical to the reference on the same inputs; citations are
 * reference-relative file:line.  Only tests, smoke() and bench.py's CPU
 * baseline use this file.
 */
#define _GNU_SOURCE
#include "sph_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define ORC_PI 3.14159265358979323846

/* std::max / std::min semantics: max(a,b) = (a<b)?b:a, min(a,b) = (b<a)?b:a */
static inline double dmax(double a, double b) { return (a < b) ? b : a; }
static inline double dmin(double a, double b) { return (b < a) ? b : a; }

/* ------------------------------------------------------------------------ */
/* EOS: hydrocodes/common/eos.hpp                                            */
/* ------------------------------------------------------------------------ */

orc_material orc_mat_ideal(double gamma) { /* eos.hpp:29 */
    orc_material m;
    memset(&m, 0, sizeof m);
    m.type = ORC_IDEAL;
    m.gamma = gamma;
    return m;
}

orc_material orc_mat_tillotson(double rho0, double A, double B, double a, double b,
                               double al, double be, double u0, double uiv, double ucv,
                               double G, double Y, double wm, double wk) { /* eos.hpp:30-39 */
    orc_material m;
    memset(&m, 0, sizeof m);
    m.type = ORC_TILLOTSON;
    m.gamma = 1.4;
    m.rho0 = rho0; m.A = A; m.B = B; m.a = a; m.b = b;
    m.alpha = al; m.beta = be; m.u0 = u0; m.uiv = uiv; m.ucv = ucv;
    m.G = G; m.Y = Y; m.wm = wm; m.wk = wk;
    m.Emod = (G > 0 ? 9.0 * A * G / (3.0 * A + G) : 0.0);
    return m;
}

/* standard sets, eos.hpp:42-50 */
orc_material orc_mat_iron(void) {
    return orc_mat_tillotson(7800, 1.28e11, 1.05e11, 0.5, 1.5, 5, 5, 9.5e6, 2.4e6, 8.67e6,
                             7.75e10, 1.0e9, 0, 0);
}
orc_material orc_mat_basalt(void) {
    return orc_mat_tillotson(2700, 2.67e10, 2.67e10, 0.5, 1.5, 5, 5, 4.87e8, 4.72e6, 1.82e7,
                             2.27e10, 3.5e8, 16.0, 1.0e61);
}
orc_material orc_mat_water(void) {
    return orc_mat_tillotson(998, 2.2e9, 9.94e9, 0.7, 0.15, 10, 5, 7.0e6, 4.19e5, 2.69e6,
                             0.0, 0.0, 0, 0);
}
orc_material orc_mat_aluminum(void) {
    return orc_mat_tillotson(2700, 7.52e10, 6.5e10, 0.5, 1.63, 5, 5, 5.0e6, 3.0e6, 1.39e7,
                             0.0, 0.0, 0, 0);
}

/* Tillotson pressure, eos.hpp:52-63 */
static double till(const orc_material* m, double rho, double u) {
    if (rho <= 0) return 0.0;
    double eta = rho / m->rho0, mu = eta - 1.0;
    double w0 = u / (m->u0 * eta * eta) + 1.0;
    double Pc = (m->a + m->b / w0) * rho * u + m->A * mu + m->B * mu * mu;
    if (rho >= m->rho0 || u <= m->uiv) return Pc;
    double z = m->rho0 / rho - 1.0;
    double Pe = m->a * rho * u +
                (m->b * rho * u / w0 + m->A * mu * exp(-m->beta * z)) * exp(-m->alpha * z * z);
    if (u >= m->ucv) return Pe;
    return ((u - m->uiv) * Pe + (m->ucv - u) * Pc) / (m->ucv - m->uiv);
}

double orc_pressure(const orc_material* m, double rho, double u) { /* eos.hpp:65-68 */
    if (m->type == ORC_IDEAL) return (m->gamma - 1.0) * rho * u;
    return till(m, rho, u);
}

/* condensed-branch value and analytic derivatives, eos.hpp:72-79 */
static void cond_d(const orc_material* m, double rho, double u, double* P, double* dPdr,
                   double* dPdu) {
    double eta = rho / m->rho0, mu = eta - 1.0;
    double w = 1.0 + u / (m->u0 * eta * eta), aob = m->a + m->b / w;
    *P = aob * rho * u + m->A * mu + m->B * mu * mu;
    *dPdu = aob * rho - m->b * rho * u / (w * w * m->u0 * eta * eta);
    double dwdr = -2.0 * u / (m->u0 * eta * eta * eta * m->rho0);
    *dPdr = aob * u + rho * u * (-m->b / (w * w)) * dwdr + m->A / m->rho0 +
            2.0 * m->B * mu / m->rho0;
}

/* expanded-branch value and analytic derivatives, eos.hpp:80-94 */
static void expd_d(const orc_material* m, double rho, double u, double* P, double* dPdr,
                   double* dPdu) {
    double eta = rho / m->rho0, mu = eta - 1.0;
    double w = 1.0 + u / (m->u0 * eta * eta);
    double z = m->rho0 / rho - 1.0, dzdr = -m->rho0 / (rho * rho);
    double E1 = exp(-m->alpha * z * z), E2 = exp(-m->beta * z);
    double G = m->b * rho * u / w + m->A * mu * E2;
    *P = m->a * rho * u + G * E1;
    double dwdr = -2.0 * u / (m->u0 * eta * eta * eta * m->rho0);
    double dGu = m->b * rho / w - m->b * rho * u / (w * w * m->u0 * eta * eta);
    *dPdu = m->a * rho + dGu * E1;
    double dbruw_dr = m->b * u / w + m->b * rho * u * (-1.0 / (w * w)) * dwdr;
    double dGr = dbruw_dr + m->A * E2 / m->rho0 + m->A * mu * (E2 * (-m->beta) * dzdr);
    double dE1dr = E1 * (-m->alpha * 2.0 * z) * dzdr;
    *dPdr = m->a * u + dGr * E1 + G * dE1dr;
}

double orc_sound_speed(const orc_material* m, double rho, double u) { /* eos.hpp:95-113 */
    if (m->type == ORC_IDEAL) {
        double P = (m->gamma - 1.0) * rho * u;
        return sqrt(dmax(m->gamma * P / dmax(rho, 1e-30), 1e-12));
    }
    if (rho <= 0) return 1e-3;
    double P, dPdr, dPdu;
    if (rho >= m->rho0 || u <= m->uiv) {
        cond_d(m, rho, u, &P, &dPdr, &dPdu);
    } else if (u >= m->ucv) {
        expd_d(m, rho, u, &P, &dPdr, &dPdu);
    } else {
        double Pc, dPcr, dPcu, Pe, dPer, dPeu;
        cond_d(m, rho, u, &Pc, &dPcr, &dPcu);
        expd_d(m, rho, u, &Pe, &dPer, &dPeu);
        double inv = 1.0 / (m->ucv - m->uiv);
        P = ((u - m->uiv) * Pe + (m->ucv - u) * Pc) * inv;
        dPdu = ((Pe + (u - m->uiv) * dPeu) + (-Pc + (m->ucv - u) * dPcu)) * inv;
        dPdr = ((u - m->uiv) * dPer + (m->ucv - u) * dPcr) * inv;
    }
    return sqrt(dmax(dPdr + P / (rho * rho) * dPdu, 1e-6));
}

void orc_eos_batch(const orc_material* m, int n, const double* rho, const double* u,
                   double* P, double* cs) {
    for (int i = 0; i < n; i++) {
        if (P) P[i] = orc_pressure(m, rho[i], u[i]);
        if (cs) cs[i] = orc_sound_speed(m, rho[i], u[i]);
    }
}

/* ------------------------------------------------------------------------ */
/* kernel + tensor helpers: hydrocodes/sph/sph.hpp:17-54                     */
/* ------------------------------------------------------------------------ */

double orc_kW(double r, double h) { /* sph.hpp:17-22 */
    double q = r / h, s = 1.0 / (ORC_PI * h * h * h);
    if (q < 1.0) return s * (1.0 - 1.5 * q * q + 0.75 * q * q * q);
    if (q < 2.0) {
        double t = 2.0 - q;
        return s * 0.25 * t * t * t;
    }
    return 0.0;
}

double orc_kdWdr(double r, double h) { /* sph.hpp:23-28 */
    double q = r / h, s = 1.0 / (ORC_PI * h * h * h);
    if (q < 1.0) return s * (-3.0 * q + 2.25 * q * q) / h;
    if (q < 2.0) {
        double t = 2.0 - q;
        return s * (-0.75 * t * t) / h;
    }
    return 0.0;
}

/* largest eigenvalue of a symmetric 3x3 by Smith's (1961) trigonometric
 * method, sph.hpp:41-54.  s = {xx, yy, zz, xy, xz, yz}. */
double orc_eig_max(const double s[6]) {
    double xx = s[0], yy = s[1], zz = s[2], xy = s[3], xz = s[4], yz = s[5];
    double p1 = xy * xy + xz * xz + yz * yz;
    double q = (xx + yy + zz) / 3.0;
    if (p1 < 1e-30) return dmax(dmax(xx, yy), zz);
    double p2 = (xx - q) * (xx - q) + (yy - q) * (yy - q) + (zz - q) * (zz - q) + 2 * p1;
    double p = sqrt(p2 / 6.0);
    double a = (xx - q) / p, b = (yy - q) / p, c = (zz - q) / p;
    double d = xy / p, e = xz / p, f = yz / p;
    double r = (a * (b * c - f * f) - d * (d * c - f * e) + e * (d * f - b * e)) / 2.0;
    r = dmax(-1.0, dmin(1.0, r));
    double phi = acos(r) / 3.0;
    return q + 2.0 * p * cos(phi);
}

/* ------------------------------------------------------------------------ */
/* parallel runtime: sph.hpp:56-70 (static chunks, serial below 2000)        */
/* ------------------------------------------------------------------------ */

typedef void (*orc_body)(void* ctx, int lo, int hi);
typedef struct { orc_body f; void* ctx; int lo, hi; } orc_chunk;

static void* orc_chunk_run(void* p) {
    orc_chunk* c = (orc_chunk*)p;
    c->f(c->ctx, c->lo, c->hi);
    return NULL;
}

static int orc_default_threads(void) {
    long nt = sysconf(_SC_NPROCESSORS_ONLN);
    if (nt <= 0) nt = 1;
    if (nt > 16) nt = 16;
    return (int)nt;
}

static void orc_parallel_for(int nthreads, int n, orc_body f, void* ctx) {
    int nt = nthreads;
    if (n < 2000 || nt <= 1) {
        f(ctx, 0, n);
        return;
    }
    int chunk = (n + nt - 1) / nt;
    pthread_t th[256];
    orc_chunk ck[256];
    int used = 0;
    for (int t = 0; t < nt && t < 256; t++) {
        int lo = t * chunk, hi = lo + chunk < n ? lo + chunk : n;
        if (lo >= hi) break;
        ck[used].f = f; ck[used].ctx = ctx; ck[used].lo = lo; ck[used].hi = hi;
        if (pthread_create(&th[used], NULL, orc_chunk_run, &ck[used]) != 0) {
            f(ctx, lo, hi); /* could not spawn: run inline */
            continue;
        }
        used++;
    }
    for (int t = 0; t < used; t++) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* particle system                                                           */
/* ------------------------------------------------------------------------ */

enum {
    F_X, F_Y, F_Z, F_VX, F_VY, F_VZ, F_AX, F_AY, F_AZ,
    F_MASS, F_RHO, F_U, F_DUDT, F_P, F_CS, F_CSIG, F_HH, F_EPSW,
    F_D, F_EPSACT, F_SIGMAX, F_PF, F_RART, F_DSCALE,
    F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ,
    F_DSXX, F_DSYY, F_DSZZ, F_DSXY, F_DSXZ, F_DSYZ,
    F_H0, F_COUNT
};

static const char* kFieldNames[F_COUNT] = {
    "x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az",
    "mass", "rho", "u", "dudt", "P", "cs", "csig", "hh", "eps_work",
    "D", "eps_act", "sigmax", "Pf", "Rart", "dscale",
    "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz",
    "dSxx", "dSyy", "dSzz", "dSxy", "dSxz", "dSyz", "h0"};

struct orc_sys {
    int n, cap;
    double* f[F_COUNT];
    int32_t* mat;
    uint8_t* fixed;
    int use_h0;
    orc_material* mats;
    int nmat, capmat;
    int cur_mat;
    orc_params prm;
    double dlo[3], dhi[3];
    int per[3];
    int nthreads;
    /* cell list (CSR, ids ascending within a cell) */
    double h_max;
    int32_t nc[3];
    double cw[3];
    int64_t ncells;
    int32_t* cell_start; /* ncells + 1 */
    int32_t* cell_ids;   /* n */
    int32_t* cell_of;    /* n */
    /* multi-flaw extension: CSR of activation strains per particle */
    int64_t* flaw_start; /* n + 1 or NULL */
    double* flaw_eps;
    int64_t nflaws;
};

orc_sys* orc_create(void) {
    orc_sys* s = (orc_sys*)calloc(1, sizeof(orc_sys));
    /* sph.hpp:86-92 defaults */
    s->prm.eta = 1.3;
    s->prm.h_init = 0.01;
    s->prm.alpha = 1.0;
    s->prm.beta = 2.0;
    s->prm.eps = 0.01;
    s->prm.alpha_u = 0.0;
    s->prm.cfl = 0.2;
    s->prm.eps_as = 0.0;
    s->prm.as_n = 4;
    s->prm.damage_on = 0;
    s->prm.flaw_model = ORC_FLAWS_SINGLE;
    s->h_max = 0.01;
    s->nc[0] = s->nc[1] = s->nc[2] = 1;
    s->cw[0] = s->cw[1] = s->cw[2] = 1;
    s->nthreads = orc_default_threads();
    return s;
}

void orc_destroy(orc_sys* s) {
    if (!s) return;
    for (int k = 0; k < F_COUNT; k++) free(s->f[k]);
    free(s->mat);
    free(s->fixed);
    free(s->mats);
    free(s->cell_start);
    free(s->cell_ids);
    free(s->cell_of);
    free(s->flaw_start);
    free(s->flaw_eps);
    free(s);
}

void orc_set_threads(orc_sys* s, int nt) { s->nthreads = nt > 0 ? nt : orc_default_threads(); }
int orc_get_threads(const orc_sys* s) { return s->nthreads; }
void orc_get_params(const orc_sys* s, orc_params* p) { *p = s->prm; }
void orc_set_params(orc_sys* s, const orc_params* p) { s->prm = *p; }

int orc_add_material(orc_sys* s, const orc_material* m) {
    if (s->nmat == s->capmat) {
        s->capmat = s->capmat ? 2 * s->capmat : 8;
        s->mats = (orc_material*)realloc(s->mats, sizeof(orc_material) * s->capmat);
    }
    s->mats[s->nmat] = *m;
    return s->nmat++;
}

void orc_set_cur_mat(orc_sys* s, int m) { s->cur_mat = m; }

void orc_set_domain(orc_sys* s, double xl, double xh, int px, double yl, double yh, int py,
                    double zl, double zh, int pz) { /* sph.hpp:96-101 */
    s->dlo[0] = xl; s->dhi[0] = xh; s->per[0] = px != 0;
    s->dlo[1] = yl; s->dhi[1] = yh; s->per[1] = py != 0;
    s->dlo[2] = zl; s->dhi[2] = zh; s->per[2] = pz != 0;
}

static void orc_reserve(orc_sys* s, int need) {
    if (need <= s->cap) return;
    int nc = s->cap ? s->cap : 1024;
    while (nc < need) nc *= 2;
    for (int k = 0; k < F_COUNT; k++) {
        s->f[k] = (double*)realloc(s->f[k], sizeof(double) * (size_t)nc);
    }
    s->mat = (int32_t*)realloc(s->mat, sizeof(int32_t) * (size_t)nc);
    s->fixed = (uint8_t*)realloc(s->fixed, (size_t)nc);
    s->cap = nc;
}

/* sph.hpp:103-111: one particle with zeroed derived state, hh = h_init */
void orc_add(orc_sys* s, double x, double y, double z, double vx, double vy, double vz,
             double m, double u, int fix) {
    orc_reserve(s, s->n + 1);
    int i = s->n;
    for (int k = 0; k < F_COUNT; k++) s->f[k][i] = 0.0;
    s->f[F_X][i] = x; s->f[F_Y][i] = y; s->f[F_Z][i] = z;
    s->f[F_VX][i] = vx; s->f[F_VY][i] = vy; s->f[F_VZ][i] = vz;
    s->f[F_MASS][i] = m;
    s->f[F_U][i] = u;
    s->f[F_HH][i] = s->prm.h_init;
    s->f[F_H0][i] = s->prm.h_init;
    s->f[F_EPSACT][i] = 1e30;
    s->f[F_DSCALE][i] = 1.0;
    s->mat[i] = s->cur_mat;
    s->fixed[i] = fix ? 1 : 0;
    s->n++;
}

void orc_add_many(orc_sys* s, int n, const double* x, const double* y, const double* z,
                  const double* vx, const double* vy, const double* vz, const double* m,
                  const double* u, const int32_t* mat, const uint8_t* fixed) {
    orc_reserve(s, s->n + n);
    int keep = s->cur_mat;
    for (int i = 0; i < n; i++) {
        if (mat) s->cur_mat = mat[i];
        orc_add(s, x[i], y[i], z[i], vx[i], vy[i], vz[i], m[i], u[i], fixed ? fixed[i] : 0);
    }
    if (mat) s->cur_mat = keep;
}

int orc_n(const orc_sys* s) { return s->n; }

double* orc_field(orc_sys* s, const char* name) {
    for (int k = 0; k < F_COUNT; k++)
        if (strcmp(name, kFieldNames[k]) == 0) return s->f[k];
    return NULL;
}
int32_t* orc_mat_array(orc_sys* s) { return s->mat; }
uint8_t* orc_fixed_array(orc_sys* s) { return s->fixed; }

void orc_set_h0(orc_sys* s, const double* h0) {
    for (int i = 0; i < s->n; i++) s->f[F_H0][i] = h0[i];
    s->use_h0 = 1;
}

static inline double h0_of(const orc_sys* s, int i) {
    return s->use_h0 ? s->f[F_H0][i] : s->prm.h_init;
}

/* ---- Mersenne Twister MT19937 (Matsumoto & Nishimura 1998) and the
 * C++ library's uniform_real_distribution<double>(a, b) built on
 * generate_canonical<double, 53>: two 32-bit draws g0 + g1 * 2^32, divided by
 * 2^64 and clamped below 1, then r * (b - a) + a. ---- */
typedef struct { uint32_t mt[624]; int idx; } orc_mt;

static void mt_seed(orc_mt* g, uint32_t seed) {
    g->mt[0] = seed;
    for (int i = 1; i < 624; i++)
        g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->idx = 624;
}

static uint32_t mt_next(orc_mt* g) {
    if (g->idx >= 624) {
        for (int i = 0; i < 624; i++) {
            uint32_t y = (g->mt[i] & 0x80000000u) | (g->mt[(i + 1) % 624] & 0x7fffffffu);
            uint32_t v = g->mt[(i + 397) % 624] ^ (y >> 1);
            if (y & 1u) v ^= 0x9908b0dfu;
            g->mt[i] = v;
        }
        g->idx = 0;
    }
    uint32_t y = g->mt[g->idx++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

static double mt_uniform(orc_mt* g, double a, double b) {
    double sum = 0.0, tmp = 1.0;
    for (int k = 0; k < 2; k++) {
        sum += (double)mt_next(g) * tmp;
        tmp *= 4294967296.0;
    }
    double r = sum / tmp;
    if (r >= 1.0) r = nextafter(1.0, 0.0);
    return r * (b - a) + a;
}

/* sph.hpp:117-128: one Weibull flaw per brittle particle */
void orc_seed_damage(orc_sys* s, double dx, uint32_t seed) {
    orc_mt g;
    mt_seed(&g, seed);
    double V = dx * dx * dx;
    for (int i = 0; i < s->n; i++) {
        const orc_material* m = &s->mats[s->mat[i]];
        if (m->wk > 0 && m->wm > 0)
            s->f[F_EPSACT][i] = pow(mt_uniform(&g, 1e-9, 1.0) / (m->wk * V), 1.0 / m->wm);
        else
            s->f[F_EPSACT][i] = 1e30;
    }
}

/* Extension (Benz & Asphaug 1995): for each brittle material, N_f = ceil(N ln N)
 * flaws over its N particles of volume dx^3 each; flaw j (1-based, in order of
 * increasing strength) has eps_j = (j / (k V_tot))^(1/m) and lands on a particle
 * drawn uniformly with the seeded generator.  Particles left without a flaw get
 * the next ones in order, so each holds >= 1.  eps_act keeps the weakest. */
int64_t orc_seed_flaws_multi(orc_sys* s, double dx, uint32_t seed) {
    orc_mt g;
    mt_seed(&g, seed);
    int n = s->n;
    int32_t* cnt = (int32_t*)calloc((size_t)n + 1, sizeof(int32_t));
    /* gather brittle particles per material */
    int32_t* list = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    typedef struct { int32_t owner; double eps; } flaw_t;
    flaw_t* flaws = NULL;
    int64_t nf = 0, capf = 0;
    for (int mi = 0; mi < s->nmat; mi++) {
        const orc_material* m = &s->mats[mi];
        if (!(m->wk > 0 && m->wm > 0)) continue;
        int nb = 0;
        for (int i = 0; i < n; i++)
            if (s->mat[i] == mi) list[nb++] = i;
        if (nb == 0) continue;
        double Vtot = (double)nb * dx * dx * dx;
        int64_t Nf = (int64_t)ceil((double)nb * log((double)nb > 1.0 ? (double)nb : 2.0));
        int64_t j = 0;
        for (; j < Nf; j++) {
            uint32_t r = mt_next(&g);
            int32_t owner = list[(int64_t)r % nb];
            if (nf == capf) {
                capf = capf ? 2 * capf : 1024;
                flaws = (flaw_t*)realloc(flaws, sizeof(flaw_t) * (size_t)capf);
            }
            flaws[nf].owner = owner;
            flaws[nf].eps = pow((double)(j + 1) / (m->wk * Vtot), 1.0 / m->wm);
            cnt[owner]++;
            nf++;
        }
        for (int q = 0; q < nb; q++) {
            int32_t i = list[q];
            if (cnt[i] > 0) continue;
            if (nf == capf) {
                capf = capf ? 2 * capf : 1024;
                flaws = (flaw_t*)realloc(flaws, sizeof(flaw_t) * (size_t)capf);
            }
            flaws[nf].owner = i;
            flaws[nf].eps = pow((double)(j + 1) / (m->wk * Vtot), 1.0 / m->wm);
            j++;
            cnt[i]++;
            nf++;
        }
    }
    free(s->flaw_start);
    free(s->flaw_eps);
    s->flaw_start = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
    s->flaw_eps = (double*)malloc(sizeof(double) * (size_t)(nf > 0 ? nf : 1));
    s->flaw_start[0] = 0;
    for (int i = 0; i < n; i++) s->flaw_start[i + 1] = s->flaw_start[i] + cnt[i];
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * ((size_t)n + 1));
    memcpy(fill, s->flaw_start, sizeof(int64_t) * ((size_t)n + 1));
    /* flaws were generated in increasing eps order per material, so each
     * particle's list comes out ascending */
    for (int64_t q = 0; q < nf; q++) s->flaw_eps[fill[flaws[q].owner]++] = flaws[q].eps;
    for (int i = 0; i < n; i++)
        s->f[F_EPSACT][i] = cnt[i] > 0 ? s->flaw_eps[s->flaw_start[i]] : 1e30;
    s->nflaws = nf;
    free(fill);
    free(flaws);
    free(list);
    free(cnt);
    return nf;
}

int64_t orc_flaw_count(const orc_sys* s) { return s->flaw_start ? s->nflaws : 0; }

void orc_flaw_arrays(const orc_sys* s, int64_t* start, double* eps) {
    if (!s->flaw_start) return;
    memcpy(start, s->flaw_start, sizeof(int64_t) * ((size_t)s->n + 1));
    memcpy(eps, s->flaw_eps, sizeof(double) * (size_t)s->nflaws);
}

void orc_set_flaws(orc_sys* s, const int64_t* start, const double* eps) {
    free(s->flaw_start);
    free(s->flaw_eps);
    s->nflaws = start[s->n];
    s->flaw_start = (int64_t*)malloc(sizeof(int64_t) * ((size_t)s->n + 1));
    s->flaw_eps = (double*)malloc(sizeof(double) * (size_t)(s->nflaws > 0 ? s->nflaws : 1));
    memcpy(s->flaw_start, start, sizeof(int64_t) * ((size_t)s->n + 1));
    memcpy(s->flaw_eps, eps, sizeof(double) * (size_t)s->nflaws);
}

/* ---- separation with per-axis minimum image, sph.hpp:130-136 ---- */
static inline void sep(const orc_sys* s, int i, int j, double* dx, double* dy, double* dz) {
    double ax = s->f[F_X][i] - s->f[F_X][j];
    double ay = s->f[F_Y][i] - s->f[F_Y][j];
    double az = s->f[F_Z][i] - s->f[F_Z][j];
    if (s->per[0]) { double L = s->dhi[0] - s->dlo[0]; ax -= L * round(ax / L); }
    if (s->per[1]) { double L = s->dhi[1] - s->dlo[1]; ay -= L * round(ay / L); }
    if (s->per[2]) { double L = s->dhi[2] - s->dlo[2]; az -= L * round(az / L); }
    *dx = ax; *dy = ay; *dz = az;
}

static inline double vnorm(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

/* sph.hpp:142-146.  The float->int conversion saturates (the reference's
 * (int) cast is undefined beyond the int range; saturation keeps every such
 * particle in the clamped border cell, as on the GPU). */
static inline int binof(const orc_sys* s, int ax, double c) {
    double q = (c - s->dlo[ax]) / s->cw[ax];
    int i;
    if (q != q) i = 0;
    else if (q >= 2147483647.0) i = 2147483647;
    else if (q <= -2147483648.0) i = (-2147483647 - 1);
    else i = (int)q;
    if (i < 0) i = 0;
    if (i >= s->nc[ax]) i = s->nc[ax] - 1;
    return i;
}

/* sph.hpp:147-162: grid of width ext / floor(ext / 2 h_max) over the domain;
 * each cell lists its particles in ascending index. */
void orc_build_cells(orc_sys* s) {
    int n = s->n;
    double hm = 1e-30;
    for (int i = 0; i < n; i++) hm = dmax(hm, s->f[F_HH][i]);
    s->h_max = hm;
    double rc = 2.0 * hm;
    for (int a = 0; a < 3; a++) {
        double ext = s->dhi[a] - s->dlo[a];
        if (ext <= 0) ext = rc;
        double q = ext / rc;
        int m = q >= 2147483647.0 ? 2147483647 : (int)q;
        if (m < 1) m = 1;
        if (s->per[a] && m < 3) m = 1;
        s->nc[a] = m;
        s->cw[a] = ext / m;
    }
    int64_t nc = (int64_t)s->nc[0] * s->nc[1] * s->nc[2];
    s->ncells = nc;
    free(s->cell_start);
    free(s->cell_ids);
    free(s->cell_of);
    s->cell_start = (int32_t*)calloc((size_t)nc + 1, sizeof(int32_t));
    s->cell_ids = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    s->cell_of = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) {
        int64_t c = ((int64_t)binof(s, 0, s->f[F_X][i]) * s->nc[1] + binof(s, 1, s->f[F_Y][i])) *
                        s->nc[2] +
                    binof(s, 2, s->f[F_Z][i]);
        s->cell_of[i] = (int32_t)c;
        s->cell_start[c + 1]++;
    }
    for (int64_t c = 0; c < nc; c++) s->cell_start[c + 1] += s->cell_start[c];
    int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nc > 0 ? nc : 1));
    memcpy(fill, s->cell_start, sizeof(int32_t) * (size_t)nc);
    for (int i = 0; i < n; i++) s->cell_ids[fill[s->cell_of[i]]++] = i;
    free(fill);
}

/* sph.hpp:163-182: 27-cell stencil (collapsed on single-cell axes), periodic
 * wrap, cells in (d0, d1, d2) order, each cell's particles ascending.  The
 * stencil is materialised as a list of cell ids for one particle. */
static int stencil(const orc_sys* s, int i, int64_t* cells) {
    int b[3] = {binof(s, 0, s->f[F_X][i]), binof(s, 1, s->f[F_Y][i]), binof(s, 2, s->f[F_Z][i])};
    int lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = s->nc[a] > 1 ? -1 : 0;
        hi[a] = s->nc[a] > 1 ? 1 : 0;
    }
    int k = 0;
    for (int d0 = lo[0]; d0 <= hi[0]; d0++) {
        int j0 = b[0] + d0;
        if (s->per[0]) j0 = ((j0 % s->nc[0]) + s->nc[0]) % s->nc[0];
        else if (j0 < 0 || j0 >= s->nc[0]) continue;
        for (int d1 = lo[1]; d1 <= hi[1]; d1++) {
            int j1 = b[1] + d1;
            if (s->per[1]) j1 = ((j1 % s->nc[1]) + s->nc[1]) % s->nc[1];
            else if (j1 < 0 || j1 >= s->nc[1]) continue;
            for (int d2 = lo[2]; d2 <= hi[2]; d2++) {
                int j2 = b[2] + d2;
                if (s->per[2]) j2 = ((j2 % s->nc[2]) + s->nc[2]) % s->nc[2];
                else if (j2 < 0 || j2 >= s->nc[2]) continue;
                cells[k++] = ((int64_t)j0 * s->nc[1] + j1) * s->nc[2] + j2;
            }
        }
    }
    return k;
}

/* ---- density + adaptive h, sph.hpp:184-208 ---- */
static void density_body(void* ctx, int lo, int hi_) {
    orc_sys* s = (orc_sys*)ctx;
    int64_t cells[27];
    const double eta = s->prm.eta;
    for (int i = lo; i < hi_; i++) {
        double sum = 0, hi = s->f[F_HH][i];
        int nc = stencil(s, i, cells);
        for (int c = 0; c < nc; c++) {
            for (int32_t k = s->cell_start[cells[c]]; k < s->cell_start[cells[c] + 1]; k++) {
                int j = s->cell_ids[k];
                double dx, dy, dz;
                sep(s, i, j, &dx, &dy, &dz);
                double r = vnorm(dx, dy, dz);
                if (r < 2.0 * hi) sum += s->f[F_MASS][j] * orc_kW(r, hi);
            }
        }
        s->f[F_RHO][i] = dmax(sum, 1e-30);
        double h0 = h0_of(s, i);
        s->f[F_HH][i] = dmin(2.0 * h0, dmax(0.5 * h0, eta * cbrt(s->f[F_MASS][i] / s->f[F_RHO][i])));
    }
}

void orc_compute_density_h(orc_sys* s, int iters) {
    for (int round = 0; round < 4; round++) {
        orc_build_cells(s);
        double hmax0 = s->h_max;
        for (int it = 0; it < iters; it++) orc_parallel_for(s->nthreads, s->n, density_body, s);
        double hm = 1e-30;
        for (int i = 0; i < s->n; i++) hm = dmax(hm, s->f[F_HH][i]);
        if (hm <= hmax0 * 1.02) break;
    }
    orc_build_cells(s);
}

/* ---- velocity gradient -> Jaumann dS/dt + deviatoric power, sph.hpp:212-258 ---- */
static void strain_body(void* ctx, int lo, int hi_) {
    orc_sys* s = (orc_sys*)ctx;
    int64_t cells[27];
    double** f = s->f;
    for (int i = lo; i < hi_; i++) {
        double G = s->mats[s->mat[i]].G;
        if (G <= 0) {
            for (int k = F_DSXX; k <= F_DSYZ; k++) f[k][i] = 0;
            f[F_EPSW][i] = 0;
            continue;
        }
        double L[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        int nc = stencil(s, i, cells);
        for (int c = 0; c < nc; c++) {
            for (int32_t k = s->cell_start[cells[c]]; k < s->cell_start[cells[c] + 1]; k++) {
                int j = s->cell_ids[k];
                if (j == i) continue;
                double rx, ry, rz;
                sep(s, i, j, &rx, &ry, &rz);
                double r = vnorm(rx, ry, rz);
                double hbar = 0.5 * (f[F_HH][i] + f[F_HH][j]);
                if (r >= 2.0 * hbar || r == 0) continue;
                double w = orc_kdWdr(r, hbar) / r;
                double g[3] = {rx * w, ry * w, rz * w};
                double Vj = f[F_MASS][j] / f[F_RHO][j];
                double d[3] = {f[F_VX][j] - f[F_VX][i], f[F_VY][j] - f[F_VY][i],
                               f[F_VZ][j] - f[F_VZ][i]};
                for (int a = 0; a < 3; a++)
                    for (int bb = 0; bb < 3; bb++) L[a][bb] += Vj * d[a] * g[bb];
            }
        }
        double exx = L[0][0], eyy = L[1][1], ezz = L[2][2];
        double exy = 0.5 * (L[0][1] + L[1][0]), exz = 0.5 * (L[0][2] + L[2][0]),
               eyz = 0.5 * (L[1][2] + L[2][1]);
        double Rxy = 0.5 * (L[0][1] - L[1][0]), Rxz = 0.5 * (L[0][2] - L[2][0]),
               Ryz = 0.5 * (L[1][2] - L[2][1]);
        double tr = (exx + eyy + ezz) / 3.0;
        double sxx = f[F_SXX][i], syy = f[F_SYY][i], szz = f[F_SZZ][i];
        double sxy = f[F_SXY][i], sxz = f[F_SXZ][i], syz = f[F_SYZ][i];
        double R[3][3] = {{0, Rxy, Rxz}, {-Rxy, 0, Ryz}, {-Rxz, -Ryz, 0}};
        double Sm[3][3] = {{sxx, sxy, sxz}, {sxy, syy, syz}, {sxz, syz, szz}};
        double J[3][3];
        for (int a = 0; a < 3; a++)
            for (int bb = 0; bb < 3; bb++) {
                double rs = 0, sr = 0;
                for (int c = 0; c < 3; c++) {
                    rs += R[a][c] * Sm[c][bb];
                    sr += Sm[a][c] * R[c][bb];
                }
                J[a][bb] = rs - sr;
            }
        f[F_DSXX][i] = 2 * G * (exx - tr) + J[0][0];
        f[F_DSYY][i] = 2 * G * (eyy - tr) + J[1][1];
        f[F_DSZZ][i] = 2 * G * (ezz - tr) + J[2][2];
        f[F_DSXY][i] = 2 * G * exy + J[0][1];
        f[F_DSXZ][i] = 2 * G * exz + J[0][2];
        f[F_DSYZ][i] = 2 * G * eyz + J[1][2];
        f[F_EPSW][i] = (sxx * exx + syy * eyy + szz * ezz + 2 * (sxy * exy + sxz * exz + syz * eyz)) /
                       f[F_RHO][i];
    }
}

void orc_compute_strain_stress(orc_sys* s) { orc_parallel_for(s->nthreads, s->n, strain_body, s); }

/* ---- EOS + damage pre-pass, sph.hpp:261-275 ---- */
static void eos_body(void* ctx, int lo, int hi_) {
    orc_sys* s = (orc_sys*)ctx;
    double** f = s->f;
    for (int i = lo; i < hi_; i++) {
        const orc_material* m = &s->mats[s->mat[i]];
        f[F_P][i] = orc_pressure(m, f[F_RHO][i], f[F_U][i]);
        f[F_CS][i] = orc_sound_speed(m, f[F_RHO][i], f[F_U][i]);
        f[F_CSIG][i] = sqrt(f[F_CS][i] * f[F_CS][i] + (4.0 / 3.0) * m->G / dmax(f[F_RHO][i], 1e-30));
        double pf = f[F_P][i], dsc = 1.0;
        if (s->prm.damage_on) {
            double sv[6] = {f[F_SXX][i], f[F_SYY][i], f[F_SZZ][i], f[F_SXY][i], f[F_SXZ][i], f[F_SYZ][i]};
            f[F_SIGMAX][i] = -f[F_P][i] + orc_eig_max(sv);
            dsc = 1.0 - f[F_D][i];
            if (f[F_P][i] < 0) pf = dsc * f[F_P][i];
        }
        f[F_PF][i] = pf;
        f[F_DSCALE][i] = dsc;
        f[F_RART][i] = (s->prm.eps_as > 0 && pf < 0) ? s->prm.eps_as * (-pf) / (f[F_RHO][i] * f[F_RHO][i]) : 0.0;
    }
}

/* ---- momentum + energy pair loop, sph.hpp:277-317 ---- */
static void force_body(void* ctx, int lo, int hi_) {
    orc_sys* s = (orc_sys*)ctx;
    int64_t cells[27];
    double** f = s->f;
    const double eta = s->prm.eta, alpha = s->prm.alpha, beta = s->prm.beta, eps = s->prm.eps;
    const double alpha_u = s->prm.alpha_u, eps_as = s->prm.eps_as;
    for (int i = lo; i < hi_; i++) {
        double ax = 0, ay = 0, az = 0, du = 0;
        double iri2 = 1.0 / (f[F_RHO][i] * f[F_RHO][i]);
        double Pi_over = f[F_PF][i] * iri2;
        double di = f[F_DSCALE][i];
        double sxx = f[F_SXX][i], syy = f[F_SYY][i], szz = f[F_SZZ][i];
        double sxy = f[F_SXY][i], sxz = f[F_SXZ][i], syz = f[F_SYZ][i];
        int nc = stencil(s, i, cells);
        for (int c = 0; c < nc; c++) {
            for (int32_t k = s->cell_start[cells[c]]; k < s->cell_start[cells[c] + 1]; k++) {
                int j = s->cell_ids[k];
                if (j == i) continue;
                double rx, ry, rz;
                sep(s, i, j, &rx, &ry, &rz);
                double r = vnorm(rx, ry, rz);
                double hbar = 0.5 * (f[F_HH][i] + f[F_HH][j]);
                if (r >= 2.0 * hbar || r == 0) continue;
                double w = orc_kdWdr(r, hbar) / r;
                double gx = rx * w, gy = ry * w, gz = rz * w;
                double vx = f[F_VX][i] - f[F_VX][j], vy = f[F_VY][i] - f[F_VY][j],
                       vz = f[F_VZ][i] - f[F_VZ][j];
                double rbar = 0.5 * (f[F_RHO][i] + f[F_RHO][j]);
                double Pij = 0, dvr = vx * rx + vy * ry + vz * rz;
                if (dvr < 0) {
                    double mu = hbar * dvr / (r * r + eps * hbar * hbar);
                    double cbar = 0.5 * (f[F_CSIG][i] + f[F_CSIG][j]);
                    Pij = (-alpha * cbar * mu + beta * mu * mu) / rbar;
                }
                double jrj2 = 1.0 / (f[F_RHO][j] * f[F_RHO][j]);
                double term = Pi_over + f[F_PF][j] * jrj2 + Pij;
                double mj = f[F_MASS][j];
                du += 0.5 * mj * term * (vx * gx + vy * gy + vz * gz);
                double mterm = term;
                if (eps_as > 0) {
                    double wdp = orc_kW(hbar / eta, hbar);
                    double fr = (wdp > 0 ? orc_kW(r, hbar) / wdp : 0.0);
                    double fn = fr * fr;
                    fn *= fn;
                    mterm += (f[F_RART][i] + f[F_RART][j]) * fn;
                }
                double mm = mj * mterm;
                ax -= gx * mm;
                ay -= gy * mm;
                az -= gz * mm;
                /* S_i . g and S_j . g (sph.hpp:34-38) */
                double six = sxx * gx + sxy * gy + sxz * gz;
                double siy = sxy * gx + syy * gy + syz * gz;
                double siz = sxz * gx + syz * gy + szz * gz;
                double tx = f[F_SXX][j], ty = f[F_SYY][j], tz = f[F_SZZ][j];
                double txy = f[F_SXY][j], txz = f[F_SXZ][j], tyz = f[F_SYZ][j];
                double sjx = tx * gx + txy * gy + txz * gz;
                double sjy = txy * gx + ty * gy + tyz * gz;
                double sjz = txz * gx + tyz * gy + tz * gz;
                double ci = iri2 * di, cj = jrj2 * f[F_DSCALE][j];
                double stx = six * ci + sjx * cj;
                double sty = siy * ci + sjy * cj;
                double stz = siz * ci + sjz * cj;
                ax += stx * mj;
                ay += sty * mj;
                az += stz * mj;
                if (alpha_u > 0) {
                    double vsig = sqrt(fabs(f[F_P][i] - f[F_P][j]) / rbar);
                    du += alpha_u * mj * vsig * (f[F_U][i] - f[F_U][j]) * orc_kdWdr(r, hbar) / rbar;
                }
            }
        }
        f[F_AX][i] = ax;
        f[F_AY][i] = ay;
        f[F_AZ][i] = az;
        f[F_DUDT][i] = du + f[F_EPSW][i] * di;
    }
}

void orc_compute_forces(orc_sys* s) {
    orc_parallel_for(s->nthreads, s->n, eos_body, s);
    orc_compute_strain_stress(s);
    orc_parallel_for(s->nthreads, s->n, force_body, s);
}

/* ---- yield: von Mises radial return, sph.hpp:320-331; Collins (extension)
 * from hydrocodes/euler/hydro_cpu.cpp:229-252 ---- */
void orc_yield_limit(orc_sys* s, int i) {
    const orc_material* m = &s->mats[s->mat[i]];
    double** f = s->f;
    double Y = m->Y;
    if (m->yield_model == ORC_YIELD_COLLINS) {
        double P = dmax(f[F_P][i], 0.0);
        double Yi = m->Y0 + m->mu_i * P / (1.0 + m->mu_i * P / dmax(m->Ylim - m->Y0, 1.0));
        double Yd = dmin(m->Yd0 + m->mu_d * P, m->Ylim);
        double D = f[F_D][i];
        Y = (1.0 - D) * Yi + D * Yd;
    }
    if (Y <= 0) {
        for (int k = F_SXX; k <= F_SYZ; k++) f[k][i] = 0;
        return;
    }
    double xx = f[F_SXX][i], yy = f[F_SYY][i], zz = f[F_SZZ][i];
    double xy = f[F_SXY][i], xz = f[F_SXZ][i], yz = f[F_SYZ][i];
    double J2 = 0.5 * (xx * xx + yy * yy + zz * zz) + (xy * xy + xz * xz + yz * yz);
    double vm = sqrt(3.0 * J2);
    if (vm > Y) {
        double fct = Y / vm;
        f[F_SXX][i] = xx * fct; f[F_SYY][i] = yy * fct; f[F_SZZ][i] = zz * fct;
        f[F_SXY][i] = xy * fct; f[F_SXZ][i] = xz * fct; f[F_SYZ][i] = yz * fct;
    }
}

/* ---- Grady-Kipp / Benz-Asphaug crack growth, sph.hpp:336-348 ---- */
static void damage_body_single(orc_sys* s, int i, double dt) {
    const orc_material* m = &s->mats[s->mat[i]];
    double** f = s->f;
    if (m->Emod <= 0 || f[F_D][i] >= 1.0) return;
    double eps_local = f[F_SIGMAX][i] / m->Emod;
    if (f[F_SIGMAX][i] > 0 && eps_local > f[F_EPSACT][i]) {
        double cg = 0.4 * sqrt(m->Emod / dmax(f[F_RHO][i], 1e-30));
        double Rs = 0.5 * h0_of(s, i) / s->prm.eta;
        double d13 = cbrt(f[F_D][i]) + (cg / Rs) * dt;
        f[F_D][i] = dmin(1.0, d13 * d13 * d13);
    }
}

/* extension: multi-flaw growth, rate x n_act^(1/3), damage <= n_act / n_flaws */
static void damage_body_multi(orc_sys* s, int i, double dt) {
    const orc_material* m = &s->mats[s->mat[i]];
    double** f = s->f;
    if (m->Emod <= 0 || f[F_D][i] >= 1.0) return;
    int64_t b = s->flaw_start[i], e = s->flaw_start[i + 1];
    if (e <= b) return;
    double eps_local = f[F_SIGMAX][i] / m->Emod;
    if (!(f[F_SIGMAX][i] > 0 && eps_local > f[F_EPSACT][i])) return;
    int64_t nact = 0;
    for (int64_t k = b; k < e; k++)
        if (eps_local > s->flaw_eps[k]) nact++;
    double cg = 0.4 * sqrt(m->Emod / dmax(f[F_RHO][i], 1e-30));
    double Rs = 0.5 * h0_of(s, i) / s->prm.eta;
    double d13 = cbrt(f[F_D][i]) + cbrt((double)nact) * (cg / Rs) * dt;
    double cap = (double)nact / (double)(e - b);
    double Dn = dmin(cap, d13 * d13 * d13);
    if (Dn > f[F_D][i]) f[F_D][i] = Dn;
}

typedef struct { orc_sys* s; double dt; } dmg_ctx;
static void damage_body(void* ctx, int lo, int hi_) {
    dmg_ctx* c = (dmg_ctx*)ctx;
    int multi = c->s->prm.flaw_model == ORC_FLAWS_MULTI && c->s->flaw_start;
    for (int i = lo; i < hi_; i++) {
        if (multi) damage_body_multi(c->s, i, c->dt);
        else damage_body_single(c->s, i, c->dt);
    }
}

void orc_grow_damage(orc_sys* s, double dt) {
    dmg_ctx c = {s, dt};
    orc_parallel_for(s->nthreads, s->n, damage_body, &c);
}

/* ---- CFL time step, sph.hpp:350-355 ---- */
double orc_timestep(const orc_sys* s) {
    double dt = 1e30;
    for (int i = 0; i < s->n; i++)
        dt = dmin(dt, s->prm.cfl * s->f[F_HH][i] / (s->f[F_CSIG][i] * (1.0 + s->prm.alpha) + 1e-30));
    return dt;
}

/* ---- KDK step, sph.hpp:357-377 ---- */
void orc_step(orc_sys* s, double dt) {
    int n = s->n;
    double** f = s->f;
    double* dudt_old = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    double* dS_old = (double*)malloc(sizeof(double) * 6 * (size_t)(n > 0 ? n : 1));
    memcpy(dudt_old, f[F_DUDT], sizeof(double) * (size_t)n);
    for (int k = 0; k < 6; k++) memcpy(dS_old + (size_t)k * n, f[F_DSXX + k], sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++)
        if (!s->fixed[i]) {
            f[F_VX][i] += f[F_AX][i] * (0.5 * dt);
            f[F_VY][i] += f[F_AY][i] * (0.5 * dt);
            f[F_VZ][i] += f[F_AZ][i] * (0.5 * dt);
        }
    for (int i = 0; i < n; i++)
        if (!s->fixed[i]) {
            f[F_X][i] += f[F_VX][i] * dt;
            f[F_Y][i] += f[F_VY][i] * dt;
            f[F_Z][i] += f[F_VZ][i] * dt;
        }
    orc_compute_density_h(s, 2);
    orc_compute_forces(s);
    if (s->prm.damage_on) orc_grow_damage(s, dt);
    for (int i = 0; i < n; i++)
        if (!s->fixed[i]) {
            f[F_VX][i] += f[F_AX][i] * (0.5 * dt);
            f[F_VY][i] += f[F_AY][i] * (0.5 * dt);
            f[F_VZ][i] += f[F_AZ][i] * (0.5 * dt);
            f[F_U][i] += 0.5 * dt * (dudt_old[i] + f[F_DUDT][i]);
            if (f[F_U][i] < 1e-12) f[F_U][i] = 1e-12;
            for (int k = 0; k < 6; k++)
                f[F_SXX + k][i] += 0.5 * dt * (dS_old[(size_t)k * n + i] + f[F_DSXX + k][i]);
            orc_yield_limit(s, i);
        }
    free(dudt_old);
    free(dS_old);
}

void orc_init(orc_sys* s) { /* sph.hpp:379 */
    orc_compute_density_h(s, 2);
    orc_compute_forces(s);
}

/* ---- inspection ---- */
void orc_grid(const orc_sys* s, int32_t nc[3], double cw[3], double* h_max) {
    for (int a = 0; a < 3; a++) { nc[a] = s->nc[a]; cw[a] = s->cw[a]; }
    if (h_max) *h_max = s->h_max;
}
int64_t orc_ncells(const orc_sys* s) { return s->ncells; }
void orc_cell_of(const orc_sys* s, int32_t* cell) {
    if (s->cell_of) memcpy(cell, s->cell_of, sizeof(int32_t) * (size_t)s->n);
}
void orc_cell_csr(const orc_sys* s, int32_t* start, int32_t* ids) {
    if (!s->cell_start) return;
    memcpy(start, s->cell_start, sizeof(int32_t) * ((size_t)s->ncells + 1));
    memcpy(ids, s->cell_ids, sizeof(int32_t) * (size_t)s->n);
}

int64_t orc_neighbors(const orc_sys* s, int kind, int32_t* counts, int32_t* ids, int64_t cap) {
    int64_t total = 0;
    int64_t cells[27];
    double* const* f = s->f;
    for (int i = 0; i < s->n; i++) {
        int cnt = 0;
        int nc = stencil(s, i, cells);
        for (int c = 0; c < nc; c++) {
            for (int32_t k = s->cell_start[cells[c]]; k < s->cell_start[cells[c] + 1]; k++) {
                int j = s->cell_ids[k];
                double rx, ry, rz;
                sep(s, i, j, &rx, &ry, &rz);
                double r = vnorm(rx, ry, rz);
                int take;
                if (kind == ORC_NBR_DENSITY) {
                    take = r < 2.0 * f[F_HH][i];
                } else {
                    double hbar = 0.5 * (f[F_HH][i] + f[F_HH][j]);
                    take = !(j == i || r >= 2.0 * hbar || r == 0);
                }
                if (take) {
                    if (ids && total < cap) ids[total] = j;
                    total++;
                    cnt++;
                }
            }
        }
        if (counts) counts[i] = cnt;
    }
    return total <= cap ? total : -total;
}
