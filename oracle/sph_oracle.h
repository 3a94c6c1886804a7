/*
 * sph_oracle.h -- CPU oracle for the SPH step loop (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C, structure-of-arrays restatement of the reference's FP64 CPU solver
 * (hydrocodes/sph/sph.hpp) and its Tillotson EOS (hydrocodes/common/eos.hpp).
 * It exists to check the CUDA solver: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load it.  The product path never calls it.
 *
 * Floating-point operations are written in the same order as the reference
 * expressions and the library is built with -ffp-contract=off, so on the same
 * inputs it reproduces the reference bit for bit (checked against the
 * reference compiled from its own headers, see oracle/Makefile and
 * tests/golden/make_golden.py).
 *
 * Physics the reference SPH does not have, all OFF by default (default-off
 * behaviour is bit-identical to the reference):
 *   - Collins / Lundborg pressure-dependent yield per material, restated from
 *     hydrocodes/euler/hydro_cpu.cpp:229-252 (intact saturating friction,
 *     damaged friction capped at Ylim, (1-D)/D blend, P clamped >= 0).
 *   - Benz & Asphaug (1995) multi-flaw Weibull damage: N ln N flaws with
 *     thresholds eps_j = (j / (k V))^(1/m) assigned to random particles; growth
 *     rate scaled by n_act^(1/3), damage capped at n_act / n_flaws.
 *   - Per-particle reference smoothing length h0 (graded lattices): the h clamp
 *     [0.5, 2] h0 and the crack radius R_s = 0.5 h0 / eta use h0_i.
 */
#ifndef DEORBIT_SPH_ORACLE_H
#define DEORBIT_SPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_IDEAL = 0, ORC_TILLOTSON = 1 };
enum { ORC_YIELD_VON_MISES = 0, ORC_YIELD_COLLINS = 1 };
enum { ORC_FLAWS_SINGLE = 0, ORC_FLAWS_MULTI = 1 };
enum { ORC_NBR_DENSITY = 0, ORC_NBR_FORCE = 1 };

/* hydrocodes/common/eos.hpp:15-27 (+ Collins fields, extension) */
typedef struct {
    int32_t type;
    int32_t yield_model;
    double gamma;
    double rho0, a, b, A, B, alpha, beta, u0, uiv, ucv;
    double G, Y, Emod, wm, wk;
    double Y0, mu_i, Ylim, Yd0, mu_d; /* Collins (yield_model == 1) */
} orc_material;

/* hydrocodes/sph/sph.hpp:86-92 (+ extension switches) */
typedef struct {
    double eta, h_init, alpha, beta, eps, alpha_u, cfl, eps_as;
    int32_t as_n, damage_on;
    int32_t flaw_model; /* ORC_FLAWS_* */
    int32_t pad_;
} orc_params;

/* ---- materials and EOS (eos.hpp) ---- */
orc_material orc_mat_ideal(double gamma);
orc_material orc_mat_tillotson(double rho0, double A, double B, double a, double b,
                               double alpha, double beta, double u0, double uiv,
                               double ucv, double G, double Y, double wm, double wk);
orc_material orc_mat_iron(void);
orc_material orc_mat_basalt(void);
orc_material orc_mat_water(void);
orc_material orc_mat_aluminum(void);
double orc_pressure(const orc_material* m, double rho, double u);
double orc_sound_speed(const orc_material* m, double rho, double u);
void orc_eos_batch(const orc_material* m, int n, const double* rho, const double* u,
                   double* P, double* cs);

/* ---- kernel and tensor helpers (sph.hpp:17-54) ---- */
double orc_kW(double r, double h);
double orc_kdWdr(double r, double h);
double orc_eig_max(const double s[6]); /* s = {xx, yy, zz, xy, xz, yz} */

/* ---- the particle system (sph.hpp:72-380) ---- */
typedef struct orc_sys orc_sys;

orc_sys* orc_create(void);
void orc_destroy(orc_sys* s);
void orc_set_threads(orc_sys* s, int nthreads); /* 0: min(hardware, 16) like the reference */
int orc_get_threads(const orc_sys* s);
void orc_get_params(const orc_sys* s, orc_params* p);
void orc_set_params(orc_sys* s, const orc_params* p);
int orc_add_material(orc_sys* s, const orc_material* m);
void orc_set_cur_mat(orc_sys* s, int mat);
void orc_set_domain(orc_sys* s, double xl, double xh, int px, double yl, double yh, int py,
                    double zl, double zh, int pz);
/* sph.hpp:103-111, one call per particle or in bulk (arrays of length n) */
void orc_add(orc_sys* s, double x, double y, double z, double vx, double vy, double vz,
             double m, double u, int fixed);
void orc_add_many(orc_sys* s, int n, const double* x, const double* y, const double* z,
                  const double* vx, const double* vy, const double* vz, const double* m,
                  const double* u, const int32_t* mat, const uint8_t* fixed);
int orc_n(const orc_sys* s);

/* field access: name in {x y z vx vy vz ax ay az mass rho u dudt P cs csig hh
 * eps_work D eps_act sigmax Pf Rart dscale Sxx Syy Szz Sxy Sxz Syz dSxx dSyy dSzz
 * dSxy dSxz dSyz h0}; returns NULL for an unknown name. */
double* orc_field(orc_sys* s, const char* name);
int32_t* orc_mat_array(orc_sys* s);
uint8_t* orc_fixed_array(orc_sys* s);
/* extension: enable per-particle h0 (copied from h0, length n) */
void orc_set_h0(orc_sys* s, const double* h0);

void orc_seed_damage(orc_sys* s, double dx, uint32_t seed);      /* sph.hpp:117-128 */
/* extension: Benz-Asphaug multi-flaw seeding; returns total flaws */
int64_t orc_seed_flaws_multi(orc_sys* s, double dx, uint32_t seed);
int64_t orc_flaw_count(const orc_sys* s);
void orc_flaw_arrays(const orc_sys* s, int64_t* start /* n+1 */, double* eps /* total */);
void orc_set_flaws(orc_sys* s, const int64_t* start, const double* eps);

void orc_build_cells(orc_sys* s);                                /* sph.hpp:147-162 */
void orc_compute_density_h(orc_sys* s, int iters);               /* sph.hpp:184-208 */
void orc_compute_strain_stress(orc_sys* s);                      /* sph.hpp:212-258 */
void orc_compute_forces(orc_sys* s);                             /* sph.hpp:260-318 */
void orc_yield_limit(orc_sys* s, int i);                         /* sph.hpp:320-331 */
void orc_grow_damage(orc_sys* s, double dt);                     /* sph.hpp:336-348 */
double orc_timestep(const orc_sys* s);                           /* sph.hpp:350-355 */
void orc_step(orc_sys* s, double dt);                            /* sph.hpp:357-377 */
void orc_init(orc_sys* s);                                       /* sph.hpp:379 */

/* ---- inspection of the last cell build (integer outputs, bit-exact) ---- */
void orc_grid(const orc_sys* s, int32_t nc[3], double cw[3], double* h_max);
int64_t orc_ncells(const orc_sys* s);
/* per particle cell id (linear, (b0*nc1+b1)*nc2+b2) */
void orc_cell_of(const orc_sys* s, int32_t* cell);
/* CSR of the cell list: start has ncells+1 entries, ids has n entries */
void orc_cell_csr(const orc_sys* s, int32_t* start, int32_t* ids);
/* neighbour sets over the current cells: kind ORC_NBR_DENSITY is
 * {j : r < 2 h_i} (self included), ORC_NBR_FORCE is {j != i : r < 2 hbar, r != 0}.
 * counts has n entries; ids (capacity cap) receives the sets in the reference's
 * visiting order.  Returns the total, or -total if cap was too small. */
int64_t orc_neighbors(const orc_sys* s, int kind, int32_t* counts, int32_t* ids, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
