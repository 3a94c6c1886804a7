/* euler_oracle.h -- CPU oracle of the Eulerian grid hydrocode (TEST ONLY).
 *
 * A plain C restatement of the reference's CPU Euler solver
 * (hydrocodes/euler/hydro_cpu.cpp): unsplit MUSCL-minmod + HLLC hydro sweeps
 * with a passive material tracer (hydro_cpu.cpp:54-74,98-136), the
 * vacuum-aware face flux (43-53), gravity (137-144), elastic-plastic
 * strength with the Jaumann rate, upwind stress advection, div S and div(S.v)
 * in Cartesian or cylindrical (r, z) geometry (145-214), von Mises and the
 * pressure-dependent ROCK yield (229-252), tensile damage growth (253-258),
 * the frozen hydrostatic reference of set_ref (259-261) with the well-balanced
 * z-sweep and gravity source against it (75-88, 114-119, 139-143), the
 * near-void reset to that reference or to an ambient density, optionally
 * conservative (272-290), acoustic fluidization activation (390-410), the CFL
 * speed (378-380), the implicit fluidization viscosity (VISC_IMP: backward
 * Euler, Jacobi-preconditioned conjugate gradients, dissipation returned as
 * heat, 286-377) and the two-stage Runge-Kutta step (411-425).  Every
 * expression keeps the reference's floating-point operation order, sums
 * included; the library is built with -ffp-contract=off.
 *
 * The oracle is test infrastructure: only tests/, the smoke check and the
 * bench's CPU legs call it, never the product path.
 */
#ifndef DEORBIT_EULER_ORACLE_H
#define DEORBIT_EULER_ORACLE_H

#include "sph_oracle.h" /* orc_material, orc_pressure, orc_sound_speed */

#ifdef __cplusplus
extern "C" {
#endif

/* Solver switches and constants: the file-scope settings of hydro_cpu.cpp:15-36
 * and 222-223 (same names in lower case, defaults from eorc_params_default). */
typedef struct {
    double gz;        /* gravity toward -z (m/s^2) */
    double tdec;      /* acoustic-fluidization vibration decay time (s); 0 = AF off */
    double eta_af;    /* AF viscosity (Pa s) */
    double c_act;     /* AF shock-activation coupling; 0 = off */
    double p_coh;     /* cohesion floor of the overburden (Pa) */
    double p_act;     /* shock-sized pressure jump that seeds vibrations (Pa) */
    double rho_cfl;   /* near-void density excluded from CFL and strength */
    double damp;      /* velocity damping per step; 1 = off */
    double rho_vac;   /* vacuum-aware flux threshold; 0 = off */
    double y_i0, mu_i, mu_d, y_d0, y_m, y_bingham;
    double c_reg, af_sat;
    int axisym;       /* cylindrical (r, z): x -> r, ny = 1 */
    int rock;         /* pressure-dependent yield */
    int af_reg;       /* vibration regeneration from plastic work */
    int af_prel;      /* overburden relief constitutive form */
    int af_seeddp;    /* seed vibrations from the acoustic velocity of the jump */
    int pad_;
    double void_amb;  /* void cells reset to this ambient density instead of the reference's */
    int void_cons;    /* conservative reset: excess mass to the densest neighbour first */
    int visc_imp;     /* fluidization viscosity by the implicit solve instead of the Lop term */
} eorc_params;

void eorc_params_default(eorc_params* p);

typedef struct eorc_grid eorc_grid;

/* Grid of nx*ny*nz cells of width dx, all fields zero; cell (i,j,k) at
 * (i*ny + j)*nz + k (hydro_cpu.cpp:90-93). */
eorc_grid* eorc_create(int nx, int ny, int nz, double dx);
void eorc_destroy(eorc_grid* g);
void eorc_set_material(eorc_grid* g, const orc_material* m);
void eorc_set_params(eorc_grid* g, const eorc_params* p);
/* Per-cell field by name: r mu mv mw E Sxx Syy Szz Sxy Sxz Syz D af rc vib Pmax;
 * NULL for an unknown name.  The array holds nx*ny*nz doubles. */
double* eorc_field(eorc_grid* g, const char* name);
/* Right-hand side of the last eorc_lop call by name (r mu mv mw E Sxx Syy Szz
 * Sxy Sxz Syz D rc vib). */
double* eorc_rhs(eorc_grid* g, const char* name);

/* set_ref (hydro_cpu.cpp:259-261): the current density and pressure become
 * the hydrostatic reference of the well-balanced sweep and the void reset;
 * eorc_clear_ref drops it. */
void eorc_set_ref(eorc_grid* g);
void eorc_clear_ref(eorc_grid* g);
void eorc_lop(eorc_grid* g);                    /* hydro_cpu.cpp:98-214 */
void eorc_vonmises(eorc_grid* g, int reg);      /* 229-252 */
void eorc_grow_damage(eorc_grid* g, double dt); /* 253-258 */
void eorc_update_af(eorc_grid* g, double dt);   /* 390-410 */
double eorc_maxspeed(const eorc_grid* g);       /* 378-380 */
/* implicit_visc(g, dt) (hydro_cpu.cpp:301-377): a no-op unless visc_imp is set
 * and eta_af > 0; eorc_visc_iters counts its conjugate-gradient iterations
 * since the grid was created (the reference's VISC_IT). */
void eorc_implicit_visc(eorc_grid* g, double dt);
long eorc_visc_iters(const eorc_grid* g);
void eorc_step_rk2(eorc_grid* g, double dt);    /* 411-425 */
/* The reference drivers' loop (hydro_cpu.cpp:452 and every mode): dt =
 * cfl*dx/maxspeed, clipped at t_end; runs until t_end or max_steps steps.
 * Returns the number of steps; *t_out receives the time reached. */
int eorc_run(eorc_grid* g, double cfl, double t_end, int max_steps, double* t_out);
/* Pressure of cell c (EOS at the cell's internal energy, clamped at 0). */
double eorc_pcell(const eorc_grid* g, int c);

#ifdef __cplusplus
}
#endif
#endif
