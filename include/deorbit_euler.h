/*
 * deorbit_euler.h -- C ABI of the GB300 Eulerian grid hydrocode
 * (libdeorbit_sph.so, beside the SPH solver of deorbit_sph.h).
 *
 * Drop-in boundary for the reference's CPU Euler solver
 * (hydrocodes/euler/hydro_cpu.cpp): the `Grid` of conserved and material
 * fields (hydro_cpu.cpp:90-93), its right-hand side `Lop` (98-214), the
 * radial return `vonmises` (229-252), `grow_damage` (253-258), the
 * acoustic-fluidization update `update_af` (390-410), the implicit
 * fluidization viscosity `implicit_visc` (286-377), the CFL speed
 * `maxspeed` (378-380), the two-stage Runge-Kutta step `step_rk2`
 * (411-425) and the drivers' time loop (e.g. hydro_cpu.cpp:452).  The
 * reference's file-scope settings (hydro_cpu.cpp:15-36, 222-223) become the
 * per-grid eu_params; its global `MAT` becomes the per-grid material.
 *
 * All arithmetic is FP64, in the reference's operation order, with no fused
 * multiply-adds: on ideal-gas grids the results equal the reference's bit for
 * bit; Tillotson grids differ only where the device's exp / pow round
 * differently from the host library's.  The implicit viscosity's
 * conjugate-gradient sums are parallel reductions (fixed order, so runs
 * repeat exactly) instead of the reference's serial sums: its solutions agree
 * with the reference's to the solver's tolerance (relative residual 1e-8).
 *
 * Fields are host arrays of nx*ny*nz doubles, cell (i,j,k) at
 * (i*ny + j)*nz + k, exactly the reference's layout.  Names: r mu mv mw E Sxx
 * Syy Szz Sxy Sxz Syz D af rc vib Pmax (hydro_cpu.cpp:91).
 *
 * Threading: one host thread per grid; calls on a grid are not re-entrant.
 * Each grid owns its CUDA stream and device buffers.  Every call returns
 * SPH_OK (0) or a negative SPH_ERR_* code (deorbit_sph.h); sph_last_error()
 * describes the last failure on the calling thread.  Calls make the grid's
 * device current for their duration and restore the caller's device.
 */
#ifndef DEORBIT_EULER_H
#define DEORBIT_EULER_H

#include <stdint.h>

#include "deorbit_sph.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The file-scope settings of hydro_cpu.cpp:17-36 and 222-223, same meaning
 * and defaults (eu_params_default). */
typedef struct eu_params {
    double gz;        /* GZ: gravity toward -z (m/s^2) */
    double tdec;      /* TDEC: vibration decay time (s); 0 = acoustic fluidization off */
    double eta_af;    /* ETA_AF: fluidization viscosity (Pa s), explicit form */
    double c_act;     /* C_ACT: shock-activation coupling; 0 = off */
    double p_coh;     /* P_COH: cohesion floor of the overburden (Pa) */
    double p_act;     /* P_ACT: shock-sized pressure rise that seeds vibrations (Pa) */
    double rho_cfl;   /* RHO_CFL: near-void density left out of CFL and strength */
    double damp;      /* DAMP: velocity damping per step; 1 = off */
    double rho_vac;   /* RHO_VAC: vacuum-aware face flux threshold; 0 = off */
    double y_i0, mu_i, mu_d, y_d0, y_m, y_bingham; /* ROCK yield constants */
    double c_reg, af_sat; /* C_REG, AF_SAT */
    int32_t axisym;   /* AXISYM: cylindrical (r, z), x -> r, ny = 1 */
    int32_t rock;     /* ROCK: pressure-dependent yield */
    int32_t af_reg;   /* AF_REG: vibration regeneration from plastic work */
    int32_t af_prel;  /* AF_PREL: overburden-relief form */
    int32_t af_seeddp;/* AF_SEEDDP: seed from the acoustic velocity of the jump */
    int32_t reserved;
    double void_amb;  /* VOID_AMB: with a reference state, void cells reset to this
                         density instead of the reference's (0 = the reference's) */
    int32_t void_cons;/* VOID_CONS: with a reference state, a void cell's excess mass
                         first moves to its densest neighbour (serial pass, index order) */
    int32_t visc_imp; /* VISC_IMP: the fluidization viscosity by the implicit solve
                         after the Runge-Kutta average instead of the Lop's explicit term */
} eu_params;

typedef struct eu_grid eu_grid;

/* Arithmetic of the step.  EU_FP64: every operation in FP64, in the
 * reference's order (the reference's CPU solver).  EU_MIXED: the state and its
 * Runge-Kutta updates, the fluidization update and dt in FP64; primitives,
 * face fluxes, the strength sources, the yield surface, damage growth and the
 * CFL speed in FP32 (the arithmetic of the reference's own GPU solver,
 * hydro.metal), at the FP32 rate of the device. */
enum eu_form { EU_FP64 = 0, EU_MIXED = 1 };

/* Reference defaults of every setting (hydro_cpu.cpp:17-36, 222). */
void eu_params_default(eu_params* out);

/* Replaces Grid(X, Y, Z, d) (hydro_cpu.cpp:92): all fields zero, material
 * ideal gas gamma 1.4 (the reference's initial MAT, hydro_cpu.cpp:15). */
int eu_create(int32_t nx, int32_t ny, int32_t nz, double dx, int32_t device, eu_grid** out);
/* eu_create with the Lop's arithmetic chosen (eu_form). */
int eu_create_form(int32_t nx, int32_t ny, int32_t nz, double dx, int32_t device, int32_t form, eu_grid** out);
int eu_destroy(eu_grid* g);
/* Replaces the global MAT (hydro_cpu.cpp:15); only the EOS, G, Y, Emod, wm and
 * wk fields are used (the SPH yield-model fields are ignored). */
int eu_set_material(eu_grid* g, const sph_material* m);
/* Replaces the file-scope settings; rejects axisym with ny != 1. */
int eu_set_params(eu_grid* g, const eu_params* p);
int eu_get_shape(const eu_grid* g, int32_t shape[3], double* dx);

/* set_ref (hydro_cpu.cpp:259-261): the current density and pressure become the
 * hydrostatic reference of the well-balanced z-sweep and gravity source
 * (hydro_cpu.cpp:75-88, 114-119, 139-143) and of the void-cell reset
 * (272-290: near-void cells return to the reference, or VOID_AMB, density).
 * eu_clear_ref drops it; eu_read_ref reads it (either pointer may be NULL). */
int eu_set_ref(eu_grid* g);
int eu_clear_ref(eu_grid* g);
int eu_read_ref(eu_grid* g, double* r0, double* p0, int64_t n);

/* A driver's adjustments applied on the device after every step of eu_step /
 * eu_run, in this order: the lowest pin_floor z-layers return to the
 * reference density at rest with no energy (EU_DRIVER_PIN_STRESS: and no
 * deviatoric stress); columns i >= sponge_from relax toward the reference
 * with weight ((i - sponge_from) / max(1, nx - 1 - sponge_from))^2 (density
 * blended, momentum and energy scaled); EU_DRIVER_VOID_AMBIENT: cells below
 * rho_cfl become ambient gas (0.27 kg/m^3) at rest with no energy and stress;
 * EU_DRIVER_TRACK_PMAX: each cell's Pmax keeps the largest pressure seen.
 * These are the reference drivers' own per-step steps: the crater mode's
 * floor pin and radial sponge (hydro_cpu.cpp:634-637: pin 2, sponge from
 * (int)(0.85 nx)), the substrate gate's pin (855), the collapse demo's held
 * floor (893-894), the Prater run's void cleanup (823-824) and the Pierazzo
 * run's peak-pressure record (769).  The pin and the sponge need a reference
 * state (eu_set_ref); eu_clear_ref turns them off.  0, -1, 0: none (the
 * default). */
enum { EU_DRIVER_PIN_STRESS = 1, EU_DRIVER_VOID_AMBIENT = 2, EU_DRIVER_TRACK_PMAX = 4 };
int eu_set_driver(eu_grid* g, int32_t pin_floor, int32_t sponge_from, int32_t flags);

/* Field i/o of one named field (n = nx*ny*nz doubles), or of several in one
 * call (copies overlap on the grid's stream, one synchronisation). */
int eu_write_field(eu_grid* g, const char* name, const double* host, int64_t n);
int eu_read_field(eu_grid* g, const char* name, double* host, int64_t n);
int eu_write_fields(eu_grid* g, int32_t nfields, const char* const* names, const double* const* host, int64_t n);
int eu_read_fields(eu_grid* g, int32_t nfields, const char* const* names, double* const* host, int64_t n);

/* Lop (hydro_cpu.cpp:98-214) of the current state; eu_read_rhs reads one
 * field of the result (r mu mv mw E Sxx Syy Szz Sxy Sxz Syz D rc vib). */
int eu_lop(eu_grid* g);
int eu_read_rhs(eu_grid* g, const char* name, double* host, int64_t n);
/* vonmises(g, reg) (229-252), grow_damage(g, dt) (253-258), update_af(g, dt)
 * (390-410) applied to the current state. */
int eu_vonmises(eu_grid* g, int32_t reg);
int eu_grow_damage(eu_grid* g, double dt);
int eu_update_af(eu_grid* g, double dt);
/* implicit_visc(g, dt) (286-377) applied to the current state: a no-op unless
 * visc_imp is set and eta_af > 0.  eu_visc_iterations reads the
 * conjugate-gradient iterations taken since the grid was created (the
 * reference's VISC_IT). */
int eu_implicit_visc(eu_grid* g, double dt);
int eu_visc_iterations(eu_grid* g, int64_t* iters);
/* maxspeed(g) (378-380), reduced on the device. */
int eu_maxspeed(eu_grid* g, double* out);
/* Pressure of every cell (Pcell, hydro_cpu.cpp:95) into host[n]. */
int eu_read_pressure(eu_grid* g, double* host, int64_t n);
/* step_rk2(g, dt) (411-425) at a host dt. */
int eu_step(eu_grid* g, double dt);
/* The drivers' loop: dt = cfl*dx/maxspeed, clipped at t_end, until t_end or
 * max_steps steps (max_steps < 0: no limit), with dt, t and the stop test on
 * the device and the steps replayed from a captured CUDA graph.  t starts at
 * the grid's current time (eu_set_time).  *steps / *t receive the steps
 * taken and the time reached (either may be NULL). */
int eu_run(eu_grid* g, double cfl, double t_end, int64_t max_steps, int64_t* steps, double* t);
int eu_set_time(eu_grid* g, double t);
int eu_get_time(eu_grid* g, double* t);

/* Measurement: device events on the grid's stream (slots 0..7), device
 * bytes held, kernels launched so far. */
int eu_synchronize(eu_grid* g);
int eu_event_record(eu_grid* g, int32_t slot);
int eu_event_elapsed(eu_grid* g, int32_t a, int32_t b, double* ms);
int eu_device_bytes(const eu_grid* g, int64_t* bytes);
int eu_launches(const eu_grid* g, int64_t* launches);

#ifdef __cplusplus
}
#endif
#endif
