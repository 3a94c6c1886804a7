/*
 * deorbit_sph.h -- C ABI of the GB300 SPH impact solver (libdeorbit_sph.so).
 *
 * Drop-in boundary for the step loop of the reference's SPH hydrocode:
 * the in-process `struct System` of hydrocodes/sph/sph.hpp:72-380 (init /
 * timestep / step over public particle arrays) and the Tillotson `Material`
 * of hydrocodes/common/eos.hpp:15-113.  Plain C types only: host pointers,
 * sizes and integer status codes; no CUDA or C++ types cross the boundary.
 *
 * Work is organised in IMPACTS: independent particle systems, each with its
 * own domain, parameters, cell grid and time step.  A context holds one or
 * many impacts and advances them together on one GPU (single-instance use =
 * one impact).  Particle fields are read and written in the caller's original
 * particle order.
 *
 * Threading: one host thread per context; calls on a context are not
 * re-entrant.  Each context owns its CUDA stream and device buffers; there is
 * no global mutable state apart from the per-thread error string.
 * Errors: every call returns SPH_OK (0) or a negative SPH_ERR_* code;
 * sph_last_error() describes the last failure on the calling thread.
 */
#ifndef DEORBIT_SPH_H
#define DEORBIT_SPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_ABI_VERSION 1

enum sph_status {
    SPH_OK = 0,
    SPH_ERR_ARG = -1,      /* invalid argument (null pointer, bad id, bad size) */
    SPH_ERR_CUDA = -2,     /* a CUDA call failed (message has the CUDA error)   */
    SPH_ERR_STATE = -3,    /* call not valid in the current state               */
    SPH_ERR_NOMEM = -4,    /* device or host allocation failed                  */
    SPH_ERR_IO = -5,       /* file could not be read / written, short read      */
    SPH_ERR_CAPACITY = -6, /* a fixed capacity (materials, impacts) exceeded    */
    SPH_ERR_TIMEOUT = -7   /* a bounded device wait ran out                     */
};

enum sph_precision {
    SPH_FP64 = 0,  /* plain form: every field and pair interaction in FP64      */
    SPH_MIXED = 1  /* FP32 pairs / EOS / stress, FP64 positions and energies    */
};

enum sph_eos_type { SPH_EOS_IDEAL = 0, SPH_EOS_TILLOTSON = 1 };
enum sph_yield_model { SPH_YIELD_VON_MISES = 0, SPH_YIELD_COLLINS = 1 };
enum sph_flaw_model { SPH_FLAWS_SINGLE = 0, SPH_FLAWS_MULTI = 1 };
enum sph_neighbor_kind { SPH_NBR_DENSITY = 0, SPH_NBR_FORCE = 1 };

/* Replaces `struct Material` (hydrocodes/common/eos.hpp:15-39).  Emod is
 * derived by sph_material_tillotson as 9AG/(3A+G) (eos.hpp:37).  The Collins
 * fields are used only when yield_model == SPH_YIELD_COLLINS (no counterpart in
 * the reference SPH; pressure-dependent yield as in
 * hydrocodes/euler/hydro_cpu.cpp:229-252). */
typedef struct sph_material {
    int32_t type;        /* sph_eos_type */
    int32_t yield_model; /* sph_yield_model */
    double gamma;
    double rho0, a, b, A, B, alpha, beta, u0, uiv, ucv;
    double G, Y, Emod, wm, wk;
    double Y0, mu_i, Ylim, Yd0, mu_d;
} sph_material;

/* Replaces the public parameter members of `System`
 * (hydrocodes/sph/sph.hpp:86-92).  flaw_model selects single-flaw seeding
 * (reference) or Benz-Asphaug multi-flaw damage (extension). */
typedef struct sph_params {
    double eta, h_init, alpha, beta, eps, alpha_u, cfl, eps_as;
    int32_t as_n, damage_on;
    int32_t flaw_model;
    int32_t reserved;
} sph_params;

/* Per-impact status. */
typedef struct sph_impact_info {
    int64_t n;          /* particles */
    int64_t steps;      /* steps taken */
    double t;           /* simulated time */
    double dt;          /* last step size used */
    double h_max;       /* max smoothing length at the last cell build */
    int32_t nc[3];      /* reference cell grid (sph.hpp:147-157) */
    double cw[3];
    int32_t density_rounds; /* adaptive-h rounds in the last step (sph.hpp:185) */
    int32_t initialized;
} sph_impact_info;

/* Conservation record of one impact, from compensated FP64 device sums. */
typedef struct sph_conservation {
    double mass, kinetic, internal, energy;
    double momentum[3];
} sph_conservation;

typedef struct sph_ctx sph_ctx;

/* ---- library -------------------------------------------------------------- */
int sph_abi_version(void);
const char* sph_last_error(void);
/* Fills a Tillotson material exactly like Material::tillotson (eos.hpp:30-39). */
void sph_material_tillotson(sph_material* out, double rho0, double A, double B, double a,
                            double b, double alpha, double beta, double u0, double uiv,
                            double ucv, double G, double Y, double wm, double wk);
/* Ideal gas, Material::ideal (eos.hpp:29). */
void sph_material_ideal(sph_material* out, double gamma);
/* Standard sets of eos.hpp:42-50: 0 iron, 1 basalt, 2 water, 3 aluminum. */
int sph_material_standard(int which, sph_material* out);
/* Reference parameter defaults (sph.hpp:86-92). */
void sph_params_default(sph_params* out);
/* Host-only flaw thresholds of System::seed_damage (sph.hpp:117-128) for n
 * particles with material ids mat[] (no GPU needed). */
int sph_seed_flaws_single(int64_t n, const int32_t* mat, const sph_material* mats, int32_t nmat,
                          double dx, uint32_t seed, double* eps_act);
/* Host-only Benz-Asphaug multi-flaw seeding (extension, no reference
 * counterpart): ptr[n+1] CSR over particles, eps[cap] activation strains,
 * *total the flaw count (SPH_ERR_CAPACITY when cap is too small), eps_act[n]
 * each particle's weakest flaw. */
int sph_seed_flaws_multi_host(int64_t n, const int32_t* mat, const sph_material* mats,
                              int32_t nmat, double dx, uint32_t seed, int64_t* ptr, double* eps,
                              int64_t cap, int64_t* total, double* eps_act);

/* ---- context -------------------------------------------------------------- */
/* Replaces constructing a `System` (sph.hpp:72).  device: CUDA ordinal.  Every
 * call on a context makes the context's device current while it runs and
 * restores the calling thread's previous current device before returning. */
int sph_create(sph_ctx** out, int precision, int device);
int sph_destroy(sph_ctx* ctx);
/* Replaces `materials.push_back(...)` (sph.hpp:82); materials are shared by all
 * impacts of the context.  *id receives the material index. */
int sph_add_material(sph_ctx* ctx, const sph_material* m, int32_t* id);

/* ---- impacts (one System each) ------------------------------------------- */
/* Creates an impact with parameters (sph.hpp:86-92) and domain
 * (set_domain, sph.hpp:96-101; periodic[a] != 0 for a periodic axis). */
int sph_impact_create(sph_ctx* ctx, const sph_params* p, const double dlo[3],
                      const double dhi[3], const int32_t periodic[3], int32_t* impact);
/* Replaces System::set_domain (sph.hpp:96-101) before sph_init. */
int sph_impact_set_domain(sph_ctx* ctx, int32_t impact, const double dlo[3],
                          const double dhi[3], const int32_t periodic[3]);
int sph_impact_set_params(sph_ctx* ctx, int32_t impact, const sph_params* p);
int sph_impact_get_params(sph_ctx* ctx, int32_t impact, sph_params* p);
/* Replaces System::add (sph.hpp:103-111) for n particles at once: hh starts at
 * h_init, derived fields at zero, eps_act 1e30, dscale 1.  mat may be NULL
 * (material 0); fixed may be NULL (none fixed). */
int sph_impact_add_particles(sph_ctx* ctx, int32_t impact, int64_t n, const double* x,
                             const double* y, const double* z, const double* vx,
                             const double* vy, const double* vz, const double* mass,
                             const double* u, const int32_t* mat, const uint8_t* fixed);
/* Replaces System::seed_damage (sph.hpp:117-128): one Weibull flaw per brittle
 * particle from mt19937(seed), eps = (U(1e-9,1] / (k dx^3))^(1/m). */
int sph_impact_seed_damage(sph_ctx* ctx, int32_t impact, double dx, uint32_t seed);
/* Extension (no reference counterpart): Benz & Asphaug (1995) multi-flaw
 * seeding, ceil(N ln N) flaws per brittle material; sets flaw_model MULTI.
 * *nflaws (may be NULL) receives the total. */
int sph_impact_seed_flaws_multi(sph_ctx* ctx, int32_t impact, double dx, uint32_t seed,
                                int64_t* nflaws);
/* Extension: per-particle reference smoothing length (graded lattices). */
int sph_impact_set_h0(sph_ctx* ctx, int32_t impact, const double* h0);
/* Batched runs stop advancing an impact once it has taken `steps` steps in
 * total (0: no limit). */
int sph_impact_set_step_limit(sph_ctx* ctx, int32_t impact, int64_t steps);
/* Releases an impact's particles and slot (serving). */
int sph_impact_remove(sph_ctx* ctx, int32_t impact);
int sph_impact_count(sph_ctx* ctx, int32_t* count);
int sph_impact_info_get(sph_ctx* ctx, int32_t impact, sph_impact_info* info);

/* ---- stepping (System::init / timestep / step) ---------------------------- */
/* Replaces System::init (sph.hpp:379) for every impact not yet initialised. */
int sph_init(sph_ctx* ctx);
/* Replaces System::timestep (sph.hpp:350-355): CFL step of one impact. */
int sph_timestep(sph_ctx* ctx, int32_t impact, double* dt);
/* Replaces System::step(dt) (sph.hpp:357-377): one KDK step of EVERY impact
 * with the caller's dt. */
int sph_step(sph_ctx* ctx, double dt);
/* Batched run: nsteps KDK steps in which each impact uses its own CFL dt
 * (device-side, as run_ic.cpp:178-180), clipped at its t_end when t_end > 0.
 * Impacts that reached t_end or their step limit stop advancing.  Unless the
 * "graphs" option is 0, steps run as a captured CUDA graph of two
 * device-controlled steps (no host round trips inside). */
int sph_run(sph_ctx* ctx, int32_t nsteps, double t_end);
/* Individual phases (for parity checks, as cpu_dump.cpp:171 uses them). */
int sph_compute_density_h(sph_ctx* ctx, int32_t iters);   /* sph.hpp:184-208 */
int sph_compute_forces(sph_ctx* ctx);                     /* sph.hpp:260-318 */
int sph_synchronize(sph_ctx* ctx);

/* ---- particle fields, original order --------------------------------------
 * name: x y z vx vy vz ax ay az mass rho u dudt P cs csig hh eps_work D eps_act
 * sigmax Pf Rart dscale Sxx Syy Szz Sxy Sxz Syz dSxx dSyy dSzz dSxy dSxz dSyz h0
 * (replaces reading / writing System's public vectors, sph.hpp:73-81). */
int sph_read_field(sph_ctx* ctx, int32_t impact, const char* name, double* out);
int sph_write_field(sph_ctx* ctx, int32_t impact, const char* name, const double* in);
/* Several fields in one call with one synchronisation (page-locked caller
 * buffers transfer at link speed): out[f] / in[f] hold n doubles of field
 * names[f], original order. */
int sph_read_fields(sph_ctx* ctx, int32_t impact, int32_t nfields, const char* const* names,
                    double* const* outs);
int sph_write_fields(sph_ctx* ctx, int32_t impact, int32_t nfields, const char* const* names,
                     const double* const* ins);
/* One step with the state crossing the boundary inside it, for callers that
 * own the particle state on the host (run_ic.cpp:177-190: a loop over
 * System::timestep / step that reads the public vectors between steps).
 * The result equals, bit for bit, sph_write_fields(ins); dt =
 * sph_timestep(impact) when dt < 0 (else the given dt >= 0); sph_step(dt);
 * sph_read_fields(outs) -- in one call whose host copies overlap the step's
 * kernels (u, D, S, the old derivatives and eps_act go up while the sort,
 * list and density passes run; x, y, z, mass, h0 and hh come down while the
 * force pass runs).  Writes the dt used
 * to *dt_used when dt_used is not null.  Every input is read before any
 * output is written, so input and output buffers may be the same memory;
 * the caller's buffers may be reused on return. */
int sph_step_fields(sph_ctx* ctx, int32_t impact, double dt, int32_t nin, const char* const* in_names,
                    const double* const* ins, int32_t nout, const char* const* out_names, double* const* outs,
                    double* dt_used);
int sph_read_mat(sph_ctx* ctx, int32_t impact, int32_t* out);
int sph_read_fixed(sph_ctx* ctx, int32_t impact, uint8_t* out);
int sph_write_fixed(sph_ctx* ctx, int32_t impact, const uint8_t* in);

/* ---- diagnostics ----------------------------------------------------------- */
int sph_conservation_get(sph_ctx* ctx, int32_t impact, sph_conservation* out);
/* Projectile diagnostics reduced on the device over the particles with
 * mat_lo <= material id <= mat_hi: what gpu_ic's progress line
 * (gpu_ic.cpp:112-117: centroid, |v|, vz, melt=%, umax) and the campaign's
 * regime classifier (boundary_daemon.py:181-212: bulk velocity, dispersion,
 * melt fraction) compute from host copies of every particle. */
typedef struct sph_diagnostics {
    int64_t count;       /* selected particles */
    int64_t melted;      /* of those with u > u_melt */
    double mean_pos[3];
    double mean_vel[3];  /* bulk velocity (unweighted mean) */
    double mean_speed;   /* mean |v| */
    double dispersion;   /* sqrt(mean |v - bulk|^2) */
    double u_max;
} sph_diagnostics;
int sph_impact_diagnostics(sph_ctx* ctx, int32_t impact, int32_t mat_lo, int32_t mat_hi, double u_melt,
                           sph_diagnostics* out);
/* Tillotson / ideal EOS on the device in the context precision
 * (eos.hpp:65-113): n (rho, u) pairs of material mat -> P, cs. */
int sph_eos_eval(sph_ctx* ctx, int32_t mat, int64_t n, const double* rho, const double* u,
                 double* P, double* cs);

/* ---- parity hooks: integer outputs of the last cell build ------------------
 * Reference cell grid (sph.hpp:147-162) of one impact: nc, cw, and its cell
 * list as CSR in original particle ids, each cell ascending (bit-exact with
 * System::cells).  start has nc0*nc1*nc2+1 entries, ids n entries. */
int sph_debug_ref_cells(sph_ctx* ctx, int32_t impact, int32_t nc[3], double cw[3],
                        int32_t* start, int64_t start_len, int32_t* ids);
/* Neighbour sets of the current state as System::for_neighbors sees them
 * (sph.hpp:163-182): kind SPH_NBR_DENSITY = {j : r < 2 h_i} (self included),
 * SPH_NBR_FORCE = {j != i : r < 2 hbar, r != 0}.  counts[n] per particle (original
 * order), ids: each set ascending in original ids, concatenated in original
 * particle order.  *total receives the number of entries; returns
 * SPH_ERR_CAPACITY when cap is too small. */
int sph_debug_neighbors(sph_ctx* ctx, int32_t impact, int32_t kind, int32_t* counts,
                        int32_t* ids, int64_t cap, int64_t* total);
/* Multi-flaw activation strains as the device holds them (extension; the
 * counterpart of the seeded flaw arrays): ptr[n+1] CSR in original particle
 * order, eps[cap] (NULL: sizes only; the engine's precision, widened to
 * double), *total the flaw count.  All-zero ptr for single-flaw impacts. */
int sph_debug_flaws(sph_ctx* ctx, int32_t impact, int64_t* ptr, double* eps, int64_t cap,
                    int64_t* total);

/* ---- primitives on caller-owned device memory ------------------------------
 * Stable radix cell sort (the cell-list build of sph.hpp:147-162 as a
 * device primitive): keys[n] (device, uint32 cell ids in [0, ncells)) ->
 * perm[n] (device): particle indices ordered by (cell, index); cell_start
 * [ncells+1] (device): first sorted position of each cell, cell_start[ncells]
 * = n.  stream is a cudaStream_t (NULL: the legacy default stream); the call
 * returns when the result is complete.  Scratch is taken with
 * cudaMallocAsync on the stream and released before returning.
 * SPH_ERR_ARG when a key is out of range (outputs then undefined). */
int sph_cell_sort(const uint32_t* keys, int64_t n, int64_t ncells, int32_t* perm,
                  int32_t* cell_start, void* stream);
/* The same cell sort without any device allocation (no counterpart in the
 * reference).  For callers that must not allocate device memory once they are
 * running: hosts with a fixed device-memory budget or their own pool allocator
 * that accounts for every byte, and latency-critical loops that cannot take an
 * allocation's cost or implicit synchronization.  They pass inputs and outputs
 * as above; the scratch is a 3.5 MiB array inside the library that every GPU
 * loading it reserves until the process exits.  Limits: n <= 262144 keys and
 * ncells <= 16777216 per call (SPH_ERR_CAPACITY beyond).  The first call on a
 * device looks up the array's device address (once per device, with that
 * device current, cached for the life of the process: the runtime's primary
 * context is assumed, so the address is not valid after cudaDeviceReset).
 * Every call waits for its result on the host, so it cannot be captured into a
 * CUDA graph: on a stream under capture it returns SPH_ERR_STATE without
 * touching the stream.  All calls share the one array, so calls that overlap
 * on the GPU (other streams or threads) race; serialize them. */
int sph_cell_sort_static(const uint32_t* keys, int64_t n, int64_t ncells, int32_t* perm,
                         int32_t* cell_start, void* stream);

/* ---- serving: continuous batching of impact runs ---------------------------
 * Replaces the campaign's one-process-per-impact loop (boundary_daemon.py:
 * 215-255 runs gpu_ic once per impact) with one resident server.  A server
 * keeps one context busy with a stream of requests (one impact each): a
 * request is admitted once it has arrived and its particles fit the device-
 * memory budget beside the resident impacts (the engine's own allocations and
 * its per-particle footprint at the current neighbour-list capacity),
 * initialised in place while the others keep their state, advanced with them
 * in chunks of device-controlled steps (own CFL dt and step limit each) and
 * retired when it has taken its steps: its fields are copied to host memory and
 * its slot and memory released.  Flaw seeding of queued requests runs on a
 * worker thread of the server while the GPU works.  sph_serve_poll and every
 * other call that touches the context belong to one thread (the serving
 * thread); sph_serve_submit may be called from any thread.  A request's
 * results do not depend on what else is resident. */
typedef struct sph_server sph_server;
enum sph_serve_flaws { SPH_SERVE_FLAWS_NONE = 0, SPH_SERVE_FLAWS_SINGLE = 1, SPH_SERVE_FLAWS_MULTI = 2 };
enum sph_serve_state { SPH_SERVE_QUEUED = 0, SPH_SERVE_RESIDENT = 1, SPH_SERVE_DONE = 2, SPH_SERVE_FAILED = 3 };
typedef struct sph_request {
    const sph_params* params;   /* as sph_impact_create */
    double lo[3], hi[3];        /* domain */
    int32_t periodic[3];
    int32_t flaws;              /* sph_serve_flaws: seeding as sph_impact_seed_damage /
                                   sph_impact_seed_flaws_multi with flaw_dx, flaw_seed */
    int64_t n;                  /* particles, arrays as sph_impact_add_particles */
    const double *x, *y, *z, *vx, *vy, *vz, *mass, *u;
    const int32_t* mat;         /* material ids of the server's context (NULL: 0) */
    const uint8_t* fixed;       /* NULL: none fixed */
    const double* h0;           /* NULL: h_init everywhere (sph_impact_set_h0) */
    double flaw_dx;
    uint32_t flaw_seed;
    int32_t reserved;
    int64_t steps;              /* KDK steps to take */
    double arrival;             /* seconds on the server clock; < 0: now */
} sph_request;
typedef struct sph_serve_record {
    int64_t n, steps;
    int32_t state;              /* sph_serve_state */
    int32_t impact;             /* impact id while resident */
    double arrival, admitted, finished;   /* server clock, seconds (-1: not yet) */
} sph_serve_record;
typedef struct sph_serve_summary {
    int64_t done, queued, resident;
    double p50_latency_s, p99_latency_s, mean_latency_s;   /* arrival -> results in host memory */
    double particle_steps;
    double throughput;          /* particle-steps / (last finish - first arrival) */
    double busy_throughput;     /* particle-steps / time spent advancing */
    double busy_s;
    double peak_device_bytes;   /* largest engine allocation seen after an admission */
    double admit_wait_s;        /* admission blocked on requests still being seeded */
    double host_s;              /* admission, initialisation and retirement between rounds */
} sph_serve_summary;
/* fields: comma-separated field names kept for each finished request (NULL:
 * x,y,z,vx,vy,vz,u,rho,P,D); the server clock starts here. */
int sph_serve_create(sph_ctx* ctx, double hbm_budget_bytes, int32_t chunk, const char* fields,
                     sph_server** out);
/* Stops the worker and removes the impacts still resident (the context stays). */
int sph_serve_destroy(sph_server* srv);
int sph_serve_now(sph_server* srv, double* t);
/* Queues a copy of the request; *id receives its id. */
int sph_serve_submit(sph_server* srv, const sph_request* req, int64_t* id);
/* One serving round: admit, advance the residents by up to `chunk` steps,
 * retire the finished ones (their ids in done_ids[cap], the count in *ndone).
 * With nothing resident it waits up to max_wait_s for the next arrival. */
int sph_serve_poll(sph_server* srv, double max_wait_s, int64_t* done_ids, int32_t cap, int32_t* ndone);
int sph_serve_request_info(sph_server* srv, int64_t id, sph_serve_record* out);
/* A finished request's field (n doubles, original particle order). */
int sph_serve_result(sph_server* srv, int64_t id, const char* field, double* out);
/* Frees a finished request's results. */
int sph_serve_release(sph_server* srv, int64_t id);
int sph_serve_stats(sph_server* srv, sph_serve_summary* out);

/* ---- files (formats of run_ic.cpp / gpu_ic.cpp) ----------------------------
 * IC: f8 header [xlo xhi ylo yhi zlo zhi n], then n x [x y z vx vy vz mass u mat
 * fixed] (run_ic.cpp:4-6).  Creates an impact with the given parameters and
 * the IC's domain; *impact receives its id. */
int sph_load_ic(sph_ctx* ctx, const char* path, const sph_params* p, int32_t* impact);
/* The campaign's grazing-impact IC generated in place (no reference C
 * counterpart: restates boundary_daemon.py:119-158, build_grazing_ic, the Python
 * builder of the IC files gpu_ic reads): a target half-space lattice of spacing
 * dx = D / (2 cppr) with frozen walls, and an impactor lattice sphere of diameter
 * D moving at theta below horizontal.  Same particles, order and domain as the
 * reference builder's file; the target lattice (all but a few thousand
 * particles) is generated on the device. */
typedef struct sph_grazing_spec {
    double theta_deg, v, D;
    double rho_imp;         /* impactor density (reference: 7800) */
    double rho_target;      /* target lattice density (reference: 2700) */
    double x_impact_frac;   /* NaN: the campaign geometry (boundary_daemon.py:150) */
    double start_h;         /* NaN: released at a + 3 dx */
    int32_t cppr;           /* lattice cells per impactor radius */
    int32_t tgt_mat, imp_mat;  /* material ids of this context */
    int32_t reserved;
} sph_grazing_spec;
void sph_grazing_spec_default(sph_grazing_spec* s);
/* New impact holding the generated IC; *dx_out and *n_out (may be NULL) get the
 * lattice spacing and the particle count. */
int sph_impact_create_grazing(sph_ctx* ctx, const sph_params* p, const sph_grazing_spec* s,
                              int32_t* impact, double* dx_out, int64_t* n_out);
/* Snapshot: int64 n, then n x f8 [x y z vx vy vz u rho h mat] (run_ic.cpp:15-30). */
int sph_write_snapshot(sph_ctx* ctx, int32_t impact, const char* path);
/* Lossless checkpoint, write-then-rename: f8 header [xlo xhi ylo yhi zlo zhi n t dx]
 * then n x 18 f8 [x y z vx vy vz mass u mat fixed D eps_act Sxx Sxy Sxz Syy Syz Szz]
 * (run_ic.cpp:32-55). */
int sph_write_checkpoint(sph_ctx* ctx, int32_t impact, const char* path, double dx);
/* Restart from a checkpoint (run_ic.cpp:76-102): new impact, t and D / eps_act /
 * S restored; *dx_out (may be NULL) receives dx. */
int sph_load_checkpoint(sph_ctx* ctx, const char* path, const sph_params* p, int32_t* impact,
                        double* dx_out);

/* ---- tuning ---------------------------------------------------------------- */
/* Launch shape of the neighbour kernels and the traversal cell width as a
 * multiple of h_init.  Zero keeps the current value. */
int sph_set_tuning(sph_ctx* ctx, int32_t block_threads, double cell_factor);
/* Named engine options: "list_mode" (neighbour-list build: 0 thread per
 * particle, 1 warp per column run, 2 warp per particle), "cell_factor",
 * "cell_factor_z" (traversal cell height over width, (0, 4]; like
 * "cell_factor", set before particles are committed), "block", "slack"
 * (neighbour-list radius slack), "graphs" (1: sph_step and sph_run replay
 * captured CUDA graphs), "force_staging" (mixed form: neighbour records of
 * the force pass staged in shared memory; 0 off, 22 / 23 / 42 bulk copies of
 * 2 or 4 entries x 2 or 3 stages, 122 / 142 16-byte async copies),
 * "host_direct" (1: field reads and writes reach device-accessible host
 * buffers directly over the CPU-GPU link; 0: device staging copies);
 * read-only "list_capacity" (entries per particle), "list_entries" (entries
 * of the current lists, own plus reverse), "device_bytes" (the context's
 * device allocations), "bytes_per_particle" (device bytes per particle of
 * capacity at the current list capacity) and "pageable_access" (1 where the
 * device reads pageable host memory). */
int sph_set_option(sph_ctx* ctx, const char* key, double value);
int sph_get_option(sph_ctx* ctx, const char* key, double* value);
/* Number of kernel launches issued by this context since creation. */
int sph_launch_count(sph_ctx* ctx, int64_t* launches);
/* CUDA-event phase times of the last step in ms: [kick+sort, density, eos,
 * force, damage+finish+dt] (mirrors gpu_ic's PROFILE line, gpu_ic.cpp:147). */
int sph_phase_times(sph_ctx* ctx, double ms[5]);
/* Opt-in CUDA-event timing of the phases and kernel classes (off by default;
 * adds one host wait per step while on). */
int sph_set_profiling(sph_ctx* ctx, int32_t on);
/* Kernel classes for sph_kernel_stats. */
enum sph_kernel_class {
    SPH_K_KICK = 0, SPH_K_SORT, SPH_K_GRID, SPH_K_LIST_DENSITY, SPH_K_DENSITY, SPH_K_EOS,
    SPH_K_LIST_FORCE, SPH_K_FORCE, SPH_K_DAMAGE, SPH_K_FINISH, SPH_K_DT, SPH_K_OTHER, SPH_K_COUNT
};
/* Accumulated device time (CUDA events on the context stream) and launch count
 * of one kernel class while profiling was on. */
int sph_kernel_stats(sph_ctx* ctx, int32_t kernel_class, double* total_ms, int64_t* launches);
int sph_kernel_stats_reset(sph_ctx* ctx);
/* CUDA events on the context's stream, slots 0..15, for device-side timing of
 * any span of calls; elapsed waits for the later event. */
int sph_event_record(sph_ctx* ctx, int32_t slot);
int sph_event_elapsed(sph_ctx* ctx, int32_t slot_a, int32_t slot_b, double* ms);

#ifdef __cplusplus
}
#endif
#endif
