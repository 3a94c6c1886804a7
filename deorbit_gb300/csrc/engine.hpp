// engine.hpp -- precision-independent interface of the SPH engine behind the C ABI.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/deorbit_sph.h"

namespace dsph {

struct SphError : std::runtime_error {
    int code;
    SphError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Layout of the campaign's grazing IC (boundary_daemon.py:119-158): the
// target lattice is the product of three coordinate ranges (the reference's
// accumulated ranges, computed on the host), generated on the device at
// commit; the impactor sphere's particles are host-built in the reference's
// order.  Built by grazing_layout() (capi.cu).
struct GrazingLayout {
    std::vector<double> xs, ys, zs;
    double wall = 0, m_target = 0;
    int32_t tgt_mat = 0, imp_mat = 1;
    std::vector<double> px, py, pz;   // impactor particles
    double vx = 0, vz = 0, m_imp = 0;
    double dlo[3] = {0, 0, 0}, dhi[3] = {0, 0, 0}, dx = 0;
    int64_t n_slab() const { return (int64_t)xs.size() * (int64_t)ys.size() * (int64_t)zs.size(); }
    int64_t n() const { return n_slab() + (int64_t)px.size(); }
};

class EngineBase {
public:
    virtual ~EngineBase() = default;
    virtual int precision() const = 0;
    virtual int add_material(const sph_material& m) = 0;
    virtual int impact_create(const sph_params& p, const double dlo[3], const double dhi[3],
                              const int32_t per[3]) = 0;
    // impact whose particles are generated at commit (grazing IC)
    virtual int impact_create_generated(const sph_params& p, std::shared_ptr<const GrazingLayout> L) = 0;
    virtual void impact_set_domain(int b, const double dlo[3], const double dhi[3],
                                   const int32_t per[3]) = 0;
    virtual void impact_set_params(int b, const sph_params& p) = 0;
    virtual sph_params impact_get_params(int b) = 0;
    virtual void impact_add_particles(int b, int64_t n, const double* x, const double* y,
                                      const double* z, const double* vx, const double* vy,
                                      const double* vz, const double* mass, const double* u,
                                      const int32_t* mat, const uint8_t* fixed) = 0;
    virtual void impact_seed_damage(int b, double dx, uint32_t seed) = 0;
    virtual int64_t impact_seed_flaws_multi(int b, double dx, uint32_t seed) = 0;
    virtual void impact_set_h0(int b, const double* h0) = 0;
    // Flaws seeded on the host beforehand, set before the impact is committed:
    // eps_act per particle and, when ptr is non-null, the multi-flaw CSR
    // (ptr[n+1], eps[nflaws]) with flaw_model MULTI.
    virtual void impact_set_flaws(int b, const double* eps_act, const int64_t* ptr, const double* eps,
                                  int64_t nflaws) = 0;
    virtual std::vector<sph_material> materials() = 0;
    // Bytes of the engine's device allocations now, and as predicted after
    // committing n more particles (capacity growth at the current list capacity).
    virtual int64_t device_bytes() = 0;
    virtual int64_t device_bytes_after_adding(int64_t n) = 0;
    virtual void impact_set_time(int b, double t) = 0;
    virtual void impact_set_step_limit(int b, int64_t steps) = 0;
    virtual void impact_remove(int b) = 0;
    virtual int impact_count() = 0;
    virtual sph_impact_info impact_info(int b) = 0;
    virtual void get_domain(int b, double dlo[3], double dhi[3], int32_t per[3]) = 0;
    virtual void init() = 0;
    virtual double timestep(int b) = 0;
    virtual void step(double dt) = 0;
    virtual void run(int nsteps, double t_end) = 0;
    virtual void compute_density_h(int iters) = 0;
    virtual void compute_forces() = 0;
    virtual void synchronize() = 0;
    virtual int64_t impact_n(int b) = 0;
    // Steps the impact has taken (host copy, current after every run / step;
    // no device round trip, unlike impact_info).
    virtual int64_t impact_steps(int b) = 0;
    virtual void read_field(int b, const char* name, double* out) = 0;
    virtual void write_field(int b, const char* name, const double* in) = 0;
    virtual void read_fields(int b, int nf, const char* const* names, double* const* outs) = 0;
    virtual void write_fields(int b, int nf, const char* const* names, const double* const* ins) = 0;
    virtual double step_fields(int b, double dt, int nin, const char* const* in_names, const double* const* ins,
                               int nout, const char* const* out_names, double* const* outs) = 0;
    virtual void read_mat(int b, int32_t* out) = 0;
    virtual void read_fixed(int b, uint8_t* out) = 0;
    virtual void write_fixed(int b, const uint8_t* in) = 0;
    virtual sph_conservation conservation(int b) = 0;
    virtual void diagnostics(int b, int mat_lo, int mat_hi, double u_melt, double out[11]) = 0;
    virtual void eos_eval(int mat, int64_t n, const double* rho, const double* u, double* P,
                          double* cs) = 0;
    virtual void debug_ref_cells(int b, int32_t nc[3], double cw[3], int32_t* start,
                                 int64_t start_len, int32_t* ids) = 0;
    virtual int64_t debug_neighbors(int b, int kind, int32_t* counts, int32_t* ids,
                                    int64_t cap) = 0;
    virtual int64_t debug_flaws(int b, int64_t* ptr, double* eps, int64_t cap) = 0;
    virtual void set_tuning(int block, double cell_factor) = 0;
    virtual void set_option(const char* key, double value) = 0;
    virtual double get_option(const char* key) = 0;
    virtual int64_t launches() = 0;
    virtual void phase_times(double ms[5]) = 0;
    virtual void set_profiling(int on) = 0;
    virtual void kernel_stats(int cls, double* ms, int64_t* n) = 0;
    virtual void kernel_stats_reset() = 0;
    virtual void event_record(int slot) = 0;
    virtual double event_elapsed(int a, int b) = 0;
};

}  // namespace dsph

// The opaque context of the C ABI.
struct sph_ctx {
    std::unique_ptr<dsph::EngineBase> eng;
    int device = 0;
};

namespace dsph {

std::unique_ptr<EngineBase> make_engine_fp64(int device);
std::unique_ptr<EngineBase> make_engine_mixed(int device);

// Host-side seeding shared by the engine and its tests (bit-compatible with the
// C++ standard library's mt19937 + uniform_real_distribution<double>).
void seed_single_flaws(int64_t n, const int32_t* mat, const sph_material* mats, int nmat,
                       double dx, uint32_t seed, double* eps_act);
// Benz & Asphaug multi-flaw seeding: fills ptr (n+1) and eps (returned count).
int64_t seed_multi_flaws(int64_t n, const int32_t* mat, const sph_material* mats, int nmat,
                         double dx, uint32_t seed, int64_t* ptr, double** eps_out,
                         double* eps_act);

}  // namespace dsph
