// capi.cu -- the C ABI of include/deorbit_sph.h over the engine, host-side
// flaw seeding and the IC / snapshot / checkpoint file formats.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "engine.hpp"

using dsph::EngineBase;
using dsph::SphError;


namespace {

thread_local std::string g_err;

}  // namespace

namespace dsph {
void set_error_message(const std::string& m) { g_err = m; }
}  // namespace dsph

namespace {

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

template <class F>
int guard(F&& f) {
    try {
        f();
        return SPH_OK;
    } catch (const SphError& e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc&) {
        return fail(SPH_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(SPH_ERR_STATE, e.what());
    }
}

EngineBase& E(sph_ctx* c) {
    if (!c || !c->eng) throw SphError(SPH_ERR_ARG, "null context");
    return *c->eng;
}

void need(const void* p, const char* what) {
    if (!p) throw SphError(SPH_ERR_ARG, std::string("null pointer: ") + what);
}

}  // namespace

namespace dsph {

// sph.hpp:117-128 with the standard library's generator and distribution.
void seed_single_flaws(int64_t n, const int32_t* mat, const sph_material* mats, int nmat,
                       double dx, uint32_t seed, double* eps_act) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> U(1e-9, 1.0);
    double V = dx * dx * dx;
    for (int64_t i = 0; i < n; i++) {
        int m = mat[i];
        if (m < 0 || m >= nmat) throw SphError(SPH_ERR_ARG, "material id out of range");
        const sph_material& M = mats[m];
        if (M.wk > 0 && M.wm > 0)
            eps_act[i] = std::pow(U(rng) / (M.wk * V), 1.0 / M.wm);
        else
            eps_act[i] = 1e30;
    }
}

// Benz & Asphaug (1995) multi-flaw seeding (same procedure as the oracle's
// extension): per brittle material, ceil(N ln N) flaws with eps_j =
// (j / (k V_tot))^(1/m) on uniformly drawn particles, then one more for every
// particle left without a flaw.
int64_t seed_multi_flaws(int64_t n, const int32_t* mat, const sph_material* mats, int nmat,
                         double dx, uint32_t seed, int64_t* ptr, double** eps_out,
                         double* eps_act) {
    std::mt19937 rng(seed);
    std::vector<int32_t> cnt(n, 0);
    std::vector<int64_t> list;
    std::vector<std::pair<int64_t, double>> flaws;
    for (int mi = 0; mi < nmat; mi++) {
        const sph_material& M = mats[mi];
        if (!(M.wk > 0 && M.wm > 0)) continue;
        list.clear();
        for (int64_t i = 0; i < n; i++)
            if (mat[i] == mi) list.push_back(i);
        int64_t nb = (int64_t)list.size();
        if (nb == 0) continue;
        double Vtot = (double)nb * dx * dx * dx;
        int64_t Nf = (int64_t)std::ceil((double)nb * std::log((double)nb > 1.0 ? (double)nb : 2.0));
        int64_t j = 0;
        for (; j < Nf; j++) {
            uint32_t r = rng();
            int64_t owner = list[(int64_t)r % nb];
            flaws.push_back({owner, std::pow((double)(j + 1) / (M.wk * Vtot), 1.0 / M.wm)});
            cnt[owner]++;
        }
        for (int64_t q = 0; q < nb; q++) {
            int64_t i = list[q];
            if (cnt[i] > 0) continue;
            flaws.push_back({i, std::pow((double)(j + 1) / (M.wk * Vtot), 1.0 / M.wm)});
            j++;
            cnt[i]++;
        }
    }
    ptr[0] = 0;
    for (int64_t i = 0; i < n; i++) ptr[i + 1] = ptr[i] + cnt[i];
    int64_t nf = (int64_t)flaws.size();
    double* eps = (double*)malloc(sizeof(double) * (size_t)(nf > 0 ? nf : 1));
    std::vector<int64_t> fill(ptr, ptr + n + 1);
    for (auto& f : flaws) eps[fill[f.first]++] = f.second;
    for (int64_t i = 0; i < n; i++) eps_act[i] = cnt[i] > 0 ? eps[ptr[i]] : 1e30;
    *eps_out = eps;
    return nf;
}

}  // namespace dsph

extern "C" {

int sph_abi_version(void) { return SPH_ABI_VERSION; }
const char* sph_last_error(void) { return g_err.c_str(); }

void sph_material_tillotson(sph_material* m, double rho0, double A, double B, double a, double b,
                            double alpha, double beta, double u0, double uiv, double ucv,
                            double G, double Y, double wm, double wk) {
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    m->type = SPH_EOS_TILLOTSON;
    m->yield_model = SPH_YIELD_VON_MISES;
    m->gamma = 1.4;
    m->rho0 = rho0; m->A = A; m->B = B; m->a = a; m->b = b;
    m->alpha = alpha; m->beta = beta; m->u0 = u0; m->uiv = uiv; m->ucv = ucv;
    m->G = G; m->Y = Y; m->wm = wm; m->wk = wk;
    m->Emod = (G > 0 ? 9.0 * A * G / (3.0 * A + G) : 0.0);
}

void sph_material_ideal(sph_material* m, double gamma) {
    if (!m) return;
    std::memset(m, 0, sizeof(*m));
    m->type = SPH_EOS_IDEAL;
    m->gamma = gamma;
}

int sph_material_standard(int which, sph_material* m) {
    if (!m) return fail(SPH_ERR_ARG, "null material");
    switch (which) {  // eos.hpp:42-50
        case 0: sph_material_tillotson(m, 7800, 1.28e11, 1.05e11, 0.5, 1.5, 5, 5, 9.5e6, 2.4e6, 8.67e6, 7.75e10, 1.0e9, 0, 0); break;
        case 1: sph_material_tillotson(m, 2700, 2.67e10, 2.67e10, 0.5, 1.5, 5, 5, 4.87e8, 4.72e6, 1.82e7, 2.27e10, 3.5e8, 16.0, 1.0e61); break;
        case 2: sph_material_tillotson(m, 998, 2.2e9, 9.94e9, 0.7, 0.15, 10, 5, 7.0e6, 4.19e5, 2.69e6, 0.0, 0.0, 0, 0); break;
        case 3: sph_material_tillotson(m, 2700, 7.52e10, 6.5e10, 0.5, 1.63, 5, 5, 5.0e6, 3.0e6, 1.39e7, 0.0, 0.0, 0, 0); break;
        default: return fail(SPH_ERR_ARG, "unknown standard material");
    }
    return SPH_OK;
}

void sph_params_default(sph_params* p) {  // sph.hpp:86-92
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->eta = 1.3;
    p->h_init = 0.01;
    p->alpha = 1.0;
    p->beta = 2.0;
    p->eps = 0.01;
    p->alpha_u = 0.0;
    p->cfl = 0.2;
    p->eps_as = 0.0;
    p->as_n = 4;
    p->damage_on = 0;
    p->flaw_model = SPH_FLAWS_SINGLE;
}

int sph_seed_flaws_single(int64_t n, const int32_t* mat, const sph_material* mats, int32_t nmat,
                          double dx, uint32_t seed, double* eps_act) {
    return guard([&] {
        if (n < 0) throw SphError(SPH_ERR_ARG, "n < 0");
        if (n > 0) { need(mat, "mat"); need(mats, "mats"); need(eps_act, "eps_act"); }
        dsph::seed_single_flaws(n, mat, mats, nmat, dx, seed, eps_act);
    });
}

int sph_seed_flaws_multi_host(int64_t n, const int32_t* mat, const sph_material* mats,
                              int32_t nmat, double dx, uint32_t seed, int64_t* ptr, double* eps,
                              int64_t cap, int64_t* total, double* eps_act) {
    return guard([&] {
        if (n < 0) throw SphError(SPH_ERR_ARG, "n < 0");
        need(ptr, "ptr");
        need(total, "total");
        if (n > 0) { need(mat, "mat"); need(mats, "mats"); need(eps_act, "eps_act"); }
        for (int64_t i = 0; i < n; i++)
            if (mat[i] < 0 || mat[i] >= nmat) throw SphError(SPH_ERR_ARG, "material id out of range");
        double* fe = nullptr;
        int64_t nf = dsph::seed_multi_flaws(n, mat, mats, nmat, dx, seed, ptr, &fe, eps_act);
        *total = nf;
        if (nf > cap || (nf > 0 && !eps)) {
            free(fe);
            throw SphError(SPH_ERR_CAPACITY, "eps buffer too small");
        }
        std::memcpy(eps, fe, sizeof(double) * (size_t)nf);
        free(fe);
    });
}

namespace {
// Makes `dev` current for the enclosing scope and restores the thread's
// previous current device when the scope ends.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            prev = -1;
        }
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
        cudaGetLastError();
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};
}  // namespace

int sph_create(sph_ctx** out, int precision, int device) {
    return guard([&] {
        need(out, "out");
        *out = nullptr;
        int ndev = 0;
        cudaError_t e = cudaGetDeviceCount(&ndev);
        if (e != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw SphError(SPH_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
        }
        if (device < 0 || device >= ndev) throw SphError(SPH_ERR_ARG, "bad device ordinal");
        DeviceGuard dg(device);
        auto c = std::make_unique<sph_ctx>();
        c->device = device;
        if (precision == SPH_FP64) c->eng = dsph::make_engine_fp64(device);
        else if (precision == SPH_MIXED) c->eng = dsph::make_engine_mixed(device);
        else throw SphError(SPH_ERR_ARG, "unknown precision");
        *out = c.release();
    });
}

int sph_destroy(sph_ctx* ctx) {
    return guard([&] {
        if (!ctx) return;
        DeviceGuard dg(ctx->device);
        delete ctx;
    });
}

// Every call on a context runs with the context's device current and gives
// the calling thread its previous current device back on return (also on
// errors), so mixing contexts and caller-owned buffers on other devices is safe.
#define CTX_SET() DeviceGuard dsph_device_guard_(ctx ? ctx->device : 0)

int sph_add_material(sph_ctx* ctx, const sph_material* m, int32_t* id) {
    return guard([&] {
        need(m, "material");
        CTX_SET();
        int i = E(ctx).add_material(*m);
        if (id) *id = i;
    });
}

int sph_impact_create(sph_ctx* ctx, const sph_params* p, const double dlo[3], const double dhi[3],
                      const int32_t periodic[3], int32_t* impact) {
    return guard([&] {
        need(p, "params");
        CTX_SET();
        int b = E(ctx).impact_create(*p, dlo, dhi, periodic);
        if (impact) *impact = b;
    });
}

int sph_impact_set_domain(sph_ctx* ctx, int32_t impact, const double dlo[3], const double dhi[3],
                          const int32_t periodic[3]) {
    return guard([&] {
        need(dlo, "dlo");
        need(dhi, "dhi");
        CTX_SET();
        E(ctx).impact_set_domain(impact, dlo, dhi, periodic);
    });
}

int sph_impact_set_params(sph_ctx* ctx, int32_t impact, const sph_params* p) {
    return guard([&] {
        need(p, "params");
        CTX_SET();
        E(ctx).impact_set_params(impact, *p);
    });
}

int sph_impact_get_params(sph_ctx* ctx, int32_t impact, sph_params* p) {
    return guard([&] {
        need(p, "params");
        *p = E(ctx).impact_get_params(impact);
    });
}

int sph_impact_add_particles(sph_ctx* ctx, int32_t impact, int64_t n, const double* x,
                             const double* y, const double* z, const double* vx, const double* vy,
                             const double* vz, const double* mass, const double* u,
                             const int32_t* mat, const uint8_t* fixed) {
    return guard([&] {
        CTX_SET();
        E(ctx).impact_add_particles(impact, n, x, y, z, vx, vy, vz, mass, u, mat, fixed);
    });
}

int sph_impact_seed_damage(sph_ctx* ctx, int32_t impact, double dx, uint32_t seed) {
    return guard([&] {
        CTX_SET();
        E(ctx).impact_seed_damage(impact, dx, seed);
    });
}

int sph_impact_seed_flaws_multi(sph_ctx* ctx, int32_t impact, double dx, uint32_t seed,
                                int64_t* nflaws) {
    return guard([&] {
        CTX_SET();
        int64_t nf = E(ctx).impact_seed_flaws_multi(impact, dx, seed);
        if (nflaws) *nflaws = nf;
    });
}

int sph_impact_set_h0(sph_ctx* ctx, int32_t impact, const double* h0) {
    return guard([&] {
        need(h0, "h0");
        CTX_SET();
        E(ctx).impact_set_h0(impact, h0);
    });
}

int sph_impact_set_step_limit(sph_ctx* ctx, int32_t impact, int64_t steps) {
    return guard([&] {
        if (steps < 0) throw SphError(SPH_ERR_ARG, "steps < 0");
        CTX_SET();
        E(ctx).impact_set_step_limit(impact, steps);
    });
}

int sph_impact_remove(sph_ctx* ctx, int32_t impact) {
    return guard([&] {
        CTX_SET();
        E(ctx).impact_remove(impact);
    });
}

int sph_impact_count(sph_ctx* ctx, int32_t* count) {
    return guard([&] {
        need(count, "count");
        *count = E(ctx).impact_count();
    });
}

int sph_impact_info_get(sph_ctx* ctx, int32_t impact, sph_impact_info* info) {
    return guard([&] {
        need(info, "info");
        CTX_SET();
        *info = E(ctx).impact_info(impact);
    });
}

int sph_init(sph_ctx* ctx) {
    return guard([&] {
        CTX_SET();
        E(ctx).init();
    });
}

int sph_timestep(sph_ctx* ctx, int32_t impact, double* dt) {
    return guard([&] {
        need(dt, "dt");
        CTX_SET();
        *dt = E(ctx).timestep(impact);
    });
}

int sph_step(sph_ctx* ctx, double dt) {
    return guard([&] {
        if (!(dt >= 0) || !std::isfinite(dt)) throw SphError(SPH_ERR_ARG, "dt must be finite and >= 0");
        CTX_SET();
        E(ctx).step(dt);
    });
}

int sph_run(sph_ctx* ctx, int32_t nsteps, double t_end) {
    return guard([&] {
        if (nsteps < 0) throw SphError(SPH_ERR_ARG, "nsteps < 0");
        CTX_SET();
        E(ctx).run(nsteps, t_end);
    });
}

int sph_compute_density_h(sph_ctx* ctx, int32_t iters) {
    return guard([&] {
        if (iters < 1) throw SphError(SPH_ERR_ARG, "iters < 1");
        CTX_SET();
        E(ctx).compute_density_h(iters);
    });
}

int sph_compute_forces(sph_ctx* ctx) {
    return guard([&] {
        CTX_SET();
        E(ctx).compute_forces();
    });
}

int sph_synchronize(sph_ctx* ctx) {
    return guard([&] {
        CTX_SET();
        E(ctx).synchronize();
    });
}

int sph_read_field(sph_ctx* ctx, int32_t impact, const char* name, double* out) {
    return guard([&] {
        need(name, "name");
        need(out, "out");
        CTX_SET();
        E(ctx).read_field(impact, name, out);
    });
}

int sph_write_field(sph_ctx* ctx, int32_t impact, const char* name, const double* in) {
    return guard([&] {
        need(name, "name");
        need(in, "in");
        CTX_SET();
        E(ctx).write_field(impact, name, in);
    });
}

int sph_read_fields(sph_ctx* ctx, int32_t impact, int32_t nfields, const char* const* names, double* const* outs) {
    return guard([&] {
        if (nfields < 0) throw SphError(SPH_ERR_ARG, "nfields < 0");
        if (nfields > 0) { need(names, "names"); need(outs, "outs"); }
        for (int f = 0; f < nfields; f++) { need(names[f], "names[f]"); need(outs[f], "outs[f]"); }
        CTX_SET();
        E(ctx).read_fields(impact, nfields, names, outs);
    });
}

int sph_write_fields(sph_ctx* ctx, int32_t impact, int32_t nfields, const char* const* names,
                     const double* const* ins) {
    return guard([&] {
        if (nfields < 0) throw SphError(SPH_ERR_ARG, "nfields < 0");
        if (nfields > 0) { need(names, "names"); need(ins, "ins"); }
        for (int f = 0; f < nfields; f++) { need(names[f], "names[f]"); need(ins[f], "ins[f]"); }
        CTX_SET();
        E(ctx).write_fields(impact, nfields, names, ins);
    });
}

int sph_step_fields(sph_ctx* ctx, int32_t impact, double dt, int32_t nin, const char* const* in_names,
                    const double* const* ins, int32_t nout, const char* const* out_names, double* const* outs,
                    double* dt_used) {
    return guard([&] {
        if (!std::isfinite(dt)) throw SphError(SPH_ERR_ARG, "dt must be finite (< 0: the impact's CFL dt)");
        if (nin < 0 || nout < 0) throw SphError(SPH_ERR_ARG, "nin < 0 or nout < 0");
        if (nin > 0) { need(in_names, "in_names"); need(ins, "ins"); }
        if (nout > 0) { need(out_names, "out_names"); need(outs, "outs"); }
        for (int f = 0; f < nin; f++) { need(in_names[f], "in_names[f]"); need(ins[f], "ins[f]"); }
        for (int f = 0; f < nout; f++) { need(out_names[f], "out_names[f]"); need(outs[f], "outs[f]"); }
        CTX_SET();
        const double d = E(ctx).step_fields(impact, dt, nin, in_names, ins, nout, out_names, outs);
        if (dt_used) *dt_used = d;
    });
}

int sph_read_mat(sph_ctx* ctx, int32_t impact, int32_t* out) {
    return guard([&] {
        need(out, "out");
        E(ctx).read_mat(impact, out);
    });
}

int sph_read_fixed(sph_ctx* ctx, int32_t impact, uint8_t* out) {
    return guard([&] {
        need(out, "out");
        CTX_SET();
        E(ctx).read_fixed(impact, out);
    });
}

int sph_write_fixed(sph_ctx* ctx, int32_t impact, const uint8_t* in) {
    return guard([&] {
        need(in, "in");
        CTX_SET();
        E(ctx).write_fixed(impact, in);
    });
}

int sph_conservation_get(sph_ctx* ctx, int32_t impact, sph_conservation* out) {
    return guard([&] {
        need(out, "out");
        CTX_SET();
        *out = E(ctx).conservation(impact);
    });
}

int sph_impact_diagnostics(sph_ctx* ctx, int32_t impact, int32_t mat_lo, int32_t mat_hi, double u_melt,
                           sph_diagnostics* out) {
    return guard([&] {
        need(out, "out");
        if (mat_lo > mat_hi) throw SphError(SPH_ERR_ARG, "mat_lo > mat_hi");
        CTX_SET();
        double r[11];
        E(ctx).diagnostics(impact, mat_lo, mat_hi, u_melt, r);
        out->count = (int64_t)r[0];
        out->melted = (int64_t)r[1];
        for (int a = 0; a < 3; a++) {
            out->mean_pos[a] = r[2 + a];
            out->mean_vel[a] = r[5 + a];
        }
        out->mean_speed = r[8];
        out->dispersion = r[9];
        out->u_max = r[10];
    });
}

int sph_eos_eval(sph_ctx* ctx, int32_t mat, int64_t n, const double* rho, const double* u,
                 double* P, double* cs) {
    return guard([&] {
        if (n < 0) throw SphError(SPH_ERR_ARG, "n < 0");
        if (n > 0) { need(rho, "rho"); need(u, "u"); need(P, "P"); need(cs, "cs"); }
        CTX_SET();
        E(ctx).eos_eval(mat, n, rho, u, P, cs);
    });
}

int sph_debug_ref_cells(sph_ctx* ctx, int32_t impact, int32_t nc[3], double cw[3], int32_t* start,
                        int64_t start_len, int32_t* ids) {
    return guard([&] {
        need(nc, "nc"); need(cw, "cw"); need(start, "start"); need(ids, "ids");
        CTX_SET();
        E(ctx).debug_ref_cells(impact, nc, cw, start, start_len, ids);
    });
}

int sph_debug_neighbors(sph_ctx* ctx, int32_t impact, int32_t kind, int32_t* counts, int32_t* ids,
                        int64_t cap, int64_t* total) {
    return guard([&] {
        need(counts, "counts");
        if (kind != SPH_NBR_DENSITY && kind != SPH_NBR_FORCE) throw SphError(SPH_ERR_ARG, "bad kind");
        CTX_SET();
        int64_t t = E(ctx).debug_neighbors(impact, kind, counts, ids, cap);
        if (total) *total = t;
    });
}

int sph_debug_flaws(sph_ctx* ctx, int32_t impact, int64_t* ptr, double* eps, int64_t cap,
                    int64_t* total) {
    return guard([&] {
        need(ptr, "ptr");
        CTX_SET();
        int64_t t = E(ctx).debug_flaws(impact, ptr, eps, cap);
        if (total) *total = t;
    });
}

// ---------------------------------------------------------------- files
namespace {

struct File {
    FILE* f = nullptr;
    File(const char* p, const char* mode) : f(std::fopen(p, mode)) {}
    ~File() { if (f) std::fclose(f); }
};

void read_exact(FILE* f, void* dst, size_t bytes, const char* what) {
    if (std::fread(dst, 1, bytes, f) != bytes) throw SphError(SPH_ERR_IO, std::string("short read: ") + what);
}

void write_exact(FILE* f, const void* src, size_t bytes) {
    if (std::fwrite(src, 1, bytes, f) != bytes) throw SphError(SPH_ERR_IO, "short write");
}

std::vector<double> field(EngineBase& e, int b, const char* nm) {
    std::vector<double> v(e.impact_n(b));
    e.read_field(b, nm, v.data());
    return v;
}

}  // namespace

namespace {

// The reference builder's coordinate range (boundary_daemon.py:111-115):
// start, start + step, ... by repeated addition while short of stop.
std::vector<double> accumulated_range(double start, double stop, double step) {
    std::vector<double> out;
    double x = start;
    while (step > 0 ? x < stop : x > stop) {
        out.push_back(x);
        x += step;
        if (out.size() > (size_t)1 << 26) throw dsph::SphError(SPH_ERR_CAPACITY, "grazing IC lattice too large");
    }
    return out;
}

// Layout of build_grazing_ic (boundary_daemon.py:119-158), operation for
// operation (Python float ** is the C pow; this file is built without FP
// contraction), so the generated particles equal the reference's file.
std::shared_ptr<dsph::GrazingLayout> grazing_layout(const sph_grazing_spec& s) {
    if (!(s.D > 0) || s.cppr < 1 || !(s.v >= 0)) throw dsph::SphError(SPH_ERR_ARG, "grazing IC: need D > 0, cppr >= 1, v >= 0");
    auto L = std::make_shared<dsph::GrazingLayout>();
    const double a = s.D / 2.0;
    const double dx = a / (double)s.cppr;
    const double m_imp = s.rho_imp * std::pow(dx, 3.0);
    const double th = s.theta_deg * (M_PI / 180.0);
    const double vx = s.v * std::cos(th), vz = -s.v * std::sin(th);
    const double Lx = std::max(20e3, 30.0 * s.D), Ly = std::max(4e3, 6.0 * s.D), Lz = std::max(6e3, 8.0 * s.D);
    const double wall = 6.0 * dx;
    const double mt = s.rho_target * std::pow(dx, 3.0);
    L->xs = accumulated_range(-0.4 * Lx + dx / 2, 0.6 * Lx, dx);
    L->ys = accumulated_range(-Ly / 2 + dx / 2, Ly / 2, dx);
    L->zs = accumulated_range(-dx / 2, -Lz, -dx);
    if (L->xs.empty() || L->ys.empty() || L->zs.empty()) throw dsph::SphError(SPH_ERR_ARG, "grazing IC: empty lattice");
    L->wall = wall;
    L->m_target = mt;
    const double z0 = std::isnan(s.start_h) ? (a + 3.0 * dx) : s.start_h;
    const double x0 = std::isnan(s.x_impact_frac) ? -0.35 * Lx : (s.x_impact_frac * Lx - z0 / std::tan(th));
    const int na = (int)std::ceil(a / dx) + 1;
    for (int i = -na; i <= na; i++)
        for (int j = -na; j <= na; j++)
            for (int k = -na; k <= na; k++)
                if (std::pow(i * dx, 2.0) + std::pow(j * dx, 2.0) + std::pow(k * dx, 2.0) <= a * a) {
                    L->px.push_back(i * dx + x0);
                    L->py.push_back(j * dx);
                    L->pz.push_back(k * dx + z0);
                }
    L->vx = vx;
    L->vz = vz;
    L->m_imp = m_imp;
    L->tgt_mat = s.tgt_mat;
    L->imp_mat = s.imp_mat;
    L->dx = dx;
    L->dlo[0] = L->xs.front() - dx;
    L->dhi[0] = L->xs.back() + dx;
    L->dlo[1] = L->ys.front() - dx;
    L->dhi[1] = L->ys.back() + dx;
    L->dlo[2] = L->zs.back() - dx;
    L->dhi[2] = z0 + a + 0.5 * Lz;
    if (L->n() > ((int64_t)1 << 31) - 1) throw dsph::SphError(SPH_ERR_CAPACITY, "grazing IC: too many particles");
    return L;
}

}  // namespace

void sph_grazing_spec_default(sph_grazing_spec* s) {
    if (!s) return;
    std::memset(s, 0, sizeof(*s));
    s->theta_deg = 10.0;
    s->v = 10000.0;
    s->D = 1000.0;        // boundary_daemon.py:36-40
    s->rho_imp = 7800.0;
    s->rho_target = 2700.0;
    s->x_impact_frac = NAN;
    s->start_h = NAN;
    s->cppr = 8;
    s->tgt_mat = 0;
    s->imp_mat = 1;
}

int sph_impact_create_grazing(sph_ctx* ctx, const sph_params* p, const sph_grazing_spec* s, int32_t* impact,
                              double* dx_out, int64_t* n_out) {
    return guard([&] {
        need(p, "params");
        need(s, "spec");
        need(impact, "impact");
        CTX_SET();
        auto L = grazing_layout(*s);
        *impact = E(ctx).impact_create_generated(*p, L);
        if (dx_out) *dx_out = L->dx;
        if (n_out) *n_out = L->n();
    });
}

int sph_load_ic(sph_ctx* ctx, const char* path, const sph_params* p, int32_t* impact) {
    return guard([&] {
        need(path, "path");
        need(p, "params");
        CTX_SET();
        File F(path, "rb");
        if (!F.f) throw SphError(SPH_ERR_IO, std::string("cannot open ") + path);
        double hdr[7];
        read_exact(F.f, hdr, sizeof hdr, "IC header");
        long long n = std::llround(hdr[6]);
        if (n < 0 || n > (1ll << 31) - 1) throw SphError(SPH_ERR_IO, "bad particle count in IC header");
        std::vector<double> rec((size_t)n * 10);
        read_exact(F.f, rec.data(), sizeof(double) * rec.size(), "IC records");
        std::vector<double> c[8];
        for (auto& v : c) v.resize(n);
        std::vector<int32_t> mat(n);
        std::vector<uint8_t> fixed(n);
        for (long long i = 0; i < n; i++) {
            for (int q = 0; q < 8; q++) c[q][i] = rec[i * 10 + q];
            mat[i] = (int32_t)rec[i * 10 + 8];
            fixed[i] = rec[i * 10 + 9] != 0.0;
        }
        double lo[3] = {hdr[0], hdr[2], hdr[4]}, hi[3] = {hdr[1], hdr[3], hdr[5]};
        int32_t per[3] = {0, 0, 0};
        EngineBase& e = E(ctx);
        int b = e.impact_create(*p, lo, hi, per);
        try {
            e.impact_add_particles(b, n, c[0].data(), c[1].data(), c[2].data(), c[3].data(), c[4].data(),
                                   c[5].data(), c[6].data(), c[7].data(), mat.data(), fixed.data());
        } catch (...) {
            e.impact_remove(b);
            throw;
        }
        if (impact) *impact = b;
    });
}

int sph_write_snapshot(sph_ctx* ctx, int32_t impact, const char* path) {
    return guard([&] {
        need(path, "path");
        CTX_SET();
        EngineBase& e = E(ctx);
        int64_t n = e.impact_n(impact);
        const char* names[9] = {"x", "y", "z", "vx", "vy", "vz", "u", "rho", "hh"};
        std::vector<std::vector<double>> cols;
        for (auto nm : names) cols.push_back(field(e, impact, nm));
        std::vector<int32_t> mat(n);
        e.read_mat(impact, mat.data());
        std::vector<double> buf((size_t)n * 10);
        for (int64_t i = 0; i < n; i++) {
            for (int q = 0; q < 9; q++) buf[i * 10 + q] = cols[q][i];
            buf[i * 10 + 9] = (double)mat[i];
        }
        File F(path, "wb");
        if (!F.f) throw SphError(SPH_ERR_IO, std::string("cannot create ") + path);
        int64_t nn = n;
        write_exact(F.f, &nn, sizeof nn);
        write_exact(F.f, buf.data(), sizeof(double) * buf.size());
    });
}

int sph_write_checkpoint(sph_ctx* ctx, int32_t impact, const char* path, double dx) {
    return guard([&] {
        need(path, "path");
        CTX_SET();
        EngineBase& e = E(ctx);
        int64_t n = e.impact_n(impact);
        sph_impact_info inf = e.impact_info(impact);
        double lo[3], hi[3];
        int32_t per[3];
        e.get_domain(impact, lo, hi, per);
        const char* names[8] = {"x", "y", "z", "vx", "vy", "vz", "mass", "u"};
        std::vector<std::vector<double>> cols;
        for (auto nm : names) cols.push_back(field(e, impact, nm));
        std::vector<double> D = field(e, impact, "D"), ea = field(e, impact, "eps_act");
        const char* sn[6] = {"Sxx", "Sxy", "Sxz", "Syy", "Syz", "Szz"};
        std::vector<std::vector<double>> S;
        for (auto nm : sn) S.push_back(field(e, impact, nm));
        std::vector<int32_t> mat(n);
        std::vector<uint8_t> fixed(n);
        e.read_mat(impact, mat.data());
        e.read_fixed(impact, fixed.data());
        std::vector<double> buf((size_t)n * 18);
        for (int64_t i = 0; i < n; i++) {
            double* r = &buf[i * 18];
            for (int q = 0; q < 8; q++) r[q] = cols[q][i];
            r[8] = (double)mat[i];
            r[9] = (double)fixed[i];
            r[10] = D[i];
            r[11] = ea[i];
            for (int q = 0; q < 6; q++) r[12 + q] = S[q][i];
        }
        double hdr[9] = {lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], (double)n, inf.t, dx};
        std::string tmp = std::string(path) + ".tmp";
        {
            File F(tmp.c_str(), "wb");
            if (!F.f) throw SphError(SPH_ERR_IO, std::string("cannot create ") + tmp);
            write_exact(F.f, hdr, sizeof hdr);
            write_exact(F.f, buf.data(), sizeof(double) * buf.size());
        }
        if (std::rename(tmp.c_str(), path) != 0) throw SphError(SPH_ERR_IO, "rename failed");
    });
}

int sph_load_checkpoint(sph_ctx* ctx, const char* path, const sph_params* p, int32_t* impact,
                        double* dx_out) {
    return guard([&] {
        need(path, "path");
        need(p, "params");
        CTX_SET();
        File F(path, "rb");
        if (!F.f) throw SphError(SPH_ERR_IO, std::string("cannot open ") + path);
        double hdr[9];
        read_exact(F.f, hdr, sizeof hdr, "checkpoint header");
        long long n = std::llround(hdr[6]);
        if (n < 0 || n > (1ll << 31) - 1) throw SphError(SPH_ERR_IO, "bad particle count in checkpoint");
        std::vector<double> rec((size_t)n * 18);
        read_exact(F.f, rec.data(), sizeof(double) * rec.size(), "checkpoint records");
        std::vector<double> c[8];
        for (auto& v : c) v.resize(n);
        std::vector<int32_t> mat(n);
        std::vector<uint8_t> fixed(n);
        std::vector<double> D(n), ea(n), S[6];
        for (auto& v : S) v.resize(n);
        for (long long i = 0; i < n; i++) {
            const double* r = &rec[i * 18];
            for (int q = 0; q < 8; q++) c[q][i] = r[q];
            mat[i] = (int32_t)r[8];
            fixed[i] = r[9] != 0.0;
            D[i] = r[10];
            ea[i] = r[11];
            for (int q = 0; q < 6; q++) S[q][i] = r[12 + q];
        }
        double lo[3] = {hdr[0], hdr[2], hdr[4]}, hi[3] = {hdr[1], hdr[3], hdr[5]};
        int32_t per[3] = {0, 0, 0};
        EngineBase& e = E(ctx);
        int b = e.impact_create(*p, lo, hi, per);
        try {
            e.impact_add_particles(b, n, c[0].data(), c[1].data(), c[2].data(), c[3].data(), c[4].data(),
                                   c[5].data(), c[6].data(), c[7].data(), mat.data(), fixed.data());
            if (n > 0) {
                e.write_field(b, "D", D.data());
                e.write_field(b, "eps_act", ea.data());
                const char* sn[6] = {"Sxx", "Sxy", "Sxz", "Syy", "Syz", "Szz"};
                for (int q = 0; q < 6; q++) e.write_field(b, sn[q], S[q].data());
            }
            e.impact_set_time(b, hdr[7]);
        } catch (...) {
            e.impact_remove(b);
            throw;
        }
        if (impact) *impact = b;
        if (dx_out) *dx_out = hdr[8];
    });
}

int sph_set_tuning(sph_ctx* ctx, int32_t block_threads, double cell_factor) {
    return guard([&] { E(ctx).set_tuning(block_threads, cell_factor); });
}

int sph_set_option(sph_ctx* ctx, const char* key, double value) {
    return guard([&] {
        need(key, "key");
        E(ctx).set_option(key, value);
    });
}

int sph_get_option(sph_ctx* ctx, const char* key, double* value) {
    return guard([&] {
        need(key, "key");
        need(value, "value");
        *value = E(ctx).get_option(key);
    });
}

int sph_launch_count(sph_ctx* ctx, int64_t* launches) {
    return guard([&] {
        need(launches, "launches");
        *launches = E(ctx).launches();
    });
}

int sph_phase_times(sph_ctx* ctx, double ms[5]) {
    return guard([&] {
        need(ms, "ms");
        E(ctx).phase_times(ms);
    });
}

int sph_set_profiling(sph_ctx* ctx, int32_t on) {
    return guard([&] { E(ctx).set_profiling(on); });
}

int sph_kernel_stats(sph_ctx* ctx, int32_t kernel_class, double* total_ms, int64_t* launches) {
    return guard([&] {
        need(total_ms, "total_ms");
        need(launches, "launches");
        E(ctx).kernel_stats(kernel_class, total_ms, launches);
    });
}

int sph_kernel_stats_reset(sph_ctx* ctx) {
    return guard([&] { E(ctx).kernel_stats_reset(); });
}

int sph_event_record(sph_ctx* ctx, int32_t slot) {
    return guard([&] {
        CTX_SET();
        E(ctx).event_record(slot);
    });
}

int sph_event_elapsed(sph_ctx* ctx, int32_t slot_a, int32_t slot_b, double* ms) {
    return guard([&] {
        need(ms, "ms");
        CTX_SET();
        *ms = E(ctx).event_elapsed(slot_a, slot_b);
    });
}

}  // extern "C"
