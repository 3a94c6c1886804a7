// euler.cu -- GB300 Eulerian grid hydrocode: the reference's CPU Euler solver
// (hydrocodes/euler/hydro_cpu.cpp) as FP64 CUDA kernels behind the C ABI of
// include/deorbit_euler.h.
//
// Layout: structure of arrays in HBM, one array per field in the reference's
// cell order (i*ny + j)*nz + k.  One Lop (hydro_cpu.cpp:98-214) is
//   k_prim   primitives (rho, v, e) and the tracer ratio rc/rho per cell, once
//            (the reference recomputes them for every face that reads a cell);
//   k_face   one launch per direction, one thread per face: MUSCL-minmod
//            reconstruction from four cells, HLLC (or the vacuum flux), the
//            tracer flux -- each face flux computed once and stored;
//   k_rhs    one thread per cell: the three directions' flux differences added
//            in the reference's order (x, y, z), gravity, then the strength
//            sources (Jaumann rate, upwind advection, div S, div(S.v)).
// The Runge-Kutta stages (k_predict, k_correct) fuse the elementwise updates
// with the void-cell reset, the radial return, damage growth and damping.
// k_maxspeed reduces the CFL speed; k_dt forms dt and the stop test on the
// device, so whole steps replay from a captured CUDA graph.
//
// This file is compiled without fused multiply-adds (--fmad=false): every
// expression is evaluated in the reference's operation order with IEEE
// rounding, so ideal-gas grids reproduce the reference bit for bit and
// Tillotson grids differ only through the device's exp / pow.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "deorbit_euler.h"
#include "engine.hpp"
#include "euler_kernels.cuh"

namespace dsph {
void set_error_message(const std::string& m);
}

namespace deu {

using dsph::SphError;

// ---------------------------------------------------------------- host engine

#define EU_CUDA(x)                                                                                     \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) throw SphError(SPH_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
    } while (0)

// Makes a device current for a call's duration and restores the caller's.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        EU_CUDA(cudaGetDevice(&prev));
        if (prev != dev) EU_CUDA(cudaSetDevice(dev));
    }
    ~DeviceScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

struct Grid {
    int device = 0;
    cudaStream_t st = nullptr;
    P p{};
    Fields g{}, g1{};
    Rhs d{};
    bool mixed = false;        // Lop in FP32 (primitives, face fluxes, sources)
    PrimT<double> W{};         // FP64 form
    FacesT<double> F{};
    PrimT<float> W32{};        // mixed form
    FacesT<float> F32{};
    Ctl* ctl = nullptr;
    double* scratch = nullptr;  // pressure read-out
    double* ref_r0 = nullptr;   // hydrostatic reference (set_ref), allocated on first use
    double* ref_p0 = nullptr;
    std::vector<void*> allocs;
    int64_t bytes = 0;
    int64_t launches = 0;
    cudaEvent_t ev[8] = {};
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;

    template <class T = double>
    T* alloc(int64_t count) {
        void* ptr = nullptr;
        const size_t b = sizeof(T) * (size_t)std::max<int64_t>(count, 1);
        cudaError_t e = cudaMalloc(&ptr, b);
        if (e != cudaSuccess) throw SphError(SPH_ERR_NOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
        allocs.push_back(ptr);
        bytes += (int64_t)b;
        EU_CUDA(cudaMemsetAsync(ptr, 0, b, st));
        return (T*)ptr;
    }

    void release() {
        if (graph) cudaGraphExecDestroy(graph);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        for (void* a : allocs) cudaFree(a);
        allocs.clear();
        if (st) cudaStreamDestroy(st);
        st = nullptr;
    }

    unsigned grid_of(int64_t count) const { return (unsigned)((count + 255) / 256); }

    void enqueue_lop(const Fields& s) {
        if (mixed) enqueue_lop_f32(p, s, W32, g.q[F_AF], F32, d, ctl, st);
        else enqueue_lop_t<double>(p, s, W, g.q[F_AF], F, d, ctl, st);
        launches += 5;
    }

    // One step_rk2 (hydro_cpu.cpp:411-425); with_dt: the drivers' dt and stop
    // test on the device first.
    void enqueue_step(bool with_dt) {
        const int64_t n = p.n;
        if (with_dt) {
            k_begin<<<1, 1, 0, st>>>(ctl);
            if (mixed) enqueue_maxspeed_f32(p, g, ctl, st);
            else enqueue_maxspeed_t<double>(p, g, ctl, st);
            k_dt<<<1, 1, 0, st>>>(p, ctl);
            launches += 3;
        }
        if (p.c_act > 0 && p.tdec > 0) {
            k_update_af<<<grid_of(n), 256, 0, st>>>(p, g, ctl);
            launches++;
        }
        enqueue_lop(g);
        if (mixed) enqueue_predict_f32(p, g, g1, d, ctl, st);
        else enqueue_predict_t<double>(p, g, g1, d, ctl, st);
        enqueue_lop(g1);
        if (mixed) enqueue_correct_f32(p, g, g1, d, ctl, st);
        else enqueue_correct_t<double>(p, g, g1, d, ctl, st);
        k_end<<<1, 1, 0, st>>>(ctl);
        launches += 3;
    }

    Ctl read_ctl() {
        Ctl h;
        EU_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        EU_CUDA(cudaStreamSynchronize(st));
        return h;
    }

    void check() {
        EU_CUDA(cudaGetLastError());
    }
};

Grid* G(eu_grid* h) {
    if (!h) throw SphError(SPH_ERR_ARG, "null grid");
    return reinterpret_cast<Grid*>(h);
}

int field_index(const char* name) {
    if (!name) throw SphError(SPH_ERR_ARG, "null field name");
    for (int q = 0; q < NF; q++)
        if (!std::strcmp(name, kFieldNames[q])) return q;
    throw SphError(SPH_ERR_ARG, std::string("unknown field: ") + name);
}

int rhs_index(const char* name) {
    if (!name) throw SphError(SPH_ERR_ARG, "null field name");
    for (int q = 0; q < ND; q++)
        if (!std::strcmp(name, kRhsNames[q])) return q;
    throw SphError(SPH_ERR_ARG, std::string("unknown right-hand-side field: ") + name);
}

template <class Fn>
int guard(Fn&& f) {
    try {
        f();
        return SPH_OK;
    } catch (const SphError& e) {
        dsph::set_error_message(e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        dsph::set_error_message("host allocation failed");
        return SPH_ERR_NOMEM;
    } catch (const std::exception& e) {
        dsph::set_error_message(e.what());
        return SPH_ERR_STATE;
    }
}

void need_n(const Grid* g, int64_t n) {
    if (n != g->p.n) throw SphError(SPH_ERR_ARG, "field size must be nx*ny*nz");
}

}  // namespace deu

using deu::G;
using deu::guard;
using deu::SphError;

namespace {

void to_params(deu::P& p, const eu_params& e) {
    p.gz = e.gz; p.tdec = e.tdec; p.eta_af = e.eta_af; p.c_act = e.c_act; p.p_coh = e.p_coh; p.p_act = e.p_act;
    p.rho_cfl = e.rho_cfl; p.damp = e.damp; p.rho_vac = e.rho_vac;
    p.y_i0 = e.y_i0; p.mu_i = e.mu_i; p.mu_d = e.mu_d; p.y_d0 = e.y_d0; p.y_m = e.y_m; p.y_bingham = e.y_bingham;
    p.c_reg = e.c_reg; p.af_sat = e.af_sat;
    p.axisym = e.axisym != 0; p.rock = e.rock != 0; p.af_reg = e.af_reg != 0; p.af_prel = e.af_prel != 0;
    p.af_seeddp = e.af_seeddp != 0;
    p.void_amb = e.void_amb;
    p.void_cons = e.void_cons != 0;
}

// Weakest-flaw activation strain of grow_damage (hydro_cpu.cpp:254), formed
// on the host with the host library's pow.
void derive(deu::P& p) {
    const deu::Mat& m = p.m;
    p.eps_act = (m.Emod > 0 && m.wk > 0) ? std::pow(1.0 / (m.wk * p.dx * p.dx * p.dx), 1.0 / m.wm) : 0.0;
    p.invdx = 1.0 / p.dx;
}

}  // namespace

extern "C" {

void eu_params_default(eu_params* out) {
    if (!out) return;
    std::memset(out, 0, sizeof *out);
    out->p_coh = 1.0e6;  // hydro_cpu.cpp:21
    out->damp = 1.0;     // hydro_cpu.cpp:24
    out->y_i0 = 1.0e7;   // hydro_cpu.cpp:30-34
    out->mu_i = 1.2;
    out->mu_d = 0.6;
    out->y_m = 2.5e9;
    out->c_reg = 0.1;    // hydro_cpu.cpp:222
    out->af_sat = 1.0;
}

int eu_create(int32_t nx, int32_t ny, int32_t nz, double dx, int32_t device, eu_grid** out) {
    return eu_create_form(nx, ny, nz, dx, device, EU_FP64, out);
}

int eu_create_form(int32_t nx, int32_t ny, int32_t nz, double dx, int32_t device, int32_t form, eu_grid** out) {
    return guard([&] {
        if (form != EU_FP64 && form != EU_MIXED) throw SphError(SPH_ERR_ARG, "unknown form");
        if (!out) throw SphError(SPH_ERR_ARG, "null output pointer");
        *out = nullptr;
        if (nx < 1 || ny < 1 || nz < 1) throw SphError(SPH_ERR_ARG, "grid dimensions must be >= 1");
        if (!(dx > 0) || !std::isfinite(dx)) throw SphError(SPH_ERR_ARG, "dx must be finite and > 0");
        const int64_t n = (int64_t)nx * ny * nz;
        if (n > ((int64_t)1 << 31) - 1) throw SphError(SPH_ERR_CAPACITY, "more than 2^31 - 1 cells");
        int ndev = 0;
        cudaError_t e = cudaGetDeviceCount(&ndev);
        if (e != cudaSuccess || ndev == 0)
            throw SphError(SPH_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
        if (device < 0 || device >= ndev) throw SphError(SPH_ERR_ARG, "bad device ordinal");
        deu::DeviceScope ds(device);
        auto* g = new deu::Grid();
        try {
            g->device = device;
            EU_CUDA(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking));
            g->p.nx = nx; g->p.ny = ny; g->p.nz = nz; g->p.n = n; g->p.dx = dx;
            g->p.m.ideal = 1;  // MAT = Material::ideal(1.4), hydro_cpu.cpp:15
            g->p.m.gamma = 1.4;
            eu_params ep;
            eu_params_default(&ep);
            to_params(g->p, ep);
            derive(g->p);
            for (int q = 0; q < deu::NF; q++) g->g.q[q] = g->alloc(n);
            for (int q = 0; q < deu::NF; q++) g->g1.q[q] = g->g.q[q];  // af, Pmax shared
            for (int q = 0; q < deu::ND; q++) g->g1.q[deu::rk_field(q)] = g->alloc(n);
            for (int q = 0; q < deu::ND; q++) g->d.q[q] = g->alloc(n);
            g->mixed = form == EU_MIXED;
            for (int q = 0; q < 7; q++) {
                if (g->mixed) g->W32.w[q] = g->alloc<float>(n);
                else g->W.w[q] = g->alloc(n);
            }
            const int64_t nfc[3] = {deu::face_count<0>(nx, ny, nz), deu::face_count<1>(nx, ny, nz),
                                    deu::face_count<2>(nx, ny, nz)};
            for (int dir = 0; dir < 3; dir++)
                for (int q = 0; q < 6; q++) {
                    if (g->mixed) g->F32.q[dir][q] = g->alloc<float>(nfc[dir]);
                    else g->F.q[dir][q] = g->alloc(nfc[dir]);
                }
            g->scratch = g->alloc(n);
            void* c = nullptr;
            EU_CUDA(cudaMalloc(&c, sizeof(deu::Ctl)));
            g->allocs.push_back(c);
            g->bytes += sizeof(deu::Ctl);
            g->ctl = (deu::Ctl*)c;
            EU_CUDA(cudaMemsetAsync(c, 0, sizeof(deu::Ctl), g->st));
            for (auto& ev : g->ev) EU_CUDA(cudaEventCreate(&ev));
            EU_CUDA(cudaStreamSynchronize(g->st));
        } catch (...) {
            g->release();
            delete g;
            throw;
        }
        *out = reinterpret_cast<eu_grid*>(g);
    });
}

int eu_destroy(eu_grid* h) {
    return guard([&] {
        if (!h) return;
        deu::Grid* g = G(h);
        {
            deu::DeviceScope ds(g->device);
            cudaStreamSynchronize(g->st);
            g->release();
        }
        delete g;
    });
}

int eu_set_material(eu_grid* h, const sph_material* m) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!m) throw SphError(SPH_ERR_ARG, "null material");
        if (m->type != SPH_EOS_IDEAL && m->type != SPH_EOS_TILLOTSON) throw SphError(SPH_ERR_ARG, "unknown EOS type");
        deu::Mat& M = g->p.m;
        M.ideal = m->type == SPH_EOS_IDEAL;
        M.gamma = m->gamma; M.rho0 = m->rho0; M.a = m->a; M.b = m->b; M.A = m->A; M.B = m->B;
        M.alpha = m->alpha; M.beta = m->beta; M.u0 = m->u0; M.uiv = m->uiv; M.ucv = m->ucv;
        M.G = m->G; M.Y = m->Y; M.Emod = m->Emod; M.wm = m->wm; M.wk = m->wk;
        derive(g->p);
        g->graph_valid = false;
    });
}

int eu_set_params(eu_grid* h, const eu_params* e) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!e) throw SphError(SPH_ERR_ARG, "null params");
        if (e->axisym && g->p.ny != 1) throw SphError(SPH_ERR_ARG, "axisym needs ny == 1");
        if (!(e->damp >= 0) || !(e->damp <= 1.0)) throw SphError(SPH_ERR_ARG, "damp must be in [0, 1]");
        if (!(e->void_amb >= 0)) throw SphError(SPH_ERR_ARG, "void_amb must be >= 0");
        to_params(g->p, *e);
        g->graph_valid = false;
    });
}

int eu_set_ref(eu_grid* h) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::DeviceScope ds(g->device);
        if (!g->ref_r0) {
            g->ref_r0 = g->alloc(g->p.n);
            g->ref_p0 = g->alloc(g->p.n);
        }
        deu::k_set_ref<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->g, g->ref_r0, g->ref_p0);
        g->launches++;
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
        g->p.ref_r0 = g->ref_r0;
        g->p.ref_p0 = g->ref_p0;
        g->graph_valid = false;
    });
}

int eu_clear_ref(eu_grid* h) {
    return guard([&] {
        deu::Grid* g = G(h);
        g->p.ref_r0 = nullptr;
        g->p.ref_p0 = nullptr;
        g->graph_valid = false;
    });
}

int eu_read_ref(eu_grid* h, double* r0, double* p0, int64_t n) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::need_n(g, n);
        if (!g->p.ref_r0) throw SphError(SPH_ERR_STATE, "no reference state (eu_set_ref)");
        deu::DeviceScope ds(g->device);
        if (r0) EU_CUDA(cudaMemcpyAsync(r0, g->ref_r0, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, g->st));
        if (p0) EU_CUDA(cudaMemcpyAsync(p0, g->ref_p0, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, g->st));
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_get_shape(const eu_grid* h, int32_t shape[3], double* dx) {
    return guard([&] {
        const deu::Grid* g = G(const_cast<eu_grid*>(h));
        if (shape) { shape[0] = g->p.nx; shape[1] = g->p.ny; shape[2] = g->p.nz; }
        if (dx) *dx = g->p.dx;
    });
}

int eu_write_field(eu_grid* h, const char* name, const double* host, int64_t n) {
    return eu_write_fields(h, 1, &name, &host, n);
}

int eu_read_field(eu_grid* h, const char* name, double* host, int64_t n) {
    return eu_read_fields(h, 1, &name, &host, n);
}

int eu_write_fields(eu_grid* h, int32_t nfields, const char* const* names, const double* const* host, int64_t n) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::need_n(g, n);
        if (nfields < 0 || (nfields > 0 && (!names || !host))) throw SphError(SPH_ERR_ARG, "bad field list");
        deu::DeviceScope ds(g->device);
        for (int32_t i = 0; i < nfields; i++) {
            if (!host[i]) throw SphError(SPH_ERR_ARG, "null host buffer");
            const int q = deu::field_index(names[i]);
            EU_CUDA(cudaMemcpyAsync(g->g.q[q], host[i], sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, g->st));
        }
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_read_fields(eu_grid* h, int32_t nfields, const char* const* names, double* const* host, int64_t n) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::need_n(g, n);
        if (nfields < 0 || (nfields > 0 && (!names || !host))) throw SphError(SPH_ERR_ARG, "bad field list");
        deu::DeviceScope ds(g->device);
        for (int32_t i = 0; i < nfields; i++) {
            if (!host[i]) throw SphError(SPH_ERR_ARG, "null host buffer");
            const int q = deu::field_index(names[i]);
            EU_CUDA(cudaMemcpyAsync(host[i], g->g.q[q], sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, g->st));
        }
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_lop(eu_grid* h) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::DeviceScope ds(g->device);
        deu::k_maxspeed_begin<<<1, 1, 0, g->st>>>(g->ctl);  // marks the control active
        g->enqueue_lop(g->g);
        g->launches++;
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_read_rhs(eu_grid* h, const char* name, double* host, int64_t n) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::need_n(g, n);
        if (!host) throw SphError(SPH_ERR_ARG, "null host buffer");
        deu::DeviceScope ds(g->device);
        const int q = deu::rhs_index(name);
        EU_CUDA(cudaMemcpyAsync(host, g->d.q[q], sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, g->st));
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_vonmises(eu_grid* h, int32_t reg) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::DeviceScope ds(g->device);
        deu::k_vonmises<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->g, reg);
        g->launches++;
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_grow_damage(eu_grid* h, double dt) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!std::isfinite(dt)) throw SphError(SPH_ERR_ARG, "dt must be finite");
        deu::DeviceScope ds(g->device);
        deu::k_grow_damage<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->g, dt);
        g->launches++;
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_update_af(eu_grid* h, double dt) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!std::isfinite(dt)) throw SphError(SPH_ERR_ARG, "dt must be finite");
        deu::DeviceScope ds(g->device);
        if (g->p.c_act > 0 && g->p.tdec > 0) {  // update_af returns at once otherwise (hydro_cpu.cpp:391)
            deu::k_set_step<<<1, 1, 0, g->st>>>(g->ctl, dt);
            deu::k_update_af<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->g, g->ctl);
            g->launches += 2;
        }
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_maxspeed(eu_grid* h, double* out) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!out) throw SphError(SPH_ERR_ARG, "null output pointer");
        deu::DeviceScope ds(g->device);
        deu::k_maxspeed_begin<<<1, 1, 0, g->st>>>(g->ctl);
        if (g->mixed) deu::enqueue_maxspeed_f32(g->p, g->g, g->ctl, g->st);
        else deu::enqueue_maxspeed_t<double>(g->p, g->g, g->ctl, g->st);
        g->launches += 2;
        g->check();
        const deu::Ctl c = g->read_ctl();
        std::memcpy(out, &c.smax_bits, sizeof(double));
    });
}

int eu_read_pressure(eu_grid* h, double* host, int64_t n) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::need_n(g, n);
        if (!host) throw SphError(SPH_ERR_ARG, "null host buffer");
        deu::DeviceScope ds(g->device);
        deu::k_pressure<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->g, g->scratch);
        g->launches++;
        g->check();
        EU_CUDA(cudaMemcpyAsync(host, g->scratch, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, g->st));
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_step(eu_grid* h, double dt) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!(dt >= 0) || !std::isfinite(dt)) throw SphError(SPH_ERR_ARG, "dt must be finite and >= 0");
        deu::DeviceScope ds(g->device);
        deu::k_set_step<<<1, 1, 0, g->st>>>(g->ctl, dt);
        g->launches++;
        g->enqueue_step(false);
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_run(eu_grid* h, double cfl, double t_end, int64_t max_steps, int64_t* steps, double* t) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!(cfl > 0) || !std::isfinite(cfl)) throw SphError(SPH_ERR_ARG, "cfl must be finite and > 0");
        if (std::isnan(t_end)) throw SphError(SPH_ERR_ARG, "t_end is NaN");
        deu::DeviceScope ds(g->device);
        deu::k_set_run<<<1, 1, 0, g->st>>>(g->ctl, cfl, t_end, max_steps);
        g->launches++;
        const deu::Ctl c0 = g->read_ctl();
        if (!g->graph_valid) {  // one driver step, captured once per settings
            if (g->graph) cudaGraphExecDestroy(g->graph);
            g->graph = nullptr;
            cudaGraph_t gr = nullptr;
            const int64_t l0 = g->launches;
            EU_CUDA(cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal));
            g->enqueue_step(true);
            cudaError_t e = cudaStreamEndCapture(g->st, &gr);
            if (e != cudaSuccess) throw SphError(SPH_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(e));
            e = cudaGraphInstantiate(&g->graph, gr, 0);
            cudaGraphDestroy(gr);
            if (e != cudaSuccess) throw SphError(SPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
            g->launches = l0;
            g->graph_valid = true;
        }
        const int64_t per_step = 16 + ((g->p.c_act > 0 && g->p.tdec > 0) ? 1 : 0) +
                                 ((g->p.void_cons && g->p.ref_r0 && g->p.rho_cfl > 0) ? 3 : 0);
        const int64_t limit = c0.max_steps;  // absolute step count, -1 = none
        deu::Ctl c = c0;
        // replay in chunks; steps past the end are no-ops (inactive control)
        int chunk = 4;
        while (c.t < c.t_end && (limit < 0 || c.steps < limit)) {
            int todo = chunk;
            if (limit >= 0) todo = (int)std::min<int64_t>(todo, limit - c.steps);
            for (int i = 0; i < todo; i++) EU_CUDA(cudaGraphLaunch(g->graph, g->st));
            g->launches += per_step * todo;
            const double t_prev = c.t;
            c = g->read_ctl();
            if (!(c.t > t_prev))  // dt collapsed (signal speed not finite): stop instead of spinning
                throw SphError(SPH_ERR_STATE, "time step collapsed: no progress in t (non-finite state?)");
            chunk = std::min(chunk * 2, 64);
        }
        if (steps) *steps = c.steps - c0.steps;
        if (t) *t = c.t;
    });
}

int eu_set_time(eu_grid* h, double t) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!std::isfinite(t)) throw SphError(SPH_ERR_ARG, "t must be finite");
        deu::DeviceScope ds(g->device);
        deu::k_set_time<<<1, 1, 0, g->st>>>(g->ctl, t);
        g->launches++;
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_get_time(eu_grid* h, double* t) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!t) throw SphError(SPH_ERR_ARG, "null output pointer");
        deu::DeviceScope ds(g->device);
        *t = g->read_ctl().t;
    });
}

int eu_synchronize(eu_grid* h) {
    return guard([&] {
        deu::Grid* g = G(h);
        deu::DeviceScope ds(g->device);
        EU_CUDA(cudaStreamSynchronize(g->st));
    });
}

int eu_event_record(eu_grid* h, int32_t slot) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (slot < 0 || slot >= 8) throw SphError(SPH_ERR_ARG, "event slot must be 0..7");
        deu::DeviceScope ds(g->device);
        EU_CUDA(cudaEventRecord(g->ev[slot], g->st));
    });
}

int eu_event_elapsed(eu_grid* h, int32_t a, int32_t b, double* ms) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) throw SphError(SPH_ERR_ARG, "bad event slots");
        deu::DeviceScope ds(g->device);
        EU_CUDA(cudaEventSynchronize(g->ev[b]));
        float f = 0;
        EU_CUDA(cudaEventElapsedTime(&f, g->ev[a], g->ev[b]));
        *ms = f;
    });
}

int eu_device_bytes(const eu_grid* h, int64_t* bytes) {
    return guard([&] {
        if (!bytes) throw SphError(SPH_ERR_ARG, "null output pointer");
        *bytes = G(const_cast<eu_grid*>(h))->bytes;
    });
}

int eu_launches(const eu_grid* h, int64_t* launches) {
    return guard([&] {
        if (!launches) throw SphError(SPH_ERR_ARG, "null output pointer");
        *launches = G(const_cast<eu_grid*>(h))->launches;
    });
}

}  // extern "C"
