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
#include <cstddef>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "deorbit_euler.h"
#include "engine.hpp"
#include "euler_kernels.cuh"

static_assert(EU_DRIVER_PIN_STRESS == deu::DRV_PIN_STRESS && EU_DRIVER_VOID_AMBIENT == deu::DRV_VOID_AMBIENT &&
                  EU_DRIVER_TRACK_PMAX == deu::DRV_TRACK_PMAX,
              "driver flags of the C ABI and the kernel agree");

namespace dsph {
void set_error_message(const std::string& m);
}

namespace deu {

using dsph::SphError;

// ---------------------------------------------------------------- implicit viscosity

// implicit_visc (hydro_cpu.cpp:286-377): backward Euler for
// d(rho v)/dt = div(eta grad v), eta = af ETA_AF in fluidized cells, each
// velocity component solved by Jacobi-preconditioned conjugate gradients to a
// relative residual of 1e-8, the kinetic energy removed returned as heat.
//
// One persistent cooperative launch does the whole update: the face
// coefficients and the diagonal, the three solves and the heating, separated
// by grid-wide barriers (two per CG iteration: after A p with its p.Ap sum,
// after the x / r / z update with its r.r and r.z sums).  Every per-cell
// expression is the reference's, in its order; the direction update
// p = z + beta p is formed again at each stencil point of A p (the same bits
// as the stored value), which saves a third barrier per iteration.  Sums are
// per-block partials combined in block order by every block alike, so every
// block holds the same scalars and the result does not depend on timing (the
// partials alternate between two sets: a block that has passed the next
// barrier cannot overwrite a set another block is still reading); the
// order differs from the reference's serial sums, so the solution agrees with
// the reference to the solver's tolerance, not bit for bit.

struct Visc {
    double *eta, *cfx, *cfy, *cfz, *dax, *dsum;
    double* x[3];  // u1 v1 w1
    double *rr, *zz, *pp[2], *qq;
    double* part;  // per-block partial sums, two sets of [3][nblk] used in turn
    int nblk;
};

// Polls of the barrier generation before a block gives up (~0.1-1 s).
constexpr long long kBarrierPolls = 1ll << 21;

// Grid-wide barrier of the persistent launch; all blocks are co-resident (the
// launch is cooperative).  The wait is bounded: a block whose poll limit runs
// out records the error, any block that sees the error stops waiting, and the
// kernel returns; the host reads the flag after the step.
static __device__ bool grid_barrier(Ctl* ctl, unsigned nblk) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = &ctl->bar_gen;
        volatile int* err = &ctl->visc_err;
        const unsigned g0 = *gen;
        __threadfence();
        if (atomicAdd(&ctl->bar_count, 1u) == nblk - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            long long polls = 0;
            while (*gen == g0 && *err == 0) {
                if (++polls > kBarrierPolls) {
                    atomicExch(&ctl->visc_err, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok = *err == 0;
    }
    __syncthreads();
    return ok != 0;
}

// The block's sums of K per-thread values into part[k * nblk + block].
template <int K>
static __device__ void block_partials(const double (&v)[K], double* part, unsigned nblk) {
    __shared__ double sh[K][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
        double s = v[k];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sh[k][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < K; k++) {
            double s = sh[k][0];
            for (int w = 1; w < (int)(blockDim.x >> 5); w++) s += sh[k][w];
            part[(int64_t)k * nblk + blockIdx.x] = s;
        }
}

// Grid total of partial k, the same value in every thread of every block.
static __device__ double grid_total(const double* part, int k, unsigned nblk) {
    const int lane = threadIdx.x & 31;
    double s = 0;
    for (unsigned b = lane; b < nblk; b += 32) s += __ldcg(part + (int64_t)k * nblk + b);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
}

static __device__ __forceinline__ double harmonic(double a, double b) {
    return (a > 0 && b > 0) ? 2.0 * a * b / (a + b) : 0.0;
}

static __global__ void __launch_bounds__(256, 3) k_implicit_visc(P p, Fields g, Visc w, Ctl* ctl) {
    if (!ctl->active) return;
    const double dt = ctl->dt, dx = p.dx, rmin = dmax2(p.rho_cfl, 1e-12);
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const bool ax = p.axisym != 0;
    const int64_t n = p.n, sx = (int64_t)ny * nz, sy = nz;
    const unsigned nb = gridDim.x;
    const int64_t c0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (int64_t)nb * blockDim.x;
    const double* r = g.q[F_R];
    int ph = 0;  // the partial set of the next sum
    auto sums = [&]() {
        double* s = w.part + (int64_t)ph * 3 * nb;
        ph ^= 1;
        return s;
    };
    auto ijk = [&](int64_t c, int& i, int& j, int& k) {
        i = (int)(c / sx);
        j = (int)((c / nz) % ny);
        k = (int)(c % nz);
    };
    auto cell_volume = [&](int i) {  // hydro_cpu.cpp:309
        const double rc = (i + 0.5) * dx, wV = ax ? rc : dx;
        return wV * dx * dx;
    };

    // fluidized cells and their viscosity
    {
        double v[1] = {0};
        for (int64_t c = c0; c < n; c += stride) {
            const bool on = r[c] > rmin && g.q[F_AF][c] > 1e-3;
            w.eta[c] = on ? g.q[F_AF][c] * p.eta_af : 0.0;
            v[0] += on ? 1.0 : 0.0;
        }
        double* part = sums();
        block_partials<1>(v, part, nb);
        if (!grid_barrier(ctl, nb)) return;
        if (grid_total(part, 0, nb) == 0) return;  // nothing fluidized: no change
    }
    // face coefficients dt A_f eta_f / dx and the curvature diagonal
    for (int64_t c = c0; c < n; c += stride) {
        int i, j, k;
        ijk(c, i, j, k);
        const double e = __ldcg(w.eta + c), rc = (i + 0.5) * dx, wV = ax ? rc : dx, Vc = wV * dx * dx;
        w.cfx[c] = i < nx - 1 ? dt * (ax ? (i + 1) * dx : dx) * harmonic(e, __ldcg(w.eta + c + sx)) : 0.0;
        w.cfy[c] = (ny > 1 && j < ny - 1) ? dt * dx * harmonic(e, __ldcg(w.eta + c + sy)) : 0.0;
        w.cfz[c] = k < nz - 1 ? dt * wV * harmonic(e, __ldcg(w.eta + c + 1)) : 0.0;
        w.dax[c] = ax ? dt * e * Vc / (rc * rc) : 0.0;
    }
    if (!grid_barrier(ctl, nb)) return;
    // diagonal: the cell's mass and every face coefficient it touches, added
    // in the order of the reference's scatter loop (hydro_cpu.cpp:315-319)
    for (int64_t c = c0; c < n; c += stride) {
        int i, j, k;
        ijk(c, i, j, k);
        double s = r[c] * cell_volume(i);
        if (i > 0) s += __ldcg(w.cfx + c - sx);
        if (ny > 1 && j > 0) s += __ldcg(w.cfy + c - sy);
        if (k > 0) s += __ldcg(w.cfz + c - 1);
        if (i < nx - 1) s += __ldcg(w.cfx + c);
        if (ny > 1 && j < ny - 1) s += __ldcg(w.cfy + c);
        if (k < nz - 1) s += __ldcg(w.cfz + c);
        w.dsum[c] = s;
    }
    if (!grid_barrier(ctl, nb)) return;

    // y = A x at cell c (hydro_cpu.cpp:321-331), x given per cell by xv
    auto amul = [&](int64_t c, int i, int j, int k, bool wd, auto xv) {
        double s = (__ldcg(w.dsum + c) + (wd ? __ldcg(w.dax + c) : 0.0)) * xv(c);
        if (i < nx - 1) s -= __ldcg(w.cfx + c) * xv(c + sx);
        if (i > 0) s -= __ldcg(w.cfx + c - sx) * xv(c - sx);
        if (ny > 1) {
            if (j < ny - 1) s -= __ldcg(w.cfy + c) * xv(c + sy);
            if (j > 0) s -= __ldcg(w.cfy + c - sy) * xv(c - sy);
        }
        if (k < nz - 1) s -= __ldcg(w.cfz + c) * xv(c + 1);
        if (k > 0) s -= __ldcg(w.cfz + c - 1) * xv(c - 1);
        return s;
    };
    auto diag = [&](int64_t c, bool wd) { return __ldcg(w.dsum + c) + (wd ? __ldcg(w.dax + c) : 0.0); };

    for (int m = 0; m < 3; m++) {  // u and the hoop component carry -v/r^2, w does not
        const bool wd = m < 2 && ax;
        double* x = m == 0 ? w.x[0] : (m == 1 ? w.x[1] : w.x[2]);
        const double* mom = m == 0 ? g.q[F_MU] : (m == 1 ? g.q[F_MV] : g.q[F_MW]);
        double bn, rn, rz;
        {  // initial guess: the current velocity; right-hand side Vc (rho v)
            double v[1] = {0};
            for (int64_t c = c0; c < n; c += stride) {
                const double b = cell_volume((int)(c / sx)) * mom[c];
                x[c] = mom[c] / r[c];
                v[0] += b * b;
            }
            double* part = sums();
            block_partials<1>(v, part, nb);
            if (!grid_barrier(ctl, nb)) return;
            bn = grid_total(part, 0, nb);
        }
        if (bn <= 0) {
            for (int64_t c = c0; c < n; c += stride) x[c] = 0;
            continue;
        }
        {  // r = b - A x, z = r / diag, p = z
            double v[2] = {0, 0};
            for (int64_t c = c0; c < n; c += stride) {
                int i, j, k;
                ijk(c, i, j, k);
                const double q = amul(c, i, j, k, wd, [&](int64_t cc) { return __ldcg(x + cc); });
                const double rv = cell_volume(i) * mom[c] - q;
                const double zv = rv / diag(c, wd);
                w.rr[c] = rv;
                w.zz[c] = zv;
                w.pp[0][c] = zv;
                v[0] += rv * rv;
                v[1] += rv * zv;
            }
            double* part = sums();
            block_partials<2>(v, part, nb);
            if (!grid_barrier(ctl, nb)) return;
            rn = grid_total(part, 0, nb);
            rz = grid_total(part, 1, nb);
        }
        const double tol2 = 1e-16 * bn;
        int cur = 0;
        double be = 0;
        for (int it = 0; it < 800 && rn > tol2; it++) {
            double pq;
            {  // p = z + beta p (after the first iteration), q = A p
                const double* po = cur ? w.pp[1] : w.pp[0];
                double* pn = cur ? w.pp[0] : w.pp[1];
                const bool first = it == 0;
                auto pv = [&](int64_t cc) {
                    return first ? __ldcg(po + cc) : __ldcg(w.zz + cc) + be * __ldcg(po + cc);
                };
                double v[1] = {0};
                for (int64_t c = c0; c < n; c += stride) {
                    int i, j, k;
                    ijk(c, i, j, k);
                    const double pc = pv(c);
                    if (!first) pn[c] = pc;
                    const double q = amul(c, i, j, k, wd, pv);
                    w.qq[c] = q;
                    v[0] += pc * q;
                }
                if (!first) cur ^= 1;
                double* part = sums();
                block_partials<1>(v, part, nb);
                if (!grid_barrier(ctl, nb)) return;
                pq = grid_total(part, 0, nb);
            }
            if (pq <= 0) break;
            const double al = rz / pq;
            double rz2;
            {  // x += alpha p, r -= alpha q, z = r / diag
                const double* pc = cur ? w.pp[1] : w.pp[0];
                double v[2] = {0, 0};
                for (int64_t c = c0; c < n; c += stride) {
                    x[c] += al * pc[c];
                    const double rv = w.rr[c] - al * w.qq[c];
                    w.rr[c] = rv;
                    const double zv = rv / diag(c, wd);
                    w.zz[c] = zv;
                    v[0] += rv * rv;
                    v[1] += rv * zv;
                }
                double* part = sums();
                block_partials<2>(v, part, nb);
                if (!grid_barrier(ctl, nb)) return;
                rn = grid_total(part, 0, nb);
                rz2 = grid_total(part, 1, nb);
            }
            if (blockIdx.x == 0 && threadIdx.x == 0) ctl->visc_iters++;
            if (rn <= tol2) break;
            be = rz2 / rz;
            rz = rz2;
        }
    }
    if (!grid_barrier(ctl, nb)) return;  // every cell's new velocity in place

    // heating: the kinetic energy removed, spread over the cells in
    // proportion to the dissipation of their faces (hydro_cpu.cpp:355-376)
    const double *u1 = w.x[0], *v1 = w.x[1], *w1 = w.x[2];
    auto face_heat = [&](int64_t a, int64_t b, double cf) {  // a is the lower cell
        const double du = __ldcg(u1 + a) - __ldcg(u1 + b), dv = __ldcg(v1 + a) - __ldcg(v1 + b),
                     dw = __ldcg(w1 + a) - __ldcg(w1 + b);
        return cf * (du * du + dv * dv + dw * dw);
    };
    double sc;
    {
        double v[3] = {0, 0, 0};
        for (int64_t c = c0; c < n; c += stride) {
            int i, j, k;
            ijk(c, i, j, k);
            const double rho = r[c], mu = g.q[F_MU][c], mv = g.q[F_MV][c], mw = g.q[F_MW][c];
            const double uc = __ldcg(u1 + c), vc = __ldcg(v1 + c), wc = __ldcg(w1 + c), Vc = cell_volume(i);
            const double keo = 0.5 * (mu * mu + mv * mv + mw * mw) / rho;
            const double ken = 0.5 * rho * (uc * uc + vc * vc + wc * wc);
            v[0] += keo * Vc;
            v[1] += ken * Vc;
            const double fx = __ldcg(w.cfx + c), fy = __ldcg(w.cfy + c), fz = __ldcg(w.cfz + c), fa = __ldcg(w.dax + c);
            if (i < nx - 1 && fx > 0) v[2] += face_heat(c, c + sx, fx);
            if (ny > 1 && j < ny - 1 && fy > 0) v[2] += face_heat(c, c + sy, fy);
            if (k < nz - 1 && fz > 0) v[2] += face_heat(c, c + 1, fz);
            if (ax && fa > 0) v[2] += fa * (uc * uc + vc * vc);
        }
        double* part = sums();
        block_partials<3>(v, part, nb);
        if (!grid_barrier(ctl, nb)) return;
        const double totold = grid_total(part, 0, nb), totnew = grid_total(part, 1, nb),
                     htot = grid_total(part, 2, nb);
        const double loss = totold - totnew;
        sc = (loss > 0 && htot > 0) ? loss / htot : 0.0;
    }
    for (int64_t c = c0; c < n; c += stride) {
        int i, j, k;
        ijk(c, i, j, k);
        // this cell's share of its faces' dissipation, in the reference's order
        double hr = 0;
        if (i > 0 && __ldcg(w.cfx + c - sx) > 0) hr += 0.5 * face_heat(c - sx, c, __ldcg(w.cfx + c - sx));
        if (ny > 1 && j > 0 && __ldcg(w.cfy + c - sy) > 0) hr += 0.5 * face_heat(c - sy, c, __ldcg(w.cfy + c - sy));
        if (k > 0 && __ldcg(w.cfz + c - 1) > 0) hr += 0.5 * face_heat(c - 1, c, __ldcg(w.cfz + c - 1));
        if (i < nx - 1 && __ldcg(w.cfx + c) > 0) hr += 0.5 * face_heat(c, c + sx, __ldcg(w.cfx + c));
        if (ny > 1 && j < ny - 1 && __ldcg(w.cfy + c) > 0) hr += 0.5 * face_heat(c, c + sy, __ldcg(w.cfy + c));
        if (k < nz - 1 && __ldcg(w.cfz + c) > 0) hr += 0.5 * face_heat(c, c + 1, __ldcg(w.cfz + c));
        const double uc = __ldcg(u1 + c), vc = __ldcg(v1 + c), wc = __ldcg(w1 + c);
        if (ax && __ldcg(w.dax + c) > 0) hr += __ldcg(w.dax + c) * (uc * uc + vc * vc);
        const double rho = r[c];
        double& mu = g.q[F_MU][c];
        double& mv = g.q[F_MV][c];
        double& mw = g.q[F_MW][c];
        const double keo = 0.5 * (mu * mu + mv * mv + mw * mw) / rho;
        mu = rho * uc;
        mv = rho * vc;
        mw = rho * wc;
        const double ken = 0.5 * (mu * mu + mv * mv + mw * mw) / rho;
        double q = sc * hr / cell_volume(i);
        if (p.af_reg && q > 0) {  // C_REG of the dissipation regenerates vibrations
            g.q[F_VIB][c] = sqrt(g.q[F_VIB][c] * g.q[F_VIB][c] + 2.0 * p.c_reg * q / rho);
            q *= (1.0 - p.c_reg);
        }
        g.q[F_E][c] += (ken - keo) + q;
    }
}

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
    double* ref_dp = nullptr;   // its well-balanced gravity face-pressure difference
    std::vector<void*> allocs;
    int64_t bytes = 0;
    int64_t launches = 0;
    cudaEvent_t ev[8] = {};
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    int64_t graph_launches = 0;  // kernels per replay of the step graph
    Visc vw{};                   // implicit viscosity work arrays, allocated on first use
    FaceFork fork{};             // side streams for the face passes (small grids)
    bool fork_faces = false;
    int pin_floor = 0;           // driver adjustments after each step (eu_set_driver)
    int sponge_from = -1;
    int driver_flags = 0;

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
        for (cudaEvent_t e : {fork.fork, fork.join[0], fork.join[1]})
            if (e) cudaEventDestroy(e);
        for (cudaStream_t s2 : fork.side)
            if (s2) cudaStreamDestroy(s2);
        for (void* a : allocs) cudaFree(a);
        allocs.clear();
        if (st) cudaStreamDestroy(st);
        st = nullptr;
    }

    unsigned grid_of(int64_t count) const { return (unsigned)((count + 255) / 256); }

    bool visc_on() const { return p.visc_imp && p.eta_af > 0; }

    // The persistent launch's blocks: as many as fit on the device at once
    // (a cooperative launch needs all of them resident), at most one per 256
    // cells.
    void ensure_visc() {
        if (vw.eta) return;
        int dev_coop = 0, nsm = 0, per_sm = 0;
        EU_CUDA(cudaDeviceGetAttribute(&dev_coop, cudaDevAttrCooperativeLaunch, device));
        if (!dev_coop) throw SphError(SPH_ERR_CUDA, "the implicit viscosity needs cooperative launches");
        EU_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
        EU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_implicit_visc, 256, 0));
        if (per_sm < 1) throw SphError(SPH_ERR_CUDA, "implicit viscosity kernel does not fit on an SM");
        const int64_t want = std::max<int64_t>(1, (p.n + 255) / 256);
        vw.nblk = (int)std::min<int64_t>(want, (int64_t)per_sm * nsm);
        for (double** a : {&vw.eta, &vw.cfx, &vw.cfy, &vw.cfz, &vw.dax, &vw.dsum, &vw.x[0], &vw.x[1], &vw.x[2],
                           &vw.rr, &vw.zz, &vw.pp[0], &vw.pp[1], &vw.qq})
            *a = alloc(p.n);
        vw.part = alloc(6 * (int64_t)vw.nblk);
    }

    void enqueue_visc() {
        ensure_visc();
        static_assert(offsetof(Ctl, visc_err) == offsetof(Ctl, bar_count) + 4, "barrier fields are adjacent");
        EU_CUDA(cudaMemsetAsync(&ctl->bar_count, 0, 8, st));  // barrier count and error flag
        P pv = p;
        Fields gv = g;
        Visc wv = vw;
        Ctl* cv = ctl;
        void* args[] = {&pv, &gv, &wv, &cv};
        EU_CUDA(cudaLaunchCooperativeKernel((const void*)k_implicit_visc, dim3((unsigned)vw.nblk), dim3(256), args, 0, st));
        launches++;
    }

    void enqueue_lop(const Fields& s) {
        const FaceFork* fk = fork_faces ? &fork : nullptr;
        EU_CUDA(mixed ? enqueue_lop_f32(p, s, W32, g.q[F_AF], F32, d, ctl, st, fk)
                      : enqueue_lop_t<double>(p, s, W, g.q[F_AF], F, d, ctl, st, fk));
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
        const bool vi = visc_on();
        if (mixed) enqueue_correct_f32(p, g, g1, d, ctl, st, vi ? 1 : 0);
        else enqueue_correct_t<double>(p, g, g1, d, ctl, st, vi ? 1 : 0);
        if (vi) {  // implicit_visc between the average and the rest (hydro_cpu.cpp:420)
            enqueue_visc();
            if (mixed) enqueue_correct_f32(p, g, g1, d, ctl, st, 2);
            else enqueue_correct_t<double>(p, g, g1, d, ctl, st, 2);
            launches++;
        }
        if (pin_floor > 0 || sponge_from >= 0 || driver_flags) {
            if ((pin_floor > 0 || sponge_from >= 0) && !p.ref_r0)
                throw SphError(SPH_ERR_STATE, "the floor pin and sponge need a reference state (eu_set_ref)");
            k_driver<<<grid_of(p.n), 256, 0, st>>>(p, g, ctl, pin_floor, sponge_from, driver_flags);
            launches++;
        }
        k_end<<<1, 1, 0, st>>>(ctl);
        launches += 3;
        if (p.void_cons && p.ref_r0 && p.rho_cfl > 0) launches += 3;
    }

    void check_visc(const Ctl& c) {
        if (c.visc_err)
            throw SphError(SPH_ERR_STATE, "implicit viscosity: a grid-wide barrier wait ran out (device busy?)");
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
    p.visc_imp = e.visc_imp != 0;
}

// Weakest-flaw activation strain of grow_damage (hydro_cpu.cpp:254), formed
// on the host with the host library's pow.
void derive(deu::P& p) {
    const deu::Mat& m = p.m;
    p.mf = deu::mat_as<float>(m);
    p.eps_act = (m.Emod > 0 && m.wk > 0) ? std::pow(1.0 / (m.wk * p.dx * p.dx * p.dx), 1.0 / m.wm) : 0.0;
    p.invdx = 1.0 / p.dx;
    p.cf.y_i0 = (float)p.y_i0; p.cf.mu_i = (float)p.mu_i; p.cf.ymi = (float)(p.y_m - p.y_i0);
    p.cf.y_d0 = (float)p.y_d0; p.cf.mu_d = (float)p.mu_d; p.cf.y_m = (float)p.y_m;
    p.cf.y_bingham = (float)p.y_bingham; p.cf.c_reg = (float)p.c_reg; p.cf.eps_act = (float)p.eps_act;
    p.cf.dx = (float)p.dx; p.cf.invdx = (float)p.invdx; p.cf.rho_vac = (float)p.rho_vac;
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
            if (g->mixed) {  // FP32 strength fields and near-void flags of the right-hand side
                for (int q = 0; q < 8; q++) g->W32.sq[q] = g->alloc<float>(n);
                g->W32.vd = g->alloc<uint8_t>(n);
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
            // Small grids: the three face passes of a Lop fill the device only
            // side by side (a pass of a 2-D grid is a few dozen blocks).
            int nsm = 0;
            EU_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
            g->fork_faces = n < (int64_t)nsm * 256 * 8;
            if (g->fork_faces) {
                for (auto& s2 : g->fork.side) EU_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
                EU_CUDA(cudaEventCreateWithFlags(&g->fork.fork, cudaEventDisableTiming));
                for (auto& e : g->fork.join) EU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            }
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
        if (g->p.ref_r0) {  // the gravity source's reference pressures follow the material
            deu::DeviceScope ds(g->device);
            deu::k_ref_dp<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->ref_r0, g->ref_dp);
            g->launches++;
            g->check();
            EU_CUDA(cudaStreamSynchronize(g->st));
        }
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
        derive(g->p);  // the FP32 copies of the settings
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
            g->ref_dp = g->alloc(g->p.n);
        }
        deu::k_set_ref<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->g, g->ref_r0, g->ref_p0);
        deu::k_ref_dp<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->ref_r0, g->ref_dp);
        g->launches += 2;
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
        g->p.ref_r0 = g->ref_r0;
        g->p.ref_p0 = g->ref_p0;
        g->p.ref_dp = g->ref_dp;
        g->graph_valid = false;
    });
}

int eu_clear_ref(eu_grid* h) {
    return guard([&] {
        deu::Grid* g = G(h);
        g->pin_floor = 0;  // the floor pin and sponge act toward the reference
        g->sponge_from = -1;
        g->p.ref_r0 = nullptr;
        g->p.ref_p0 = nullptr;
        g->p.ref_dp = nullptr;
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
        if (g->visc_on()) g->check_visc(g->read_ctl());
    });
}

int eu_set_driver(eu_grid* h, int32_t pin_floor, int32_t sponge_from, int32_t flags) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (pin_floor < 0 || pin_floor > g->p.nz) throw SphError(SPH_ERR_ARG, "pin_floor must be in [0, nz]");
        if (sponge_from >= g->p.nx) throw SphError(SPH_ERR_ARG, "sponge_from must be < nx (or negative: off)");
        if (flags & ~(EU_DRIVER_PIN_STRESS | EU_DRIVER_VOID_AMBIENT | EU_DRIVER_TRACK_PMAX))
            throw SphError(SPH_ERR_ARG, "unknown driver flag");
        if ((pin_floor > 0 || sponge_from >= 0) && !g->p.ref_r0)
            throw SphError(SPH_ERR_STATE, "the floor pin and sponge need a reference state (eu_set_ref)");
        const int isp = sponge_from < 0 ? -1 : sponge_from;
        if (pin_floor == g->pin_floor && isp == g->sponge_from && flags == g->driver_flags) return;
        g->pin_floor = pin_floor;
        g->sponge_from = isp;
        g->driver_flags = flags;
        g->graph_valid = false;  // the step graph holds the adjustments
    });
}

int eu_implicit_visc(eu_grid* h, double dt) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!(dt >= 0) || !std::isfinite(dt)) throw SphError(SPH_ERR_ARG, "dt must be finite and >= 0");
        deu::DeviceScope ds(g->device);
        if (g->visc_on()) {  // implicit_visc returns at once otherwise (hydro_cpu.cpp:302)
            deu::k_set_step<<<1, 1, 0, g->st>>>(g->ctl, dt);
            g->launches++;
            g->enqueue_visc();
        }
        g->check();
        EU_CUDA(cudaStreamSynchronize(g->st));
        g->check_visc(g->read_ctl());
    });
}

int eu_visc_iterations(eu_grid* h, int64_t* iters) {
    return guard([&] {
        deu::Grid* g = G(h);
        if (!iters) throw SphError(SPH_ERR_ARG, "null output pointer");
        deu::DeviceScope ds(g->device);
        *iters = g->read_ctl().visc_iters;
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
        // The implicit viscosity's cooperative launch is issued directly, not
        // from a graph: steps with it are enqueued one by one.
        const bool direct = g->visc_on();
        if (!direct && !g->graph_valid) {  // one driver step, captured once per settings
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
            g->graph_launches = g->launches - l0;
            g->launches = l0;
            g->graph_valid = true;
        }
        const int64_t limit = c0.max_steps;  // absolute step count, -1 = none
        deu::Ctl c = c0;
        // replay in chunks; steps past the end are no-ops (inactive control)
        int chunk = 4;
        while (c.t < c.t_end && (limit < 0 || c.steps < limit)) {
            int todo = chunk;
            if (limit >= 0) todo = (int)std::min<int64_t>(todo, limit - c.steps);
            for (int i = 0; i < todo; i++) {
                if (direct) {
                    g->enqueue_step(true);
                } else {
                    EU_CUDA(cudaGraphLaunch(g->graph, g->st));
                    g->launches += g->graph_launches;
                }
            }
            const double t_prev = c.t;
            c = g->read_ctl();
            g->check_visc(c);
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
