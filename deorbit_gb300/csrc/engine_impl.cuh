// engine_impl.cuh -- host orchestration of the SPH engine, templated on the
// arithmetic type R of per-particle fields and pair interactions.
// Instantiated for double (plain form) and float (mixed form).
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "engine.hpp"
#include "engine_kernels.cuh"
#include "scan_sort.cuh"

namespace dsph {

// A failed runtime call becomes an exception; the thread's last-error state is
// cleared so that a later, unrelated check does not report it again.
#define DSPH_CUDA(x)                                                                    \
    do {                                                                                \
        cudaError_t e_ = (x);                                                           \
        if (e_ != cudaSuccess) {                                                        \
            cudaGetLastError();                                                         \
            throw SphError(SPH_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
        }                                                                               \
    } while (0)

// ----------------------------------------------------------------- aux kernels
template <class T>
static __global__ void k_read_col(const T* col, const int32_t* pos_of_gid, int64_t gid_base, int64_t n,
                           double* out) {
    int64_t l = gtid();
    if (l >= n) return;
    out[l] = (double)col[pos_of_gid[gid_base + l]];
}
template <class T>
static __global__ void k_write_col(T* col, const int32_t* pos_of_gid, int64_t gid_base, int64_t n,
                            const double* in) {
    int64_t l = gtid();
    if (l >= n) return;
    col[pos_of_gid[gid_base + l]] = (T)in[l];
}
// Up to kColIo columns in one launch (step_fields): column c holds doubles,
// or floats where f32[c] (the mixed form's FP32 columns), converted as
// k_read_col / k_write_col convert them.
constexpr int kColIo = 16;
struct ColIo {
    void* col[kColIo];
    double* buf[kColIo];
    int32_t f32[kColIo];
    int32_t nc;
};
static __global__ void k_write_cols(ColIo s, const int32_t* pos_of_gid, int64_t gid_base, int64_t n) {
    int64_t l = gtid();
    if (l >= n) return;
    const int32_t k = pos_of_gid[gid_base + l];
    for (int c = 0; c < s.nc; c++) {
        const double v = s.buf[c][l];
        if (s.f32[c]) static_cast<float*>(s.col[c])[k] = (float)v;
        else static_cast<double*>(s.col[c])[k] = v;
    }
}
static __global__ void k_read_cols(ColIo s, const int32_t* pos_of_gid, int64_t gid_base, int64_t n) {
    int64_t l = gtid();
    if (l >= n) return;
    const int32_t k = pos_of_gid[gid_base + l];
    for (int c = 0; c < s.nc; c++)
        s.buf[c][l] = s.f32[c] ? (double)static_cast<const float*>(s.col[c])[k]
                               : static_cast<const double*>(s.col[c])[k];
}
static __global__ void k_read_u8(const uint8_t* col, const int32_t* pos_of_gid, int64_t gid_base,
                          int64_t n, uint8_t* out) {
    int64_t l = gtid();
    if (l >= n) return;
    out[l] = col[pos_of_gid[gid_base + l]];
}
static __global__ void k_write_u8(uint8_t* col, const int32_t* pos_of_gid, int64_t gid_base, int64_t n,
                           const uint8_t* in) {
    int64_t l = gtid();
    if (l >= n) return;
    col[pos_of_gid[gid_base + l]] = in[l];
}

template <class R>
static __global__ void k_eos_eval(const MatT<R>* mats, int mat, int64_t n, const double* rho,
                           const double* u, double* P, double* cs) {
    int64_t k = gtid();
    if (k >= n) return;
    R p, c;
    eos_P_cs(mats[mat], (R)rho[k], (R)u[k], p, c);
    P[k] = (double)p;
    cs[k] = (double)c;
}

// Reference cell id (linear, sph.hpp:160) of every particle of an impact, in
// gid order, for the on-device reference cell sort.
template <class R>
static __global__ void k_ref_keys(View<R> v, int b, const int32_t* pos_of_gid, int64_t gid_base,
                           int64_t n, uint32_t* keys, int32_t* counts) {
    int64_t l = gtid();
    if (l >= n) return;
    const ImpactD& I = v.imps[b];
    int64_t k = pos_of_gid[gid_base + l];
    unsigned long long rb = v.refbin[k];
    int64_t c = ((int64_t)(rb & 0x1fffff) * I.nc[1] + (int64_t)((rb >> 21) & 0x1fffff)) * I.nc[2] +
                (int64_t)((rb >> 42) & 0x1fffff);
    const int64_t ncell = (int64_t)I.nc[0] * I.nc[1] * I.nc[2];
    if (c < 0 || c >= ncell) c = ncell;  // stale bins: parked past the last cell
    keys[l] = (uint32_t)c;
    atomicAdd(&counts[c], 1);
}

// Exact neighbour sets (FP64 criteria) for the parity hook: with offs null
// only the counts, else the set of sorted position idx at out[offs[idx]...].
template <class R>
static __global__ void k_debug_nbr(View<R> v, int b, int kind, int32_t* out, int32_t* cnt_out,
                                   const int64_t* offs) {
    int64_t idx = gtid();
    const ImpactD& I = v.imps[b];
    if (idx >= I.n) return;
    const int64_t k = I.off + idx;
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    const unsigned long long bi = v.refbin[k];
    const float m = 4.0f * I.margin + 1e-6f * (pi.w + I.hmax_f);
    const float Rs = (kind == 0 ? 2.0f * pi.w : pi.w + I.hmax_f) + 2.0f * m;
    const double hi = (double)v.hh[k];
    int cnt = 0;
    traverse<R, true>(v, I, pi, ci, Rs, [&](int32_t j, float, float, float) {
        if (!ref_member(bi, v.refbin[j], I)) return;
        double dx, dy, dz;
        double r = sep_exact(v, I, k, j, dx, dy, dz);
        bool take;
        if (kind == 0) {
            take = r < 2.0 * hi;
        } else {
            double hsum = __dadd_rn(hi, (double)v.hh[j]);
            take = !(j == (int32_t)k || r >= hsum || r == 0.0);
        }
        if (take) {
            if (offs) out[offs[idx] + cnt] = v.gid[j] - (int32_t)I.gid_base;
            cnt++;
        }
    });
    if (!offs) cnt_out[idx] = cnt;
}

// Compensated FP64 conservation sums of one impact, fixed summation order.
template <class R>
static __global__ void k_conservation(View<R> v, int b, double* out) {
    __shared__ double sh[8][256];
    const ImpactD& I = v.imps[b];
    double s[8], c[8];
    for (int q = 0; q < 8; q++) s[q] = c[q] = 0.0;
    for (int64_t idx = threadIdx.x; idx < I.n; idx += blockDim.x) {
        int64_t k = I.off + idx;
        double m = (double)v.mass[k];
        double vx = v.vx[k], vy = v.vy[k], vz = v.vz[k];
        double val[7] = {m, 0.5 * m * (vx * vx + vy * vy + vz * vz), m * v.u[k], m * vx, m * vy, m * vz, 0.0};
        for (int q = 0; q < 6; q++) {
            double y = val[q] - c[q];
            double t = s[q] + y;
            c[q] = (t - s[q]) - y;
            s[q] = t;
        }
    }
    for (int q = 0; q < 6; q++) sh[q][threadIdx.x] = s[q] - c[q];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int q = 0; q < 6; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 6; q++) out[q] = sh[q][0];
}

// Projectile diagnostics of one impact (the quantities gpu_ic's progress line
// and the campaign's regime classifier derive from a snapshot,
// gpu_ic.cpp:112-117, boundary_daemon.py:181-212), over the particles with
// mat_lo <= mat <= mat_hi: count, melted count (u > u_melt), position and
// velocity means, mean speed, velocity dispersion, u max.  One block, fixed
// summation order, compensated FP64 sums; the dispersion takes a second pass
// about the mean.  out: [count, melted, mx, my, mz, mvx, mvy, mvz, mspeed,
// dispersion, umax].
__device__ __forceinline__ double block_sum(double x, double* sh) {
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = x;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < nw; i++) t += sh[i];  // same order in every thread
    return t;
}

template <class R>
static __global__ void __launch_bounds__(512) k_diagnostics(View<R> v, int b, int mat_lo, int mat_hi,
                                                            double u_melt, double* out) {
    __shared__ double sh[32];
    const ImpactD& I = v.imps[b];
    double s[9], c[9];
    for (int q = 0; q < 9; q++) s[q] = c[q] = 0.0;
    double umax = -1e300;
    auto kadd = [&](int q, double x) {
        const double y = x - c[q];
        const double t = s[q] + y;
        c[q] = (t - s[q]) - y;
        s[q] = t;
    };
    for (int64_t idx = threadIdx.x; idx < I.n; idx += blockDim.x) {
        const int64_t k = I.off + idx;
        const int m = v.mat[k];
        if (m < mat_lo || m > mat_hi) continue;
        const double vx = v.vx[k], vy = v.vy[k], vz = v.vz[k], u = v.u[k];
        kadd(0, 1.0);
        kadd(1, u > u_melt ? 1.0 : 0.0);
        kadd(2, v.x[k]); kadd(3, v.y[k]); kadd(4, v.z[k]);
        kadd(5, vx); kadd(6, vy); kadd(7, vz);
        kadd(8, sqrt(vx * vx + vy * vy + vz * vz));
        umax = fmax(umax, u);
    }
    double tot[9];
    for (int q = 0; q < 9; q++) tot[q] = block_sum(s[q] - c[q], sh);
    for (int o = 16; o > 0; o >>= 1) umax = fmax(umax, __shfl_xor_sync(0xffffffffu, umax, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = umax;
    __syncthreads();
    double um = -1e300;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) um = fmax(um, sh[i]);
    const double n = tot[0] > 0.0 ? tot[0] : 1.0;
    const double mvx = tot[5] / n, mvy = tot[6] / n, mvz = tot[7] / n;
    double sd = 0.0, cd = 0.0;
    for (int64_t idx = threadIdx.x; idx < I.n; idx += blockDim.x) {
        const int64_t k = I.off + idx;
        const int m = v.mat[k];
        if (m < mat_lo || m > mat_hi) continue;
        const double dx = v.vx[k] - mvx, dy = v.vy[k] - mvy, dz = v.vz[k] - mvz;
        const double y = (dx * dx + dy * dy + dz * dz) - cd;
        const double t = sd + y;
        cd = (t - sd) - y;
        sd = t;
    }
    const double var = block_sum(sd - cd, sh);
    if (threadIdx.x == 0) {
        out[0] = tot[0];
        out[1] = tot[1];
        out[2] = tot[2] / n; out[3] = tot[3] / n; out[4] = tot[4] / n;
        out[5] = mvx; out[6] = mvy; out[7] = mvz;
        out[8] = tot[8] / n;
        out[9] = sqrt(var / n);
        out[10] = tot[0] > 0.0 ? um : 0.0;
    }
}

// After a sort: offsets change, and positions may have (bins are stale).
static __global__ void k_impact_reset_omax(ImpactD* imps, int nimp) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nimp) {
        imps[b].omax_bits = 0u;
        imps[b].bins_ok = 0;
    }
}

static __global__ void k_set_mask_dt(ImpactD* imps, int nimp, const int32_t* mask, const double* dt,
                              const double* t_end) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    imps[b].mask = mask[b];
    if (dt) imps[b].dt = dt[b];
    if (t_end) imps[b].t_end = t_end[b];
}

// Fills for generated impacts.
template <class T>
static __global__ void k_fill(T* p, int64_t n, T v) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
static __global__ void k_gid_iota(int32_t* gid, int32_t* pos_of_gid, int64_t n, int64_t gid_base, int64_t at) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    gid[at + i] = (int32_t)(gid_base + i);
    pos_of_gid[gid_base + i] = (int32_t)(at + i);
}

// Target lattice of the grazing IC (boundary_daemon.py:136-143) at rows
// [at, at + nx ny nz): particle l = (ix ny + iy) nz + iz sits at
// (xs[ix], ys[iy], zs[iz]), at rest, frozen within `wall` of the x / y ends or
// of the bottom layer -- the reference's loop order and comparisons.
template <class R>
static __global__ void k_gen_slab(int64_t at, int nx, int ny, int nz, const double* xs, const double* ys,
                                  const double* zs, double wall, R mass_t, double* x, double* y, double* z,
                                  double* vx, double* vy, double* vz, double* u, R* mass, uint8_t* fixed) {
    const int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= (int64_t)nx * ny * nz) return;
    const int iz = (int)(l % nz);
    const int64_t r = l / nz;
    const int iy = (int)(r % ny), ix = (int)(r / ny);
    const double X = xs[ix], Y = ys[iy], Z = zs[iz];
    const bool fx = fabs(X - xs[0]) < wall || fabs(X - xs[nx - 1]) < wall;
    const bool fxy = fx || fabs(Y - ys[0]) < wall || fabs(Y - ys[ny - 1]) < wall;
    const bool frozen = fxy || Z < zs[nz - 1] + wall;
    const int64_t k = at + l;
    x[k] = X;
    y[k] = Y;
    z[k] = Z;
    vx[k] = 0.0;
    vy[k] = 0.0;
    vz[k] = 0.0;
    u[k] = 0.0;
    mass[k] = mass_t;
    fixed[k] = frozen ? 1 : 0;
}

// ----------------------------------------------------------------- engine
template <class R>
class Engine final : public EngineBase {
public:
    static constexpr int kNR = 21;   // carried R columns
    static constexpr int kND = 7;    // carried FP64 columns: x y z u vx vy vz
    static constexpr int kNDer = 20; // derived R columns
    enum { RC_AX, RC_AY, RC_AZ, RC_DUDT, RC_MASS, RC_HH, RC_D, RC_EPSACT,
           RC_H0, RC_S0, RC_DS0 = RC_S0 + 6 };
    enum { DR_RHO, DR_P, DR_CS, DR_CSIG, DR_PF, DR_DSCALE, DR_RART, DR_SIGMAX, DR_EPSW, DR_PFR2,
           DR_DSR2, DR_VOL, DR_DUDTN, DR_DSN0, DR_RHOLO = DR_DSN0 + 6 };

    struct ImpactH {
        sph_params prm{};
        double dlo[3]{}, dhi[3]{};
        int32_t per[3]{};
        bool used = false, alive = false, committed = false, initialized = false;
        int64_t n = 0, gid_base = 0;
        std::vector<double> sx, sy, sz, svx, svy, svz, smass, su, seps, sh0;
        std::vector<int32_t> smat;
        std::vector<uint8_t> sfixed;
        std::vector<int32_t> mat_host;
        bool use_h0 = false;
        double h0max = 0;
        bool multi = false;
        std::vector<int64_t> flaw_ptr;
        std::vector<double> flaw_eps;
        bool flaws_on_device = false;  // its segment of the device flaw pool is current
        double t = 0, dt_last = 0;
        int64_t steps = 0;
        int64_t step_limit = 0;
        std::shared_ptr<const GrazingLayout> gen;  // particles generated at commit
    };

    explicit Engine(int device) : dev_(device) {
        DSPH_CUDA(cudaSetDevice(dev_));
        DSPH_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
        DSPH_CUDA(cudaStreamCreateWithFlags(&copy_st_, cudaStreamNonBlocking));
        DSPH_CUDA(cudaEventCreateWithFlags(&copy_ev_, cudaEventDisableTiming));
        DSPH_CUDA(cudaStreamCreateWithFlags(&out_st_, cudaStreamNonBlocking));
        DSPH_CUDA(cudaEventCreateWithFlags(&out_ev_, cudaEventDisableTiming));
        DSPH_CUDA(cudaEventCreateWithFlags(&late_ev_, cudaEventDisableTiming));
        DSPH_CUDA(cudaMalloc(&mats_d_, sizeof(MatT<R>) * kMaxMaterials));
        DSPH_CUDA(cudaMalloc(&flags_d_, sizeof(int32_t) * 4));
        DSPH_CUDA(cudaMalloc(&wait_err_d_, sizeof(int32_t)));
        DSPH_CUDA(cudaMemsetAsync(wait_err_d_, 0, sizeof(int32_t), st_));
        DSPH_CUDA(cudaMalloc(&ntask_, sizeof(int32_t)));
        DSPH_CUDA(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev_));
        {
            int pa = 0;
            if (cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, dev_) != cudaSuccess) {
                cudaGetLastError();
                pa = 0;
            }
            pageable_access_ = pa != 0;
        }
        DSPH_CUDA(cudaMallocHost(&flags_h_, sizeof(int32_t) * 4));
        DSPH_CUDA(cudaMemsetAsync(flags_d_, 0, sizeof(int32_t) * 4, st_));
        for (int i = 0; i < 6; i++) DSPH_CUDA(cudaEventCreate(&ev_[i]));
        for (int i = 0; i < 5; i++) phase_ms_[i] = 0;
    }

    ~Engine() override {
        cudaSetDevice(dev_);
        cudaStreamSynchronize(st_);
        for (void* p : allocs_) cudaFree(p);
        cudaFree(mats_d_);
        cudaFree(flags_d_);
        cudaFree(wait_err_d_);
        cudaFree(ntask_);
        cudaFreeHost(flags_h_);
        for (int i = 0; i < 6; i++) cudaEventDestroy(ev_[i]);
        for (auto& e : prof_pool_) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
        for (int g = 0; g < kGraphKinds; g++)
            for (int p = 0; p < 2; p++)
                if (graph_exec_[g][p]) cudaGraphExecDestroy(graph_exec_[g][p]);
        for (int i = 0; i < 16; i++) if (user_ev_[i]) cudaEventDestroy(user_ev_[i]);
        cudaStreamSynchronize(copy_st_);
        cudaStreamSynchronize(out_st_);
        cudaEventDestroy(copy_ev_);
        cudaEventDestroy(out_ev_);
        cudaEventDestroy(late_ev_);
        cudaStreamDestroy(copy_st_);
        cudaStreamDestroy(out_st_);
        cudaStreamDestroy(st_);
    }

    int precision() const override { return sizeof(R) == 8 ? SPH_FP64 : SPH_MIXED; }

    // ------------------------------------------------------------- materials
    int add_material(const sph_material& m) override {
        if ((int)mats_h_.size() >= kMaxMaterials) throw SphError(SPH_ERR_CAPACITY, "too many materials");
        mats_h_.push_back(m);
        upload_materials();
        return (int)mats_h_.size() - 1;
    }

    // ------------------------------------------------------------- impacts
    int impact_create(const sph_params& p, const double dlo[3], const double dhi[3],
                      const int32_t per[3]) override {
        int slot = -1;
        for (size_t b = 0; b < imp_.size(); b++)
            if (!imp_[b].used) { slot = (int)b; break; }
        if (slot < 0) {
            if (imp_.size() >= 65535) throw SphError(SPH_ERR_CAPACITY, "too many impacts");
            imp_.emplace_back();
            slot = (int)imp_.size() - 1;
        }
        ImpactH& h = imp_[slot];
        h = ImpactH();
        h.used = true;
        h.alive = true;
        h.prm = p;
        for (int a = 0; a < 3; a++) {
            h.dlo[a] = dlo ? dlo[a] : 0.0;
            h.dhi[a] = dhi ? dhi[a] : 0.0;
            h.per[a] = per ? (per[a] != 0) : 0;
        }
        return slot;
    }

    ImpactH& imp(int b) {
        if (b < 0 || b >= (int)imp_.size() || !imp_[b].used) throw SphError(SPH_ERR_ARG, "bad impact id");
        return imp_[b];
    }

    int impact_create_generated(const sph_params& p, std::shared_ptr<const GrazingLayout> L) override {
        for (int m : {L->tgt_mat, L->imp_mat})
            if (m < 0 || m >= (int)mats_h_.size()) throw SphError(SPH_ERR_ARG, "material id out of range");
        const int32_t per[3] = {0, 0, 0};
        const int b = impact_create(p, L->dlo, L->dhi, per);
        ImpactH& h = imp_[b];
        h.gen = L;
        h.n = L->n();
        h.mat_host.assign((size_t)h.n, L->imp_mat);
        std::fill(h.mat_host.begin(), h.mat_host.begin() + L->n_slab(), L->tgt_mat);
        return b;
    }

    void impact_set_domain(int b, const double dlo[3], const double dhi[3], const int32_t per[3]) override {
        ImpactH& h = imp(b);
        if (h.committed) throw SphError(SPH_ERR_STATE, "domain is fixed once particles are on the device");
        for (int a = 0; a < 3; a++) { h.dlo[a] = dlo[a]; h.dhi[a] = dhi[a]; h.per[a] = per ? (per[a] != 0) : 0; }
    }

    void impact_set_params(int b, const sph_params& p) override {
        ImpactH& h = imp(b);
        h.prm = p;
        if (h.committed) {
            pull_table();
            fill_params(tab_[b], h);
            push_table();
        }
    }
    sph_params impact_get_params(int b) override { return imp(b).prm; }

    void impact_add_particles(int b, int64_t n, const double* x, const double* y, const double* z,
                              const double* vx, const double* vy, const double* vz,
                              const double* mass, const double* u, const int32_t* mat,
                              const uint8_t* fixed) override {
        ImpactH& h = imp(b);
        if (h.committed) throw SphError(SPH_ERR_STATE, "particles can only be added before init");
        if (h.gen) throw SphError(SPH_ERR_STATE, "the impact holds a generated IC");
        if (n < 0 || (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !mass || !u)))
            throw SphError(SPH_ERR_ARG, "null particle array");
        for (int64_t i = 0; i < n; i++) {
            int32_t m = mat ? mat[i] : 0;
            if (m < 0 || m >= (int)mats_h_.size()) throw SphError(SPH_ERR_ARG, "material id out of range");
        }
        auto app = [n](std::vector<double>& v, const double* s) { v.insert(v.end(), s, s + n); };
        app(h.sx, x); app(h.sy, y); app(h.sz, z);
        app(h.svx, vx); app(h.svy, vy); app(h.svz, vz);
        app(h.smass, mass); app(h.su, u);
        for (int64_t i = 0; i < n; i++) {
            h.smat.push_back(mat ? mat[i] : 0);
            h.sfixed.push_back(fixed ? (fixed[i] ? 1 : 0) : 0);
            h.seps.push_back(1e30);
            h.sh0.push_back(h.prm.h_init);
        }
        h.mat_host.insert(h.mat_host.end(), h.smat.end() - n, h.smat.end());
        h.n += n;
    }

    void impact_seed_damage(int b, double dx, uint32_t seed) override {
        ImpactH& h = imp(b);
        std::vector<double> eps(h.n);
        seed_single_flaws(h.n, h.mat_host.data(), mats_h_.data(), (int)mats_h_.size(), dx, seed, eps.data());
        if (!h.committed) h.seps = eps;
        else write_field(b, "eps_act", eps.data());
    }

    int64_t impact_seed_flaws_multi(int b, double dx, uint32_t seed) override {
        ImpactH& h = imp(b);
        if (h.flaws_on_device) flaw_live_ -= (int64_t)h.flaw_eps.size();  // the old segment is dead
        h.flaws_on_device = false;
        std::vector<double> eps(h.n);
        h.flaw_ptr.assign(h.n + 1, 0);
        double* fe = nullptr;
        int64_t nf = seed_multi_flaws(h.n, h.mat_host.data(), mats_h_.data(), (int)mats_h_.size(), dx,
                                      seed, h.flaw_ptr.data(), &fe, eps.data());
        h.flaw_eps.assign(fe, fe + nf);
        free(fe);
        h.multi = true;
        h.prm.flaw_model = SPH_FLAWS_MULTI;
        if (!h.committed) {
            h.seps = eps;
        } else {
            write_field(b, "eps_act", eps.data());
            pull_table();
            fill_params(tab_[b], h);
            push_table();
            sync_flaws();
        }
        return nf;
    }

    void impact_set_h0(int b, const double* h0) override {
        ImpactH& h = imp(b);
        h.use_h0 = true;
        h.h0max = 0;
        for (int64_t i = 0; i < h.n; i++) h.h0max = std::max(h.h0max, h0[i]);
        if (!h.committed) {
            h.sh0.assign(h0, h0 + h.n);
        } else {
            write_field(b, "h0", h0);
            pull_table();
            fill_params(tab_[b], h);
            push_table();
        }
    }

    void impact_set_flaws(int b, const double* eps_act, const int64_t* ptr, const double* eps,
                          int64_t nflaws) override {
        ImpactH& h = imp(b);
        if (h.committed) throw SphError(SPH_ERR_STATE, "flaws are set before the impact is initialised");
        if (eps_act) h.seps.assign(eps_act, eps_act + h.n);
        if (ptr) {
            if (ptr[0] != 0 || ptr[h.n] != nflaws) throw SphError(SPH_ERR_ARG, "flaw CSR does not match its count");
            h.flaw_ptr.assign(ptr, ptr + h.n + 1);
            h.flaw_eps.assign(eps, eps + nflaws);
            h.multi = true;
            h.prm.flaw_model = SPH_FLAWS_MULTI;
        }
    }

    std::vector<sph_material> materials() override { return mats_h_; }

    // Device bytes per particle of capacity: both carried buffers, derived
    // columns, geometry and force records, reverse lists and the own list at
    // the current list capacity (the allocations of ensure_particle_capacity
    // and alloc_lists), plus the per-id sort arrays.
    int64_t bytes_per_particle() const {
        const int64_t R4 = sizeof(R) == 4;
        int64_t b = 2 * (kND * 8 + kNR * (int64_t)sizeof(R) + 1 + 1 + 2 + 4) + kNDer * (int64_t)sizeof(R);
        b += 16 + 16 + 4 + 8 * R4 + 16 + 96 * R4 + 4 + 4 + 8 + 4 + 4 + 4 + 4 + 4 * kExtraCap;
        b += 16 * (((int64_t)cap_nbr_ + 3) / 4);
        b += 4 + 12 + 8;  // pos_of_gid, three key arrays, two id arrays
        return b;
    }
    int64_t device_bytes() override { return dev_bytes_; }
    int64_t device_bytes_after_adding(int64_t n) override {
        int64_t staged = 0, staged_flaws = 0;
        for (auto& h : imp_)
            if (h.used && h.alive && !h.committed) {
                staged += h.n;
                staged_flaws += (int64_t)h.flaw_eps.size();
            }
        const int64_t need = N_ + staged + n;
        int64_t extra = 0;
        if (need > cap_) {
            const int64_t nc = std::max<int64_t>(need, (int64_t)(cap_ * 1.5) + 1024);
            extra += (nc - cap_) * bytes_per_particle();
        }
        // multi-flaw thresholds (~ln n per particle) and their per-id pointers
        const double lnn = std::log((double)std::max<int64_t>(n, 2));
        extra += (int64_t)((double)n * (lnn + 1.0)) * (int64_t)sizeof(R) + 8 * (n + staged) +
                 staged_flaws * (int64_t)sizeof(R);
        return dev_bytes_ + extra;
    }

    void impact_set_step_limit(int b, int64_t steps) override {
        ImpactH& h = imp(b);
        h.step_limit = steps;
        if (h.committed) {
            pull_table();
            tab_[b].max_steps = steps;
            push_table();
        }
    }

    void impact_set_time(int b, double t) override {
        ImpactH& h = imp(b);
        h.t = t;
        if (h.committed) {
            pull_table();
            tab_[b].t = t;
            push_table();
        }
    }

    void impact_remove(int b) override {
        ImpactH& h = imp(b);
        bool was_committed = h.committed;
        h.alive = false;
        if (h.flaws_on_device) flaw_live_ -= (int64_t)h.flaw_eps.size();  // its pool segment is dead
        if (was_committed) {
            pull_table();
            tab_[b].alive = 0;
            tab_[b].mask = 0;
            push_table();
            sort_reorder(true);  // purge its particles before the slot can be reused
            release_gids(h.gid_base, h.n);
        }
        h = ImpactH();
        if (was_committed) {
            assign_cell_bases();
            push_table();
        }
    }

    int impact_count() override {
        int c = 0;
        for (auto& h : imp_) c += h.used ? 1 : 0;
        return c;
    }

    sph_impact_info impact_info(int b) override {
        ImpactH& h = imp(b);
        sph_impact_info inf{};
        inf.n = h.n;
        inf.steps = h.steps;
        inf.t = h.t;
        inf.dt = h.dt_last;
        inf.initialized = h.initialized ? 1 : 0;
        if (h.committed) {
            pull_table();
            const ImpactD& I = tab_[b];
            inf.h_max = I.h_max;
            inf.t = I.t;
            for (int a = 0; a < 3; a++) { inf.nc[a] = I.nc[a]; inf.cw[a] = I.cw[a]; }
            inf.density_rounds = I.rounds;
        }
        return inf;
    }

    void get_domain(int b, double dlo[3], double dhi[3], int32_t per[3]) override {
        ImpactH& h = imp(b);
        for (int a = 0; a < 3; a++) { dlo[a] = h.dlo[a]; dhi[a] = h.dhi[a]; per[a] = h.per[a]; }
    }

    int64_t impact_n(int b) override { return imp(b).n; }
    int64_t impact_steps(int b) override { return imp(b).steps; }

    // ------------------------------------------------------------- stepping
    void init() override {
        commit();
        std::vector<int32_t> mask(imp_.size(), 0);
        bool any = false;
        for (size_t b = 0; b < imp_.size(); b++)
            if (imp_[b].used && imp_[b].alive && imp_[b].committed && !imp_[b].initialized) {
                mask[b] = 1;
                any = true;
            }
        if (!any) return;
        set_masks(mask, nullptr, nullptr);
        sort_reorder(true);
        build_list<kListSuperset>(true);
        density_rounds(2, true);
        forces(true);
        launch_n(k_adopt_derivatives<R>, N_);
        dt_reduce();
        for (size_t b = 0; b < imp_.size(); b++)
            if (mask[b]) imp_[b].initialized = true;
        check_async();
    }

    double timestep(int b) override {
        ImpactH& h = imp(b);
        if (!h.committed) throw SphError(SPH_ERR_STATE, "impact has no device state yet (call sph_init)");
        pull_table();
        return bitsd_host(tab_[b].dt_bits);
    }

    void step(double dt) override {
        commit();
        std::vector<int32_t> mask(imp_.size(), 0);
        std::vector<double> dts(imp_.size(), dt);
        for (size_t b = 0; b < imp_.size(); b++)
            if (imp_[b].used && imp_[b].alive && imp_[b].committed) mask[b] = 1;
        set_masks(mask, &dts, nullptr);
        if (use_graphs_ && !profiling_ && N_ > 0) {
            const int p = cur_;
            DSPH_CUDA(cudaGraphLaunch(ensure_graph(kGraphHostDt), st_));
            launches_ += graph_launches_[kGraphHostDt][p];
            cur_ = p ^ 1;  // the step's gather moved the carried state
        } else {
            one_step(true);
        }
        grow_lists_after_overflow();
        pull_table();
        for (size_t b = 0; b < imp_.size(); b++)
            if (mask[b]) {
                imp_[b].t = tab_[b].t;
                imp_[b].steps = tab_[b].nsteps;
                imp_[b].dt_last = dt;
                imp_[b].initialized = true;
            }
        check_async();
    }

    // One KDK step of the masked impacts (sph.hpp:357-377).  host_sync: the
    // adaptive-h round loop reads its convergence flag back; otherwise all four
    // rounds are issued and converged impacts skip them on the device.
    // before_eos (optional) runs between the head (kick, drift, sort, list,
    // density rounds: x, y, z and h final, u, D and S not yet read) and the
    // tail (EOS, forces, damage, finish, dt).
    void one_step(bool host_sync, const std::function<void()>* before_eos = nullptr) {
        step_head(host_sync);
        if (before_eos) (*before_eos)();
        step_tail();
    }
    void step_head(bool host_sync) {
        if (profiling_) DSPH_CUDA(cudaEventRecord(ev_[0], st_));
        cls(KC_KICK);
        launch_n(k_kick_drift<R>, N_);
        sort_reorder(false);
        cls(KC_LIST_DENSITY);
        build_list<kListSuperset>(false);
        if (profiling_) DSPH_CUDA(cudaEventRecord(ev_[1], st_));
        density_rounds(2, host_sync);
        if (profiling_) DSPH_CUDA(cudaEventRecord(ev_[2], st_));
        if (host_sync) refresh_list_if_needed();
        else refresh_list_device();
    }
    void step_tail() {
        const int nimp = (int)imp_.size();
        cls(KC_EOS);
        launch_n(k_eos<R>, N_);
        if (profiling_) DSPH_CUDA(cudaEventRecord(ev_[3], st_));
        cls(KC_FORCE);
        launch_force();
        if (profiling_) DSPH_CUDA(cudaEventRecord(ev_[4], st_));
        cls(KC_DAMAGE);
        launch_n(k_damage<R>, N_);
        cls(KC_FINISH);
        launch_n(k_finish<R>, N_);
        cls(KC_DT);
        dt_reduce();
        launch_small(k_run_control, nimp, 1);
        cls(KC_OTHER);
        if (profiling_) {
            DSPH_CUDA(cudaEventRecord(ev_[5], st_));
            record_phases();
            prof_flush();
        }
    }

    void kernel_stats(int c, double* ms, int64_t* n) override {
        if (c < 0 || c >= KC_N) throw SphError(SPH_ERR_ARG, "bad kernel class");
        *ms = kstat_ms_[c];
        *n = kstat_n_[c];
    }
    void kernel_stats_reset() override {
        for (int c = 0; c < KC_N; c++) { kstat_ms_[c] = 0; kstat_n_[c] = 0; }
    }
    void event_record(int slot) override {
        if (slot < 0 || slot >= 16) throw SphError(SPH_ERR_ARG, "event slot out of range");
        if (!user_ev_[slot]) DSPH_CUDA(cudaEventCreate(&user_ev_[slot]));
        DSPH_CUDA(cudaEventRecord(user_ev_[slot], st_));
    }
    double event_elapsed(int a, int b) override {
        if (a < 0 || a >= 16 || b < 0 || b >= 16 || !user_ev_[a] || !user_ev_[b])
            throw SphError(SPH_ERR_ARG, "event slot not recorded");
        DSPH_CUDA(cudaEventSynchronize(user_ev_[b]));
        float ms = 0;
        DSPH_CUDA(cudaEventElapsedTime(&ms, user_ev_[a], user_ev_[b]));
        return ms;
    }

    void run(int nsteps, double t_end) override {
        commit();
        std::vector<int32_t> mask(imp_.size(), 0);
        std::vector<double> te(imp_.size(), t_end > 0 ? t_end : 0.0);
        for (size_t b = 0; b < imp_.size(); b++)
            if (imp_[b].used && imp_[b].alive && imp_[b].committed && imp_[b].initialized) mask[b] = 1;
        set_masks(mask, nullptr, &te);
        const int nimp = (int)imp_.size();
        int s = 0;
        if (use_graphs_ && !profiling_ && N_ > 0) {
            // two captured steps per launch (the gather alternates the carried
            // buffers, so a two-step graph returns to its own parity); an odd
            // step first through the one-step graph of the current parity
            if (nsteps % 2) {
                const int p = cur_;
                DSPH_CUDA(cudaGraphLaunch(ensure_graph(kGraphOne), st_));
                launches_ += graph_launches_[kGraphOne][p];
                cur_ = p ^ 1;  // the step's gather moved the carried state
                s = 1;
            }
            // every 16 steps the list-overflow flag is read back, so a grown
            // neighbour count costs at most 16 steps of the consumers' fallback
            for (int since = 0; s + 1 < nsteps; s += 2) {
                if (++since > 8) {
                    grow_lists_after_overflow();
                    since = 1;
                }
                DSPH_CUDA(cudaGraphLaunch(ensure_graph(kGraphTwo), st_));
                launches_ += graph_launches_[kGraphTwo][cur_];
            }
            grow_lists_after_overflow();
        }
        for (; s < nsteps; s++) {
            launch_small(k_run_control, nimp, 0);
            one_step(true);
            grow_lists_after_overflow();
        }
        pull_table();
        for (size_t b = 0; b < imp_.size(); b++)
            if (mask[b]) {
                imp_[b].t = tab_[b].t;
                imp_[b].steps = tab_[b].nsteps;
                imp_[b].dt_last = tab_[b].dt;
            }
        check_async();
    }

    // Captures device-controlled steps (no host round trips: all four
    // adaptive-h rounds are issued and converged impacts skip them; list
    // overflow and slack are handled by the consumers' fallback) into one
    // executable graph per kind and buffer parity: two run steps (device dt),
    // one run step, or one step at the dt the host put in the impact table.
    // Re-captured whenever buffers, sizes or options change.  Capture issues
    // no work; the parity the graph starts from is restored afterwards.
    cudaGraphExec_t ensure_graph(int kind) {
        const int p = cur_;
        const int64_t shape = N_ * 65536 + (int64_t)imp_.size() + (any_periodic() ? (1ll << 62) : 0);
        cudaGraphExec_t& ge = graph_exec_[kind][p];
        if (ge && graph_key_[kind][p] == layout_epoch_ && graph_n_[kind][p] == shape) return ge;
        const int nimp = (int)imp_.size();
        const int64_t l0 = launches_;
        const uint64_t epoch0 = layout_epoch_;
        const int64_t n0 = N_;
        DSPH_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < (kind == kGraphTwo ? 2 : 1); k++) {
            if (kind == kGraphHead) {
                step_head(false);
                break;
            }
            if (kind == kGraphTail) {
                step_tail();
                break;
            }
            if (kind != kGraphHostDt) launch_small(k_run_control, nimp, 0);
            one_step(false);
        }
        cudaGraph_t g = nullptr;
        DSPH_CUDA(cudaStreamEndCapture(st_, &g));
        // A new particle count or impact table usually changes only kernel
        // parameters and grid sizes: update the executable graph in place
        // (cheaper than a fresh instantiation) and instantiate only when the
        // topology changed.
        bool updated = false;
        if (ge) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(ge, g, &info) == cudaSuccess;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(ge);
                ge = nullptr;
            }
        }
        if (!updated) DSPH_CUDA(cudaGraphInstantiate(&ge, g, 0));
        cudaGraphDestroy(g);
        graph_launches_[kind][p] = launches_ - l0;
        launches_ = l0;
        cur_ = p;  // a one-step capture flips the parity without running anything
        if (layout_epoch_ != epoch0 || N_ != n0)
            throw SphError(SPH_ERR_STATE, "graph capture changed the buffer layout");
        graph_key_[kind][p] = layout_epoch_;
        graph_n_[kind][p] = shape;
        return ge;
    }

    void compute_density_h(int iters) override {
        commit();
        set_all_masks();
        sort_reorder(true);
        build_list<kListSuperset>(true);
        density_rounds(iters, true);
        check_async();
    }

    void compute_forces() override {
        commit();
        set_all_masks();
        if (!grid_valid_) {
            sort_reorder(true);
            build_list<kListSuperset>(true);
            final_grid_build();
        }
        forces(true);
        launch_n(k_adopt_derivatives<R>, N_);
        dt_reduce();
        check_async();
    }

    void synchronize() override {
        DSPH_CUDA(cudaStreamSynchronize(st_));
        check_waits();
    }
    // A kernel whose bounded wait on its bulk copies ran out leaves its outputs
    // unwritten and sets the error word; the next synchronisation reports it.
    void check_waits() {
        int32_t e = 0;
        DSPH_CUDA(cudaMemcpy(&e, wait_err_d_, sizeof(int32_t), cudaMemcpyDeviceToHost));
        if (e) {
            DSPH_CUDA(cudaMemset(wait_err_d_, 0, sizeof(int32_t)));
            throw SphError(SPH_ERR_TIMEOUT, "a kernel's bounded wait for its staged copies ran out");
        }
    }

    // ------------------------------------------------------------- fields
    void read_field(int b, const char* name, double* out) override {
        ImpactH& h = imp(b);
        commit();
        if (h.n == 0) return;
        ensure_stage(h.n);
        bool ok = with_column(name, [&](auto* col) {
            launch_n_raw(k_read_col<std::remove_pointer_t<decltype(col)>>, h.n, col, pos_of_gid_, h.gid_base, h.n, stage_d_);
        });
        if (!ok) throw SphError(SPH_ERR_ARG, std::string("unknown field ") + name);
        DSPH_CUDA(cudaMemcpyAsync(out, stage_d_, sizeof(double) * h.n, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    void write_field(int b, const char* name, const double* in) override {
        ImpactH& h = imp(b);
        commit();
        if (h.n == 0) return;
        ensure_stage(h.n);
        DSPH_CUDA(cudaMemcpyAsync(stage_d_, in, sizeof(double) * h.n, cudaMemcpyHostToDevice, st_));
        bool ok = with_column(name, [&](auto* col) {
            launch_n_raw(k_write_col<std::remove_pointer_t<decltype(col)>>, h.n, col, pos_of_gid_, h.gid_base, h.n, (const double*)stage_d_);
        });
        if (!ok) throw SphError(SPH_ERR_ARG, std::string("unknown field ") + name);
        std::string nm(name);
        if (nm == "x" || nm == "y" || nm == "z" || nm == "hh") grid_valid_ = false;
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    // Several fields in one pass, through one staging slice per field: the
    // host copies run back to back on a copy stream while the compute stream
    // gathers (reads) or scatters (writes) the neighbouring fields, each pair
    // ordered by an event, and both streams are synchronised once -- pinned
    // caller buffers stream at link speed.
    // Address through which kernels reach a caller's host buffer directly over
    // the coherent CPU-GPU link (page-locked memory, or any host memory where
    // the device reads pageable memory through the host page tables), or null:
    // then the buffer goes through a device staging copy.
    void* host_direct(const void* p) {
        if (!host_direct_ || !p) return nullptr;
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if ((a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged) && a.devicePointer)
            return a.devicePointer;
        if (a.type == cudaMemoryTypeUnregistered && pageable_access_) return const_cast<void*>(p);
        return nullptr;
    }

    void read_fields(int b, int nf, const char* const* names, double* const* outs) override {
        ImpactH& h = imp(b);
        commit();
        if (h.n == 0 || nf <= 0) return;
        for (int f = 0; f < nf; f++)
            if (!with_column(names[f], [](auto*) {})) throw SphError(SPH_ERR_ARG, std::string("unknown field ") + names[f]);
        // fields whose buffers the device reaches directly: one kernel each,
        // writing the caller's memory in original order
        std::vector<int> staged;
        for (int f = 0; f < nf; f++) {
            double* dst = static_cast<double*>(host_direct(outs[f]));
            if (!dst) {
                staged.push_back(f);
                continue;
            }
            with_column(names[f], [&](auto* col) {
                launch_n_raw(k_read_col<std::remove_pointer_t<decltype(col)>>, h.n, col, pos_of_gid_, h.gid_base, h.n, dst);
            });
        }
        if (staged.empty()) {
            DSPH_CUDA(cudaStreamSynchronize(st_));
            return;
        }
        ensure_stage((int64_t)nf * h.n);
        for (int f : staged) {
            double* slice = stage_d_ + (int64_t)f * h.n;
            with_column(names[f], [&](auto* col) {
                launch_n_raw(k_read_col<std::remove_pointer_t<decltype(col)>>, h.n, col, pos_of_gid_, h.gid_base, h.n, slice);
            });
            DSPH_CUDA(cudaEventRecord(copy_ev_, st_));
            DSPH_CUDA(cudaStreamWaitEvent(copy_st_, copy_ev_, 0));
            DSPH_CUDA(cudaMemcpyAsync(outs[f], slice, sizeof(double) * h.n, cudaMemcpyDeviceToHost, copy_st_));
        }
        DSPH_CUDA(cudaStreamSynchronize(copy_st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    void write_fields(int b, int nf, const char* const* names, const double* const* ins) override {
        ImpactH& h = imp(b);
        commit();
        if (h.n == 0 || nf <= 0) return;
        for (int f = 0; f < nf; f++)
            if (!with_column(names[f], [](auto*) {})) throw SphError(SPH_ERR_ARG, std::string("unknown field ") + names[f]);
        std::vector<int> staged;
        for (int f = 0; f < nf; f++) {
            const double* src = static_cast<const double*>(host_direct(ins[f]));
            if (!src) {
                staged.push_back(f);
                continue;
            }
            with_column(names[f], [&](auto* col) {
                launch_n_raw(k_write_col<std::remove_pointer_t<decltype(col)>>, h.n, col, pos_of_gid_, h.gid_base, h.n, src);
            });
            std::string nm(names[f]);
            if (nm == "x" || nm == "y" || nm == "z" || nm == "hh") grid_valid_ = false;
        }
        if (staged.empty()) {
            DSPH_CUDA(cudaStreamSynchronize(st_));  // the caller may reuse its buffers on return
            return;
        }
        ensure_stage((int64_t)nf * h.n);
        // the staging slices may still feed earlier work on the compute stream
        DSPH_CUDA(cudaEventRecord(copy_ev_, st_));
        DSPH_CUDA(cudaStreamWaitEvent(copy_st_, copy_ev_, 0));
        for (int f : staged) {
            double* slice = stage_d_ + (int64_t)f * h.n;
            DSPH_CUDA(cudaMemcpyAsync(slice, ins[f], sizeof(double) * h.n, cudaMemcpyHostToDevice, copy_st_));
            DSPH_CUDA(cudaEventRecord(copy_ev_, copy_st_));
            DSPH_CUDA(cudaStreamWaitEvent(st_, copy_ev_, 0));
            with_column(names[f], [&](auto* col) {
                launch_n_raw(k_write_col<std::remove_pointer_t<decltype(col)>>, h.n, col, pos_of_gid_, h.gid_base, h.n,
                             (const double*)slice);
            });
            std::string nm(names[f]);
            if (nm == "x" || nm == "y" || nm == "z" || nm == "hh") grid_valid_ = false;
        }
        DSPH_CUDA(cudaStreamSynchronize(copy_st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    // One step with the caller's host fields crossing the boundary inside it:
    // the result of write_fields(ins); dt = timestep(b) when dt < 0; step(dt);
    // read_fields(outs), bit for bit, with the copies overlapping the step.
    // Inputs that no kernel of the step's head reads or writes (u, D, S, the
    // old derivatives dudt and dS, eps_act) are copied up while the head
    // (kick, drift, sort, list, density rounds) runs and are scattered, in the
    // order the sort left, between the head and the tail (EOS, forces,
    // damage, finish, dt); the other inputs go first.  Outputs
    // final at the end of the head (x, y, z, mass, h0, hh) are gathered there
    // and copied down while the tail runs, on a second copy stream, so both
    // link directions carry data at once.  Head and tail replay captured
    // graphs (one per buffer parity) unless graphs are off or profiling is on.
    // Always through device staging slices.
    double step_fields(int b, double dt, int nin, const char* const* in_names, const double* const* ins,
                       int nout, const char* const* out_names, double* const* outs) override {
        ImpactH& h = imp(b);
        commit();
        if (!h.committed) throw SphError(SPH_ERR_STATE, "impact has no device state yet (call sph_init)");
        for (int f = 0; f < nin; f++)
            if (!with_column(in_names[f], [](auto*) {}))
                throw SphError(SPH_ERR_ARG, std::string("unknown field ") + in_names[f]);
        for (int f = 0; f < nout; f++)
            if (!with_column(out_names[f], [](auto*) {}))
                throw SphError(SPH_ERR_ARG, std::string("unknown field ") + out_names[f]);
        if (dt < 0) {
            pull_table();
            dt = bitsd_host(tab_[b].dt_bits);
        }
        const int64_t n = h.n;
        if (n == 0 || N_ == 0) {
            write_fields(b, nin, in_names, ins);
            step(dt);
            read_fields(b, nout, out_names, outs);
            return dt;
        }
        std::vector<int32_t> mask(imp_.size(), 0);
        std::vector<double> dts(imp_.size(), dt);
        for (size_t i = 0; i < imp_.size(); i++)
            if (imp_[i].used && imp_[i].alive && imp_[i].committed) mask[i] = 1;
        set_masks(mask, &dts, nullptr);
        ensure_stage((int64_t)(nin + nout) * n);
        // carried fields that only the tail reads (EOS, forces, damage, finish)
        auto is_late = [](const char* s) {
            static const char* ln[] = {"u", "D", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz", "dudt",
                                       "dSxx", "dSyy", "dSzz", "dSxy", "dSxz", "dSyz", "eps_act"};
            for (const char* l : ln) if (!std::strcmp(s, l)) return true;
            return false;
        };
        auto is_head_final = [](const char* s) {
            static const char* ln[] = {"x", "y", "z", "mass", "h0", "hh"};
            for (const char* l : ln) if (!std::strcmp(s, l)) return true;
            return false;
        };
        auto in_slice = [&](int f) { return stage_d_ + (int64_t)f * n; };
        auto out_slice = [&](int f) { return stage_d_ + (int64_t)(nin + f) * n; };
        // one launch moves up to kColIo columns between staging slices and the
        // columns of the current buffer parity
        auto cols_io = [&](bool write, const std::vector<int>& fs) {
            for (size_t at = 0; at < fs.size(); at += kColIo) {
                ColIo s{};
                for (size_t c = at; c < fs.size() && c < at + kColIo; c++) {
                    const int f = fs[c];
                    const char* nm = write ? in_names[f] : out_names[f];
                    with_column(nm, [&](auto* col) {
                        s.col[s.nc] = col;
                        s.f32[s.nc] = sizeof(*col) == 4;
                    });
                    s.buf[s.nc++] = write ? in_slice(f) : out_slice(f);
                }
                if (write) launch_n_raw(k_write_cols, n, s, pos_of_gid_, h.gid_base, n);
                else launch_n_raw(k_read_cols, n, s, pos_of_gid_, h.gid_base, n);
            }
        };
        // the staging slices may still feed earlier work on the compute stream
        DSPH_CUDA(cudaEventRecord(copy_ev_, st_));
        DSPH_CUDA(cudaStreamWaitEvent(copy_st_, copy_ev_, 0));
        // head inputs: each field's copy, then its scatter while the next copies
        std::vector<int> late, head_out, tail_out;
        for (int f = 0; f < nin; f++) {
            if (is_late(in_names[f])) {
                late.push_back(f);
                continue;
            }
            DSPH_CUDA(cudaMemcpyAsync(in_slice(f), ins[f], sizeof(double) * n, cudaMemcpyHostToDevice, copy_st_));
            DSPH_CUDA(cudaEventRecord(copy_ev_, copy_st_));
            DSPH_CUDA(cudaStreamWaitEvent(st_, copy_ev_, 0));
            cols_io(true, {f});
            std::string nm(in_names[f]);
            if (nm == "x" || nm == "y" || nm == "z" || nm == "hh") grid_valid_ = false;
        }
        for (int f = 0; f < nout; f++) (is_head_final(out_names[f]) ? head_out : tail_out).push_back(f);
        // Host calls are ordered so that every copy is issued after the kernels
        // it should overlap are queued: from pageable memory a copy holds the
        // calling thread until it is done, from page-locked memory it does not.
        const std::function<void()> between = [&]() {
            for (int f : late)
                DSPH_CUDA(cudaMemcpyAsync(in_slice(f), ins[f], sizeof(double) * n, cudaMemcpyHostToDevice,
                                          copy_st_));
            DSPH_CUDA(cudaEventRecord(late_ev_, copy_st_));
            if (!late.empty()) {
                DSPH_CUDA(cudaStreamWaitEvent(st_, late_ev_, 0));
                cols_io(true, late);
            }
            if (!head_out.empty()) {
                cols_io(false, head_out);
                DSPH_CUDA(cudaEventRecord(out_ev_, st_));
            }
        };
        if (use_graphs_ && !profiling_) {
            const int p = cur_;
            DSPH_CUDA(cudaGraphLaunch(ensure_graph(kGraphHead), st_));
            launches_ += graph_launches_[kGraphHead][p];
            cur_ = p ^ 1;  // the head's sort moved the carried state
            between();
            DSPH_CUDA(cudaGraphLaunch(ensure_graph(kGraphTail), st_));
            launches_ += graph_launches_[kGraphTail][cur_];
        } else {
            one_step(false, &between);
        }
        // every input is read before any output is written, so the caller's
        // input and output buffers may be the same memory
        DSPH_CUDA(cudaStreamWaitEvent(out_st_, late_ev_, 0));
        if (!head_out.empty()) {
            DSPH_CUDA(cudaStreamWaitEvent(out_st_, out_ev_, 0));
            for (int f : head_out)
                DSPH_CUDA(cudaMemcpyAsync(outs[f], out_slice(f), sizeof(double) * n, cudaMemcpyDeviceToHost,
                                          out_st_));
        }
        // tail outputs: each field's gather, then its copy while the next gathers
        for (int f : tail_out) {
            cols_io(false, {f});
            DSPH_CUDA(cudaEventRecord(out_ev_, st_));
            DSPH_CUDA(cudaStreamWaitEvent(out_st_, out_ev_, 0));
            DSPH_CUDA(cudaMemcpyAsync(outs[f], out_slice(f), sizeof(double) * n, cudaMemcpyDeviceToHost, out_st_));
        }
        grow_lists_after_overflow();
        pull_table();
        for (size_t i = 0; i < imp_.size(); i++)
            if (mask[i]) {
                imp_[i].t = tab_[i].t;
                imp_[i].steps = tab_[i].nsteps;
                imp_[i].dt_last = dt;
                imp_[i].initialized = true;
            }
        DSPH_CUDA(cudaStreamSynchronize(copy_st_));
        DSPH_CUDA(cudaStreamSynchronize(out_st_));
        check_async();
        return dt;
    }

    void read_mat(int b, int32_t* out) override {
        ImpactH& h = imp(b);
        for (int64_t i = 0; i < h.n; i++) out[i] = h.mat_host[i];
    }

    void read_fixed(int b, uint8_t* out) override {
        ImpactH& h = imp(b);
        commit();
        if (h.n == 0) return;
        ensure_stage(h.n);
        launch_n_raw(k_read_u8, h.n, (const uint8_t*)fixed_[cur_], (const int32_t*)pos_of_gid_, h.gid_base, h.n, (uint8_t*)stage_d_);
        DSPH_CUDA(cudaMemcpyAsync(out, stage_d_, h.n, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    void write_fixed(int b, const uint8_t* in) override {
        ImpactH& h = imp(b);
        commit();
        if (h.n == 0) return;
        ensure_stage(h.n);
        DSPH_CUDA(cudaMemcpyAsync(stage_d_, in, h.n, cudaMemcpyHostToDevice, st_));
        launch_n_raw(k_write_u8, h.n, fixed_[cur_], (const int32_t*)pos_of_gid_, h.gid_base, h.n, (const uint8_t*)stage_d_);
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    sph_conservation conservation(int b) override {
        ImpactH& h = imp(b);
        commit();
        sph_conservation c{};
        if (h.n == 0) return c;
        ensure_stage(8);
        if (!grid_valid_) sort_reorder(true);
        k_conservation<R><<<1, 256, 0, st_>>>(view(), b, stage_d_);
        launches_++;
        double out[8];
        DSPH_CUDA(cudaMemcpyAsync(out, stage_d_, sizeof(double) * 6, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        c.mass = out[0];
        c.kinetic = out[1];
        c.internal = out[2];
        c.energy = out[1] + out[2];
        c.momentum[0] = out[3];
        c.momentum[1] = out[4];
        c.momentum[2] = out[5];
        return c;
    }

    void diagnostics(int b, int mat_lo, int mat_hi, double u_melt, double out[11]) override {
        ImpactH& h = imp(b);
        commit();
        for (int q = 0; q < 11; q++) out[q] = 0.0;
        if (h.n == 0) return;
        ensure_stage(16);
        if (!grid_valid_) sort_reorder(true);
        k_diagnostics<R><<<1, 512, 0, st_>>>(view(), b, mat_lo, mat_hi, u_melt, stage_d_);
        DSPH_CUDA(cudaGetLastError());
        launches_++;
        DSPH_CUDA(cudaMemcpyAsync(out, stage_d_, sizeof(double) * 11, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    void eos_eval(int mat, int64_t n, const double* rho, const double* u, double* P, double* cs) override {
        if (mat < 0 || mat >= (int)mats_h_.size()) throw SphError(SPH_ERR_ARG, "material id out of range");
        if (n <= 0) return;
        ensure_stage(4 * n);
        double* d = stage_d_;
        DSPH_CUDA(cudaMemcpyAsync(d, rho, sizeof(double) * n, cudaMemcpyHostToDevice, st_));
        DSPH_CUDA(cudaMemcpyAsync(d + n, u, sizeof(double) * n, cudaMemcpyHostToDevice, st_));
        launch_n_raw(k_eos_eval<R>, n, (const MatT<R>*)mats_d_, mat, n, (const double*)d, (const double*)(d + n), d + 2 * n, d + 3 * n);
        DSPH_CUDA(cudaMemcpyAsync(P, d + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaMemcpyAsync(cs, d + 3 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    // ------------------------------------------------------------- parity hooks
    void debug_ref_cells(int b, int32_t nc[3], double cw[3], int32_t* start, int64_t start_len,
                         int32_t* ids) override {
        ImpactH& h = imp(b);
        commit();
        if (!grid_valid_) {
            set_all_masks();
            sort_reorder(true);
            final_grid_build();
        }
        pull_table();
        const ImpactD& I = tab_[b];
        int64_t ncell = (int64_t)I.nc[0] * I.nc[1] * I.nc[2];
        for (int a = 0; a < 3; a++) { nc[a] = I.nc[a]; cw[a] = I.cw[a]; }
        if (start_len < ncell + 1) throw SphError(SPH_ERR_CAPACITY, "start array too short");
        int64_t n = h.n;
        // keys in local-id order -> stable radix sort -> CSR
        uint32_t* keys = dalloc_tmp<uint32_t>(n + 1);
        uint32_t* k2 = dalloc_tmp<uint32_t>(n + 1);
        uint32_t* k3 = dalloc_tmp<uint32_t>(n + 1);
        int32_t* v2 = dalloc_tmp<int32_t>(n + 1);
        int32_t* v3 = dalloc_tmp<int32_t>(n + 1);
        int32_t* cnt = dalloc_tmp<int32_t>(ncell + 2);
        void* scr = dalloc_tmp<char>(radix_scratch_bytes(std::max(n, ncell + 1)) + scan_scratch_bytes(ncell + 1) + 64);
        DSPH_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (ncell + 2), st_));
        if (n > 0) {
            launch_n_raw(k_ref_keys<R>, n, view(), b, (const int32_t*)pos_of_gid_, h.gid_base, n, keys, cnt);
            int bits = 1;
            while ((1ll << bits) <= ncell) bits++;
            launches_ += radix_sort_pairs(keys, nullptr, k2, v2, k3, v3, n, bits, scr, st_);
        }
        launches_ += exclusive_scan_i32(cnt, cnt, ncell + 1, scr, st_);
        DSPH_CUDA(cudaMemcpyAsync(start, cnt, sizeof(int32_t) * (ncell + 1), cudaMemcpyDeviceToHost, st_));
        if (n > 0) DSPH_CUDA(cudaMemcpyAsync(ids, v2, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        free_tmp();
    }

    int64_t debug_neighbors(int b, int kind, int32_t* counts, int32_t* ids, int64_t cap) override {
        ImpactH& h = imp(b);
        commit();
        if (!grid_valid_) {
            set_all_masks();
            sort_reorder(true);
            final_grid_build();
        }
        pull_table();
        const ImpactD& I = tab_[b];
        int64_t n = I.n;
        // pass 1: set sizes per sorted position
        int32_t* cnt = dalloc_tmp<int32_t>(n + 1);
        if (n > 0) launch_n_raw(k_debug_nbr<R>, n, view(), b, kind, (int32_t*)nullptr, cnt, (const int64_t*)nullptr);
        std::vector<int32_t> hcnt(n), gidv(n);  // gidv: local id of each sorted position
        if (n > 0) {
            DSPH_CUDA(cudaMemcpyAsync(hcnt.data(), cnt, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st_));
            DSPH_CUDA(cudaMemcpyAsync(gidv.data(), gid_[cur_] + I.off, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st_));
        }
        DSPH_CUDA(cudaStreamSynchronize(st_));
        std::vector<int64_t> where(h.n, -1);
        for (int64_t q = 0; q < n; q++) where[gidv[q] - h.gid_base] = q;
        int64_t total = 0;
        for (int64_t l = 0; l < h.n; l++) {
            counts[l] = where[l] >= 0 ? hcnt[where[l]] : 0;
            total += counts[l];
        }
        if (!ids || total > cap) {
            free_tmp();
            if (ids) throw SphError(SPH_ERR_CAPACITY, "neighbour id buffer too small");
            return total;
        }
        // pass 2: each set written at its place in the caller's (original) order
        std::vector<int64_t> offs(std::max<int64_t>(n, 1));
        {
            int64_t o = 0;
            for (int64_t l = 0; l < h.n; l++) {
                if (where[l] >= 0) offs[where[l]] = o;
                o += counts[l];
            }
        }
        int64_t* offs_d = dalloc_tmp<int64_t>(std::max<int64_t>(n, 1));
        int32_t* out = dalloc_tmp<int32_t>(total + 1);
        if (n > 0) {
            DSPH_CUDA(cudaMemcpyAsync(offs_d, offs.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, st_));
            launch_n_raw(k_debug_nbr<R>, n, view(), b, kind, out, cnt, (const int64_t*)offs_d);
            if (total > 0) DSPH_CUDA(cudaMemcpyAsync(ids, out, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, st_));
        }
        DSPH_CUDA(cudaStreamSynchronize(st_));
        free_tmp();
        int64_t o = 0;
        for (int64_t l = 0; l < h.n; l++) {
            std::sort(ids + o, ids + o + counts[l]);
            o += counts[l];
        }
        return total;
    }

    // Multi-flaw CSR of one impact as the device holds it (original particle
    // order; activation strains in the engine's precision, widened to double).
    int64_t debug_flaws(int b, int64_t* ptr, double* eps, int64_t cap) override {
        ImpactH& h = imp(b);
        commit();
        if (!(h.multi && h.flaws_on_device) || h.n == 0) {
            for (int64_t l = 0; l <= h.n; l++) ptr[l] = 0;
            return 0;
        }
        std::vector<int64_t> db(h.n), de(h.n);
        DSPH_CUDA(cudaMemcpyAsync(db.data(), flaw_beg_d_ + h.gid_base, sizeof(int64_t) * h.n, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaMemcpyAsync(de.data(), flaw_end_d_ + h.gid_base, sizeof(int64_t) * h.n, cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        const int64_t base = db[0], total = de[h.n - 1] - base;
        for (int64_t l = 0; l < h.n; l++) ptr[l] = db[l] - base;
        ptr[h.n] = total;
        if (eps && total > cap) throw SphError(SPH_ERR_CAPACITY, "flaw buffer too small");
        if (eps && total > 0) {
            std::vector<R> e(total);
            DSPH_CUDA(cudaMemcpyAsync(e.data(), flaw_eps_d_ + base, sizeof(R) * total, cudaMemcpyDeviceToHost, st_));
            DSPH_CUDA(cudaStreamSynchronize(st_));
            for (int64_t q = 0; q < total; q++) eps[q] = (double)e[q];
        }
        return total;
    }

    // ------------------------------------------------------------- tuning
    void set_tuning(int block, double cell_factor) override {
        if (block > 0) {
            if (block % 32 != 0 || block > 1024) throw SphError(SPH_ERR_ARG, "block must be a multiple of 32 <= 1024");
            block_ = block;
        }
        if (cell_factor > 0) {
            bool any_committed = false;
            for (auto& h : imp_) any_committed |= h.committed;
            if (any_committed) throw SphError(SPH_ERR_STATE, "cell factor must be set before particles are committed");
            cell_factor_ = cell_factor;
        }
    }
    void set_option(const char* key, double value) override {
        std::string k(key);
        layout_epoch_++;
        if (k == "graphs") {
            use_graphs_ = value != 0;
            return;
        }
        if (k == "list_mode") {
            if (value != 0 && value != 1 && value != 2)
                throw SphError(SPH_ERR_ARG, "list_mode is 0 (thread), 1 (warp per column run) or 2 (warp per particle)");
            list_mode_ = (int)value;
        } else if (k == "slack") {
            if (!(value >= 0.0 && value <= 1.0)) throw SphError(SPH_ERR_ARG, "slack must be in [0, 1]");
            slack_ = value;
            if (!tab_.empty()) {
                pull_table();
                for (auto& I : tab_) I.slack = (float)slack_;
                push_table();
            }
        } else if (k == "cell_factor") {
            set_tuning(0, value);
        } else if (k == "cell_factor_z") {
            if (!(value > 0.0 && value <= 4.0)) throw SphError(SPH_ERR_ARG, "cell_factor_z must be in (0, 4]");
            for (auto& h : imp_)
                if (h.committed) throw SphError(SPH_ERR_STATE, "cell factors must be set before particles are committed");
            cell_factor_z_ = value;
        } else if (k == "block") {
            set_tuning((int)value, 0);
        } else if (k == "levels") {
            for (auto& h : imp_)
                if (h.committed) throw SphError(SPH_ERR_STATE, "levels are set before particles are committed");
            levels_ = value != 0;
        } else if (k == "host_direct") {
            host_direct_ = value != 0;
        } else if (k == "force_staging") {
            const int fsv = (int)value;
            if (!(value == fsv && (fsv == 0 || fsv == 22 || fsv == 23 || fsv == 42 || fsv == 122 || fsv == 142)))
                throw SphError(SPH_ERR_ARG, "force_staging is 0 (off), 10 x entries + stages with bulk copies "
                                            "(22, 23, 42) or 100 + that with 16-byte async copies (122, 142)");
            if constexpr (sizeof(R) == 4) {
                if (fsv == 22) allow_force_smem<2, 2, false>();
                if (fsv == 23) allow_force_smem<2, 3, false>();
                if (fsv == 42) allow_force_smem<4, 2, false>();
                if (fsv == 122) allow_force_smem<2, 2, true>();
                if (fsv == 142) allow_force_smem<4, 2, true>();
            }
            force_staging_ = fsv;
        } else {
            throw SphError(SPH_ERR_ARG, "unknown option " + k);
        }
    }
    double get_option(const char* key) override {
        std::string k(key);
        if (k == "list_mode") return list_mode_;
        if (k == "force_staging") return force_staging_;
        if (k == "host_direct") return host_direct_ ? 1 : 0;
        if (k == "levels") return levels_ ? 1 : 0;
        if (k == "levels_active") return levels_active_ ? 1 : 0;
        if (k == "pageable_access") return pageable_access_ ? 1 : 0;
        if (k == "graphs") return use_graphs_ ? 1 : 0;
        if (k == "slack") return slack_;
        if (k == "cell_factor") return cell_factor_;
        if (k == "cell_factor_z") return cell_factor_z_;
        if (k == "block") return block_;
        if (k == "list_capacity") return cap_nbr_;
        if (k == "list_entries") return (double)list_entries();
        if (k == "device_bytes") return (double)dev_bytes_;
        if (k == "bytes_per_particle") return (double)bytes_per_particle();
        throw SphError(SPH_ERR_ARG, "unknown option " + k);
    }
    int64_t launches() override { return launches_; }
    void phase_times(double ms[5]) override { for (int i = 0; i < 5; i++) ms[i] = phase_ms_[i]; }
    void set_profiling(int on) override { profiling_ = on != 0; }

private:
    // entries of the current neighbour lists (0 before the first build)
    unsigned long long list_entries() {
        if (N_ <= 0 || !nbr_cnt_ || !xcnt_) return 0;
        // a plain allocation: the engine's own allocator would invalidate
        // the captured step graphs
        unsigned long long* d = nullptr;
        DSPH_CUDA(cudaMalloc(&d, sizeof(unsigned long long)));
        unsigned long long h = 0;
        DSPH_CUDA(cudaMemsetAsync(d, 0, sizeof(h), st_));
        k_sum_list_entries<<<std::max(1, std::min(nsm_ * 4, (int)((N_ + 255) / 256))), 256, 0, st_>>>(
            nbr_cnt_, xcnt_, N_, cap_nbr_, d);
        DSPH_CUDA(cudaGetLastError());
        DSPH_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        cudaFree(d);
        return h;
    }

    // ------------------------------------------------------------- helpers
    static double bitsd_host(unsigned long long b) {
        double d;
        std::memcpy(&d, &b, 8);
        return d;
    }

    template <class T>
    T* dalloc(size_t n) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1));
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw SphError(SPH_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        allocs_.push_back(p);
        alloc_bytes_.push_back((int64_t)(sizeof(T) * std::max<size_t>(n, 1)));
        dev_bytes_ += alloc_bytes_.back();
        layout_epoch_++;
        return static_cast<T*>(p);
    }
    void dfree(void* p) {
        if (!p) return;
        auto it = std::find(allocs_.begin(), allocs_.end(), p);
        if (it != allocs_.end()) {
            const size_t i = (size_t)(it - allocs_.begin());
            dev_bytes_ -= alloc_bytes_[i];
            alloc_bytes_.erase(alloc_bytes_.begin() + (std::ptrdiff_t)i);
            allocs_.erase(it);
        }
        cudaFree(p);
    }
    template <class T>
    T* dalloc_tmp(size_t n) {
        T* p = dalloc<T>(n);
        tmp_.push_back(p);
        return p;
    }
    void free_tmp() {
        for (void* p : tmp_) dfree(p);
        tmp_.clear();
    }

    void check_async() {
        cudaError_t e = cudaPeekAtLastError();
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw SphError(SPH_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
        }
    }

    // A launch the runtime rejects (configuration, resources) is reported at
    // once with the kernel's name, not at the next synchronisation.
    void launched(const void* fn) {
        const cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) return;
        const char* name = nullptr;
        if (cudaFuncGetName(&name, fn) != cudaSuccess || !name) name = "?";
        cudaGetLastError();
        throw SphError(SPH_ERR_CUDA, std::string("launch of ") + name + ": " + cudaGetErrorString(e));
    }

    template <class Kern, class... Args>
    void launch_n_raw(Kern k, int64_t n, Args... args) {
        if (n <= 0) return;
        int bs = 256;
        prof_begin();
        k<<<(unsigned)((n + bs - 1) / bs), bs, 0, st_>>>(args...);
        launched((const void*)k);
        prof_end();
        launches_++;
    }
    template <class Kern>
    void launch_n(Kern k, int64_t n, int bs = 0) {
        if (n <= 0) return;
        if (bs <= 0) bs = 256;
        prof_begin();
        k<<<(unsigned)((n + bs - 1) / bs), bs, 0, st_>>>(view());
        launched((const void*)k);
        prof_end();
        launches_++;
    }
    // The force pass; in the mixed form optionally with its neighbour records
    // staged in shared memory by bulk copies (option "force_staging").
    template <int SE, int SS, bool ASYNC>
    void launch_force_staged(unsigned grid) {
        using FS = ForceStaging<SE, SS>;
        static_assert(FS::kSmemBytes <= 227 * 1024, "force staging exceeds the shared memory of a block");
        k_force<R, SE, SS, ASYNC><<<grid, FS::kBlock, FS::kSmemBytes, st_>>>(view(), wait_err_d_);
        launched((const void*)k_force<R, SE, SS, ASYNC>);
    }
    // Some resident impact has a periodic axis: the pair kernels then take
    // the minimum-image branches (the choice is part of a captured graph's key).
    bool any_periodic() const {
        for (const ImpactH& h : imp_)
            if (h.used && h.alive && (h.per[0] | h.per[1] | h.per[2])) return true;
        return false;
    }
    void launch_force() {
        if (N_ <= 0) return;
        prof_begin();
        const unsigned grid = (unsigned)((N_ + 127) / 128);
        bool done = false;
        if (sizeof(R) == 4 && !levels_active_) {
            done = true;
            switch (force_staging_) {
                case 22: launch_force_staged<2, 2, false>(grid); break;
                case 23: launch_force_staged<2, 3, false>(grid); break;
                case 42: launch_force_staged<4, 2, false>(grid); break;
                case 122: launch_force_staged<2, 2, true>(grid); break;
                case 142: launch_force_staged<4, 2, true>(grid); break;
                default: done = false;
            }
        }
        if (levels_active_) {  // graded impacts resident: the level-aware pass (never staged)
            k_force<R, 0, 0, false, true><<<grid, 128, 0, st_>>>(view(), wait_err_d_);
            launched((const void*)k_force<R, 0, 0, false, true>);
        } else if (!done && any_periodic()) {
            k_force<R, 0, 0, false, false, true><<<grid, 128, 0, st_>>>(view(), wait_err_d_);
            launched((const void*)k_force<R, 0, 0, false, false, true>);
        } else if (!done) {  // no resident impact is periodic: pair loop without minimum image
            k_force<R, 0, 0, false, false, false><<<grid, 128, 0, st_>>>(view(), wait_err_d_);
            launched((const void*)k_force<R, 0, 0, false, false, false>);
        }
        prof_end();
        launches_++;
    }
    template <int SE, int SS, bool ASYNC>
    void allow_force_smem() {
        DSPH_CUDA(cudaFuncSetAttribute(k_force<R, SE, SS, ASYNC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       ForceStaging<SE, SS>::kSmemBytes));
    }

    template <class Kern, class... Args>
    void launch_small(Kern k, int nimp, Args... args) {
        if (nimp <= 0) return;
        prof_begin();
        k<<<(nimp + 127) / 128, 128, 0, st_>>>(tab_d_, nimp, args...);
        launched((const void*)k);
        prof_end();
        launches_++;
    }

    // ---- per-kernel-class CUDA-event timing on the engine stream
public:
    enum KClass { KC_KICK, KC_SORT, KC_GRID, KC_LIST_DENSITY, KC_DENSITY, KC_EOS, KC_LIST_FORCE,
                  KC_FORCE, KC_DAMAGE, KC_FINISH, KC_DT, KC_OTHER, KC_N };

private:
    void prof_begin() {
        if (!profiling_) return;
        if (np_ >= prof_pool_.size()) {
            cudaEvent_t a, b;
            DSPH_CUDA(cudaEventCreate(&a));
            DSPH_CUDA(cudaEventCreate(&b));
            prof_pool_.push_back({a, b});
            prof_cls_.push_back(0);
        }
        DSPH_CUDA(cudaEventRecord(prof_pool_[np_].first, st_));
    }
    void prof_end() {
        if (!profiling_) return;
        DSPH_CUDA(cudaEventRecord(prof_pool_[np_].second, st_));
        prof_cls_[np_] = cur_cls_;
        np_++;
    }
    void prof_flush() {
        if (!profiling_ || np_ == 0) return;
        DSPH_CUDA(cudaEventSynchronize(prof_pool_[np_ - 1].second));
        for (size_t i = 0; i < np_; i++) {
            float ms = 0;
            DSPH_CUDA(cudaEventElapsedTime(&ms, prof_pool_[i].first, prof_pool_[i].second));
            kstat_ms_[prof_cls_[i]] += ms;
            kstat_n_[prof_cls_[i]] += 1;
        }
        np_ = 0;
    }
    void cls(int c) { cur_cls_ = c; }

public:

    void ensure_stage(int64_t n) {
        if (n <= stage_cap_) return;
        dfree(stage_d_);
        stage_cap_ = std::max<int64_t>(n, 1024);
        stage_d_ = dalloc<double>(stage_cap_);
    }

    View<R> view() {
        View<R> v{};
        v.n = N_;
        v.cap = cap_nbr_;
        v.ls = cap_;
        v.x = dcol_[cur_][0]; v.y = dcol_[cur_][1]; v.z = dcol_[cur_][2]; v.u = dcol_[cur_][3];
        v.vx = dcol_[cur_][4]; v.vy = dcol_[cur_][5]; v.vz = dcol_[cur_][6];
        R** r = rcol_[cur_];
        v.ax = r[RC_AX]; v.ay = r[RC_AY]; v.az = r[RC_AZ];
        v.dudt = r[RC_DUDT]; v.mass = r[RC_MASS]; v.hh = r[RC_HH]; v.D = r[RC_D];
        v.eps_act = r[RC_EPSACT]; v.h0 = r[RC_H0];
        for (int c = 0; c < 6; c++) { v.S[c] = r[RC_S0 + c]; v.dS[c] = r[RC_DS0 + c]; }
        v.mat = mat_[cur_]; v.fixed = fixed_[cur_]; v.imp = impc_[cur_]; v.gid = gid_[cur_];
        v.rho = der_[DR_RHO]; v.P = der_[DR_P]; v.cs = der_[DR_CS]; v.csig = der_[DR_CSIG];
        v.Pf = der_[DR_PF]; v.dscale = der_[DR_DSCALE]; v.Rart = der_[DR_RART];
        v.sigmax = der_[DR_SIGMAX]; v.epsw = der_[DR_EPSW]; v.pfr2 = der_[DR_PFR2];
        v.dsr2 = der_[DR_DSR2]; v.vol = der_[DR_VOL]; v.dudt_new = der_[DR_DUDTN];
        for (int c = 0; c < 6; c++) v.dS_new[c] = der_[DR_DSN0 + c];
        v.rho_lo = der_[DR_RHOLO];
        v.pf = pf_; v.cpk = cpk_; v.refbin = refbin_;
        v.pk = pk_; v.fr = fr_; v.lf = lf_;
        v.cell_ptr = cell_cnt_;
        v.nbr = nbr_; v.nbr_cnt = nbr_cnt_; v.hlist = hlist_;
        v.xnbr = xnbr_; v.xcnt = xcnt_;
        v.flags = flags_d_;
        v.imps = tab_d_;
        v.mats = mats_d_;
        v.flaw_beg = flaw_beg_d_;
        v.flaw_end = flaw_end_d_;
        v.flaw_eps = flaw_eps_d_;
        return v;
    }

    template <class F>
    bool with_column(const char* name, F f) {
        std::string s(name);
        static const char* dn[] = {"x", "y", "z", "u", "vx", "vy", "vz"};
        for (int c = 0; c < kND; c++) if (s == dn[c]) { f(dcol_[cur_][c]); return true; }
        static const char* rn[] = {"ax", "ay", "az", "dudt", "mass", "hh", "D",
                                   "eps_act", "h0", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz",
                                   "dSxx", "dSyy", "dSzz", "dSxy", "dSxz", "dSyz"};
        for (int c = 0; c < kNR; c++) if (s == rn[c]) { f(rcol_[cur_][c]); return true; }
        static const char* en[] = {"rho", "P", "cs", "csig", "Pf", "dscale", "Rart", "sigmax", "eps_work"};
        for (int c = 0; c < 9; c++) if (s == en[c]) { f(der_[c]); return true; }
        return false;
    }

    void upload_materials() {
        std::vector<MatT<R>> m(kMaxMaterials);
        std::memset(m.data(), 0, sizeof(MatT<R>) * kMaxMaterials);
        for (size_t i = 0; i < mats_h_.size(); i++) {
            const sph_material& s = mats_h_[i];
            MatT<R>& d = m[i];
            d.type = s.type; d.yield_model = s.yield_model;
            d.gamma = (R)s.gamma; d.rho0 = (R)s.rho0; d.a = (R)s.a; d.b = (R)s.b; d.A = (R)s.A; d.B = (R)s.B;
            d.alpha = (R)s.alpha; d.beta = (R)s.beta; d.u0 = (R)s.u0; d.uiv = (R)s.uiv; d.ucv = (R)s.ucv;
            d.G = (R)s.G; d.Y = (R)s.Y; d.Emod = (R)s.Emod; d.wm = (R)s.wm; d.wk = (R)s.wk;
            d.Y0 = (R)s.Y0; d.mu_i = (R)s.mu_i; d.Ylim = (R)s.Ylim; d.Yd0 = (R)s.Yd0; d.mu_d = (R)s.mu_d;
        }
        DSPH_CUDA(cudaMemcpyAsync(mats_d_, m.data(), sizeof(MatT<R>) * kMaxMaterials, cudaMemcpyHostToDevice, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    // Impact table: host mirror <-> device (only at configuration changes).
    void pull_table() {
        if (tab_.empty() || !tab_d_) return;
        DSPH_CUDA(cudaMemcpyAsync(tab_.data(), tab_d_, sizeof(ImpactD) * tab_.size(), cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }
    void push_table() {
        if (tab_.empty()) return;
        if ((int)tab_.size() > tab_cap_) {
            dfree(tab_d_);
            tab_cap_ = (int)tab_.size() * 2;
            tab_d_ = dalloc<ImpactD>(tab_cap_);
        }
        DSPH_CUDA(cudaMemcpyAsync(tab_d_, tab_.data(), sizeof(ImpactD) * tab_.size(), cudaMemcpyHostToDevice, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
    }

    void fill_params(ImpactD& I, const ImpactH& h) {
        const sph_params& p = h.prm;
        I.eta = p.eta; I.h_init = p.h_init; I.alpha = p.alpha; I.beta = p.beta; I.eps = p.eps;
        I.alpha_u = p.alpha_u; I.cfl = p.cfl; I.eps_as = p.eps_as;
        I.damage_on = p.damage_on != 0;
        I.multi_flaw = (p.flaw_model == SPH_FLAWS_MULTI && h.multi) ? 1 : 0;
        I.use_h0 = h.use_h0 ? 1 : 0;
        double h0m = h.use_h0 ? h.h0max : p.h_init;
        I.hcap = (float)(2.0 * h0m);
        I.slack = (float)slack_;
        // W polynomial at q = 1/eta, for the artificial-stress ratio W(r)/W(dp)
        double q = 1.0 / p.eta, poly;
        if (q < 1.0) poly = 1.0 - 1.5 * q * q + 0.75 * q * q * q;
        else if (q < 2.0) { double t = 2.0 - q; poly = 0.25 * t * t * t; }
        else poly = 0.0;
        I.inv_poly_eta = poly > 0 ? 1.0 / poly : 0.0;
        I.inv_poly_eta_f = (float)I.inv_poly_eta;
        for (int a = 0; a < 3; a++) {
            I.dlo[a] = h.dlo[a]; I.dhi[a] = h.dhi[a]; I.per[a] = h.per[a];
        }
    }

    // Fine traversal grid of an impact: cells of ~cell_factor * h_init over the
    // domain (padded on open axes; z cells cell_factor_z times that height),
    // exact period on periodic axes.
    void make_fine_grid(ImpactD& I, const ImpactH& h) {
        double w00 = cell_factor_ * h.prm.h_init;
        if (!(w00 > 0)) w00 = 1.0;
        double bblo[3], bbhi[3];
        for (int a = 0; a < 3; a++) { bblo[a] = 1e300; bbhi[a] = -1e300; }
        const std::vector<double>* P[3] = {&h.sx, &h.sy, &h.sz};
        for (int a = 0; a < 3; a++)
            for (double c : *P[a]) { bblo[a] = std::min(bblo[a], c); bbhi[a] = std::max(bbhi[a], c); }
        const int lim[3] = {2047, 2047, 1023};
        int64_t cells = 1;
        for (int a = 0; a < 3; a++) {
            const double w0 = a == 2 ? w00 * cell_factor_z_ : w00;
            double lo = h.dlo[a], ext = h.dhi[a] - h.dlo[a];
            if (!(ext > 0)) {  // no domain on this axis: cover the particles
                lo = (bblo[a] <= bbhi[a] ? bblo[a] : 0.0) - 2 * w0;
                ext = (bblo[a] <= bbhi[a] ? bbhi[a] - bblo[a] : 0.0) + 4 * w0;
            }
            if (h.per[a] && h.dhi[a] > h.dlo[a]) {
                int nf = std::max(1, (int)std::floor(ext / w0));
                nf = std::min(nf, lim[a]);
                I.glo[a] = h.dlo[a];
                I.nf[a] = nf;
                I.w[a] = ext / nf;
            } else {
                double pad = 0.02 * ext + 2 * w0;  // room just past the domain before clamping
                double span = ext + 2 * pad;
                int nf = (int)std::ceil(span / w0);
                double w = w0;
                if (nf > lim[a]) { nf = lim[a]; w = span / nf; }
                I.glo[a] = lo - pad;
                I.nf[a] = std::max(nf, 1);
                I.w[a] = w;
            }
            cells *= I.nf[a];
        }
        // keep the empty-cell overhead bounded
        int64_t budget = std::max<int64_t>(64 * std::max<int64_t>(h.n, 1), 1 << 20);
        while (cells > budget) {
            cells = 1;
            for (int a = 0; a < 3; a++) {
                if (h.per[a] && h.dhi[a] > h.dlo[a]) {
                    int nf = std::max(1, I.nf[a] / 2);
                    I.w[a] = (h.dhi[a] - h.dlo[a]) / nf;
                    I.nf[a] = nf;
                } else {
                    double span = I.nf[a] * I.w[a];
                    I.w[a] *= 1.26;
                    I.nf[a] = std::max(1, (int)std::ceil(span / I.w[a]));
                }
                cells *= I.nf[a];
            }
        }
        for (int a = 0; a < 3; a++) {
            I.iw[a] = 1.0 / I.w[a];
            I.iwf[a] = (float)I.iw[a];
            I.wf[a] = (float)I.w[a];
            I.Lf[a] = (float)(h.dhi[a] - h.dlo[a]);
        }
        I.ncells = cells;
        I.nlev = 1;
        I.lev_h0[0] = 0.0f;
        I.lev_base[0] = 0;
        for (int a = 0; a < 3; a++) {
            I.lev_lo[0][a] = 0;
            I.lev_nf[0][a] = I.nf[a];
        }
        make_levels(I, h, budget);
    }

    // Levels of a graded impact: power-of-two bands of the reference smoothing
    // length h0 above its smallest value, each with cells 2^L base cells wide
    // over the box of its particles padded by two level cells per side, when
    // the h0 range spans more than a factor 2.  A particle that later leaves
    // its level's box is clamped into the border cells and flags the level, so
    // searches never skip that level and never prune its border columns; tight
    // boxes keep a coarse particle's search off the empty cells of the finer
    // levels' boxes.
    void make_levels(ImpactD& I, const ImpactH& h, int64_t budget) {
        if (!levels_ || !h.use_h0 || h.per[0] || h.per[1] || h.per[2] || h.sh0.empty()) return;
        float h0min = 3.4e38f, h0max = 0.0f;
        for (double v0 : h.sh0) {
            h0min = std::min(h0min, (float)v0);
            h0max = std::max(h0max, (float)v0);
        }
        if (!(h0min > 0.0f) || !(h0max >= 2.0f * h0min)) return;
        int nlev = 1;
        while (nlev < kMaxLevels && h0max >= h0min * (float)(1 << nlev)) nlev++;
        float th[kMaxLevels];
        th[0] = 0.0f;
        for (int L = 1; L < nlev; L++) th[L] = h0min * (float)(1 << L);
        int lo[kMaxLevels][3], hi[kMaxLevels][3];
        for (int L = 0; L < nlev; L++)
            for (int a = 0; a < 3; a++) { lo[L][a] = INT_MAX; hi[L][a] = INT_MIN; }
        const std::vector<double>* P[3] = {&h.sx, &h.sy, &h.sz};
        for (int64_t i = 0; i < h.n; i++) {
            const float v0 = (float)h.sh0[i];
            int L = 0;
            while (L + 1 < nlev && v0 >= th[L + 1]) L++;
            for (int a = 0; a < 3; a++) {
                const double q = ((*P[a])[i] - I.glo[a]) * I.iw[a];
                int ib = q < 0 ? 0 : (q >= I.nf[a] ? I.nf[a] - 1 : (int)std::floor(q));
                lo[L][a] = std::min(lo[L][a], ib >> L);
                hi[L][a] = std::max(hi[L][a], ib >> L);
            }
        }
        int64_t total = 0, lbase[kMaxLevels];
        int llo[kMaxLevels][3], lnf[kMaxLevels][3];
        for (int L = 0; L < nlev; L++) {
            int64_t cells = 1;
            for (int a = 0; a < 3; a++) {
                const int top = (I.nf[a] - 1) >> L;
                if (lo[L][a] > hi[L][a]) { lo[L][a] = 0; hi[L][a] = 0; }  // an empty level: one cell
                const int pad = 2;
                llo[L][a] = std::max(0, lo[L][a] - pad);
                const int e = std::min(top, hi[L][a] + pad);
                lnf[L][a] = e - llo[L][a] + 1;
                cells *= lnf[L][a];
            }
            lbase[L] = total;
            total += cells;
        }
        if (total > budget) return;  // keep one grid
        I.nlev = nlev;
        for (int L = 0; L < nlev; L++) {
            I.lev_h0[L] = th[L];
            I.lev_base[L] = lbase[L];
            for (int a = 0; a < 3; a++) {
                I.lev_lo[L][a] = llo[L][a];
                I.lev_nf[L][a] = lnf[L][a];
            }
        }
        I.ncells = total;
    }

    void assign_cell_bases() {
        int64_t base = 0;
        levels_active_ = false;
        for (size_t b = 0; b < imp_.size(); b++) {
            ImpactD& I = tab_[b];
            if (imp_[b].used && imp_[b].alive && imp_[b].committed) {
                I.cell_base = base;
                base += I.ncells;
                levels_active_ = levels_active_ || I.nlev > 1;
            } else {
                I.cell_base = 0;
                I.alive = 0;
                I.mask = 0;
            }
        }
        if (base >= (int64_t)0xfffffff0ll) throw SphError(SPH_ERR_CAPACITY, "too many traversal cells");
        C_ = base;
        if (C_ + 1 > Ccap_) {
            dfree(cell_cnt_);
            dfree(cell_hmax_);
            Ccap_ = std::max<int64_t>(C_ + 1, (int64_t)(Ccap_ * 1.5));
            cell_cnt_ = dalloc<int32_t>(Ccap_);
            cell_hmax_ = dalloc<unsigned int>(Ccap_);
        }
        ensure_scratch();
    }

    void ensure_scratch() {
        size_t need = std::max(radix_scratch_bytes(std::max<int64_t>(Gcap_, 1)),
                               scan_scratch_bytes(std::max<int64_t>(Ccap_, 1))) + 256;
        if (need > scratch_bytes_) {
            dfree(scratch_);
            scratch_bytes_ = need;
            scratch_ = dalloc<char>(need);
        }
    }

    // gid ranges: first fit in a free list
    int64_t alloc_gids(int64_t n) {
        for (size_t i = 0; i < free_gids_.size(); i++) {
            if (free_gids_[i].second >= n) {
                int64_t base = free_gids_[i].first;
                free_gids_[i].first += n;
                free_gids_[i].second -= n;
                if (free_gids_[i].second == 0) free_gids_.erase(free_gids_.begin() + i);
                return base;
            }
        }
        int64_t base = G_;
        G_ += n;
        return base;
    }
    void release_gids(int64_t base, int64_t n) {
        if (n <= 0) return;
        free_gids_.push_back({base, n});
        std::sort(free_gids_.begin(), free_gids_.end());
        std::vector<std::pair<int64_t, int64_t>> merged;
        for (auto& r : free_gids_) {
            if (!merged.empty() && merged.back().first + merged.back().second == r.first)
                merged.back().second += r.second;
            else
                merged.push_back(r);
        }
        free_gids_ = merged;
        // trailing free range shrinks the id space
        if (!free_gids_.empty() && free_gids_.back().first + free_gids_.back().second == G_) {
            G_ = free_gids_.back().first;
            free_gids_.pop_back();
        }
    }

    void ensure_gid_capacity(int64_t need) {
        if (need <= Gcap_) return;
        int64_t nc = std::max<int64_t>(need, (int64_t)(Gcap_ * 1.5) + 1024);
        int32_t* npos = dalloc<int32_t>(nc);
        if (pos_of_gid_ && Gcap_ > 0)
            DSPH_CUDA(cudaMemcpyAsync(npos, pos_of_gid_, sizeof(int32_t) * Gcap_, cudaMemcpyDeviceToDevice, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        dfree(pos_of_gid_);
        pos_of_gid_ = npos;
        for (uint32_t** p : {&keys_by_gid_, &skeys_, &tkeys_}) { dfree(*p); *p = dalloc<uint32_t>(nc); }
        for (int32_t** p : {&sgid_, &tgid_}) { dfree(*p); *p = dalloc<int32_t>(nc); }
        Gcap_ = nc;
        ensure_scratch();
    }

    void ensure_particle_capacity(int64_t need) {
        if (need <= cap_) return;
        int64_t nc = std::max<int64_t>(need, (int64_t)(cap_ * 1.5) + 1024);
        DSPH_CUDA(cudaStreamSynchronize(st_));
        for (int side = 0; side < 2; side++) {
            bool keep = side == cur_;
            auto grow = [&](auto*& p, size_t esz) {
                using T = std::remove_reference_t<decltype(*p)>;
                T* q = dalloc<T>(nc);
                if (keep && p && N_ > 0)
                    DSPH_CUDA(cudaMemcpyAsync(q, p, esz * N_, cudaMemcpyDeviceToDevice, st_));
                DSPH_CUDA(cudaStreamSynchronize(st_));
                dfree(p);
                p = q;
            };
            for (int c = 0; c < kND; c++) grow(dcol_[side][c], sizeof(double));
            for (int c = 0; c < kNR; c++) grow(rcol_[side][c], sizeof(R));
            grow(mat_[side], 1);
            grow(fixed_[side], 1);
            grow(impc_[side], 2);
            grow(gid_[side], 4);
        }
        for (int c = 0; c < kNDer; c++) { dfree(der_[c]); der_[c] = dalloc<R>(nc); }
        dfree(pf_); pf_ = dalloc<float4>(nc);
        dfree(pf_tmp_); pf_tmp_ = dalloc<float4>(nc);
        dfree(cpk_tmp_); cpk_tmp_ = dalloc<uint32_t>(nc);
        dfree(pk_); pk_ = dalloc<float2>(sizeof(R) == 4 ? nc : 1);
        dfree(lf_); lf_ = dalloc<float4>(nc);
        dfree(fr_); fr_ = dalloc<float4>(sizeof(R) == 4 ? 6 * nc : 2);  // 96-byte records, 32-byte aligned
        dfree(tasks_); tasks_ = dalloc<int32_t>(nc);
        dfree(cpk_); cpk_ = dalloc<uint32_t>(nc);
        dfree(refbin_); refbin_ = dalloc<unsigned long long>(nc);
        dfree(src_); src_ = dalloc<int32_t>(nc);
        dfree(nbr_cnt_); nbr_cnt_ = dalloc<int32_t>(nc);
        dfree(hlist_); hlist_ = dalloc<float>(nc);
        dfree(xcnt_); xcnt_ = dalloc<int32_t>(nc);
        dfree(xnbr_); xnbr_ = dalloc<int32_t>((size_t)nc * kExtraCap);
        // derived columns start at zero so reads before the first force pass are defined
        for (int c = 0; c < kNDer; c++) DSPH_CUDA(cudaMemsetAsync(der_[c], 0, sizeof(R) * nc, st_));
        cap_ = nc;
        alloc_lists();
    }

    void alloc_lists() {
        dfree(nbr_);
        const size_t blocks = (size_t)(cap_nbr_ + 3) / 4;  // lists are stored in 4-entry blocks
        nbr_ = dalloc<int32_t>((size_t)cap_ * blocks * 4);
    }

    // Moves staged impacts onto the device.
    void commit() {
        bool any = false;
        for (auto& h : imp_) any |= (h.used && h.alive && !h.committed);
        if (!any) return;
        pull_table();
        if (tab_.size() < imp_.size()) tab_.resize(imp_.size());
        int64_t add = 0;
        for (auto& h : imp_) if (h.used && h.alive && !h.committed) add += h.n;
        ensure_particle_capacity(N_ + add);
        for (size_t b = 0; b < imp_.size(); b++) {
            ImpactH& h = imp_[b];
            if (!(h.used && h.alive && !h.committed)) continue;
            ImpactD& I = tab_[b];
            std::memset(&I, 0, sizeof(ImpactD));
            fill_params(I, h);
            make_fine_grid(I, h);
            I.alive = 1;
            I.t = h.t;
            I.max_steps = h.step_limit;
            I.dt_bits = 0x7ff0000000000000ull;
            I.nc[0] = I.nc[1] = I.nc[2] = 1;
            I.cw[0] = I.cw[1] = I.cw[2] = 1;
            h.gid_base = alloc_gids(h.n);
            I.gid_base = h.gid_base;
            ensure_gid_capacity(G_);
            upload_impact(b, h);
            h.committed = true;
            // staging no longer needed except materials (seeding) and flaws
            h.sx.clear(); h.sy.clear(); h.sz.clear(); h.svx.clear(); h.svy.clear(); h.svz.clear();
            h.smass.clear(); h.su.clear(); h.seps.clear(); h.sh0.clear(); h.smat.clear(); h.sfixed.clear();
            h.sx.shrink_to_fit(); h.sy.shrink_to_fit(); h.sz.shrink_to_fit();
            h.gen.reset();
        }
        assign_cell_bases();
        push_table();
        if (any_multi()) sync_flaws();
        grid_valid_ = false;
    }

    bool any_multi() {
        for (auto& h : imp_) if (h.used && h.alive && h.multi) return true;
        return false;
    }

    template <class T>
    void dfill(T* p, int64_t n, T v) {
        if (n > 0) k_fill<T><<<(unsigned)((n + 255) / 256), 256, 0, st_>>>(p, n, v);
    }

    // Generated impact: the target lattice by k_gen_slab, the impactor from its
    // host-built coordinates, everything else filled on the device.
    void upload_generated(size_t b, ImpactH& h) {
        const GrazingLayout& L = *h.gen;
        const int64_t n = h.n, at = N_, ns = L.n_slab(), ni = (int64_t)L.px.size();
        const int c = cur_;
        double* coord = dalloc_tmp<double>(L.xs.size() + L.ys.size() + L.zs.size());
        std::vector<double> all(L.xs);
        all.insert(all.end(), L.ys.begin(), L.ys.end());
        all.insert(all.end(), L.zs.begin(), L.zs.end());
        DSPH_CUDA(cudaMemcpyAsync(coord, all.data(), sizeof(double) * all.size(), cudaMemcpyHostToDevice, st_));
        const int nx = (int)L.xs.size(), ny = (int)L.ys.size(), nz = (int)L.zs.size();
        if (ns > 0)
            k_gen_slab<R><<<(unsigned)((ns + 255) / 256), 256, 0, st_>>>(
                at, nx, ny, nz, coord, coord + nx, coord + nx + ny, L.wall, (R)L.m_target, dcol_[c][0],
                dcol_[c][1], dcol_[c][2], dcol_[c][4], dcol_[c][5], dcol_[c][6], dcol_[c][3],
                rcol_[c][RC_MASS], fixed_[c]);
        const int64_t ai = at + ns;
        if (ni > 0) {
            DSPH_CUDA(cudaMemcpyAsync(dcol_[c][0] + ai, L.px.data(), sizeof(double) * ni, cudaMemcpyHostToDevice, st_));
            DSPH_CUDA(cudaMemcpyAsync(dcol_[c][1] + ai, L.py.data(), sizeof(double) * ni, cudaMemcpyHostToDevice, st_));
            DSPH_CUDA(cudaMemcpyAsync(dcol_[c][2] + ai, L.pz.data(), sizeof(double) * ni, cudaMemcpyHostToDevice, st_));
            dfill(dcol_[c][3] + ai, ni, 0.0);
            dfill(dcol_[c][4] + ai, ni, L.vx);
            dfill(dcol_[c][5] + ai, ni, 0.0);
            dfill(dcol_[c][6] + ai, ni, L.vz);
            dfill(rcol_[c][RC_MASS] + ai, ni, (R)L.m_imp);
            dfill(fixed_[c] + ai, ni, (uint8_t)0);
        }
        dfill(mat_[c] + at, ns, (uint8_t)L.tgt_mat);
        dfill(mat_[c] + ai, ni, (uint8_t)L.imp_mat);
        const std::vector<R> eps(h.seps.begin(), h.seps.end()), h0(h.sh0.begin(), h.sh0.end());
        if (eps.empty()) dfill(rcol_[c][RC_EPSACT] + at, n, (R)1e30);
        else DSPH_CUDA(cudaMemcpyAsync(rcol_[c][RC_EPSACT] + at, eps.data(), sizeof(R) * n, cudaMemcpyHostToDevice, st_));
        if (h0.empty()) dfill(rcol_[c][RC_H0] + at, n, (R)h.prm.h_init);
        else DSPH_CUDA(cudaMemcpyAsync(rcol_[c][RC_H0] + at, h0.data(), sizeof(R) * n, cudaMemcpyHostToDevice, st_));
        dfill(rcol_[c][RC_HH] + at, n, (R)h.prm.h_init);
        for (int col : {RC_AX, RC_AY, RC_AZ, RC_DUDT, RC_D}) dfill(rcol_[c][col] + at, n, R(0));
        for (int q = 0; q < 6; q++) {
            dfill(rcol_[c][RC_S0 + q] + at, n, R(0));
            dfill(rcol_[c][RC_DS0 + q] + at, n, R(0));
        }
        dfill(impc_[c] + at, n, (uint16_t)b);
        k_gid_iota<<<(unsigned)((n + 255) / 256), 256, 0, st_>>>(gid_[c], pos_of_gid_, n, h.gid_base, at);
        DSPH_CUDA(cudaGetLastError());
        DSPH_CUDA(cudaStreamSynchronize(st_));  // the host vectors above must outlive the copies
        free_tmp();
        N_ += n;
    }

    void upload_impact(size_t b, ImpactH& h) {
        if (h.gen) {
            upload_generated(b, h);
            return;
        }
        int64_t n = h.n, at = N_;
        if (n == 0) return;
        auto up = [&](auto* dst, const auto& src) {
            using T = std::remove_pointer_t<decltype(dst)>;
            std::vector<T> tmp(src.begin(), src.end());
            DSPH_CUDA(cudaMemcpyAsync(dst + at, tmp.data(), sizeof(T) * n, cudaMemcpyHostToDevice, st_));
            DSPH_CUDA(cudaStreamSynchronize(st_));
        };
        int c = cur_;
        up(dcol_[c][0], h.sx); up(dcol_[c][1], h.sy); up(dcol_[c][2], h.sz); up(dcol_[c][3], h.su);
        up(dcol_[c][4], h.svx); up(dcol_[c][5], h.svy); up(dcol_[c][6], h.svz);
        up(rcol_[c][RC_MASS], h.smass);
        up(rcol_[c][RC_EPSACT], h.seps);
        up(rcol_[c][RC_H0], h.sh0);
        std::vector<double> hinit(n, h.prm.h_init);
        up(rcol_[c][RC_HH], hinit);
        for (int col : {RC_AX, RC_AY, RC_AZ, RC_DUDT, RC_D})
            DSPH_CUDA(cudaMemsetAsync(rcol_[c][col] + at, 0, sizeof(R) * n, st_));
        for (int q = 0; q < 6; q++) {
            DSPH_CUDA(cudaMemsetAsync(rcol_[c][RC_S0 + q] + at, 0, sizeof(R) * n, st_));
            DSPH_CUDA(cudaMemsetAsync(rcol_[c][RC_DS0 + q] + at, 0, sizeof(R) * n, st_));
        }
        std::vector<uint8_t> m8(n);
        for (int64_t i = 0; i < n; i++) m8[i] = (uint8_t)h.smat[i];
        up(mat_[c], m8);
        up(fixed_[c], h.sfixed);
        std::vector<uint16_t> im(n, (uint16_t)b);
        up(impc_[c], im);
        std::vector<int32_t> g(n), pos(n);
        for (int64_t i = 0; i < n; i++) { g[i] = (int32_t)(h.gid_base + i); pos[i] = (int32_t)(at + i); }
        up(gid_[c], g);
        DSPH_CUDA(cudaMemcpyAsync(pos_of_gid_ + h.gid_base, pos.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        N_ += n;
    }

    // Multi-flaw thresholds on the device: one pool of thresholds (engine
    // precision) holding a segment per impact, and per particle id the begin /
    // end of its thresholds in the pool.  A committed impact's segment is
    // appended once; a removed impact's segment turns dead and stays until the
    // pool has to grow while more than half of it is dead, when the live
    // segments are rewritten compactly.  Admitting or retiring an impact thus
    // moves only that impact's thresholds.
    void sync_flaws() {
        if (G_ > flaw_gcap_) {  // per-id ranges follow the id space
            const int64_t nc = std::max<int64_t>(G_, (int64_t)(flaw_gcap_ * 1.5) + 1024);
            int64_t* nb = dalloc<int64_t>(nc);
            int64_t* ne = dalloc<int64_t>(nc);
            if (flaw_gcap_ > 0) {
                DSPH_CUDA(cudaMemcpyAsync(nb, flaw_beg_d_, sizeof(int64_t) * flaw_gcap_, cudaMemcpyDeviceToDevice, st_));
                DSPH_CUDA(cudaMemcpyAsync(ne, flaw_end_d_, sizeof(int64_t) * flaw_gcap_, cudaMemcpyDeviceToDevice, st_));
            }
            DSPH_CUDA(cudaStreamSynchronize(st_));
            dfree(flaw_beg_d_);
            dfree(flaw_end_d_);
            flaw_beg_d_ = nb;
            flaw_end_d_ = ne;
            flaw_gcap_ = nc;
        }
        int64_t need = 0;
        for (auto& h : imp_)
            if (h.used && h.alive && h.committed && h.multi && !h.flaws_on_device) need += (int64_t)h.flaw_eps.size();
        if (need == 0) return;
        if (flaw_used_ + need > flaw_cap_) {
            const bool compact = flaw_used_ - flaw_live_ > flaw_live_;  // more than half dead
            const int64_t keep = compact ? flaw_live_ : flaw_used_;
            const int64_t nc = std::max<int64_t>(keep + need, (int64_t)((keep + need) * 1.5) + 4096);
            R* np = dalloc<R>(nc);
            if (!compact && flaw_used_ > 0)
                DSPH_CUDA(cudaMemcpyAsync(np, flaw_eps_d_, sizeof(R) * flaw_used_, cudaMemcpyDeviceToDevice, st_));
            DSPH_CUDA(cudaStreamSynchronize(st_));
            dfree(flaw_eps_d_);
            flaw_eps_d_ = np;
            flaw_cap_ = nc;
            if (compact) {  // every live segment is written again below
                flaw_used_ = 0;
                flaw_live_ = 0;
                for (auto& h : imp_) h.flaws_on_device = false;
            }
        }
        std::vector<R> seg;
        std::vector<int64_t> beg, end;
        for (auto& h : imp_) {
            if (!(h.used && h.alive && h.committed && h.multi) || h.flaws_on_device) continue;
            const int64_t nf = (int64_t)h.flaw_eps.size(), off = flaw_used_;
            seg.resize(std::max<int64_t>(nf, 1));
            for (int64_t q = 0; q < nf; q++) seg[q] = (R)h.flaw_eps[q];
            beg.resize(h.n);
            end.resize(h.n);
            for (int64_t l = 0; l < h.n; l++) {
                beg[l] = off + h.flaw_ptr[l];
                end[l] = off + h.flaw_ptr[l + 1];
            }
            if (nf > 0)
                DSPH_CUDA(cudaMemcpyAsync(flaw_eps_d_ + off, seg.data(), sizeof(R) * nf, cudaMemcpyHostToDevice, st_));
            if (h.n > 0) {
                DSPH_CUDA(cudaMemcpyAsync(flaw_beg_d_ + h.gid_base, beg.data(), sizeof(int64_t) * h.n,
                                          cudaMemcpyHostToDevice, st_));
                DSPH_CUDA(cudaMemcpyAsync(flaw_end_d_ + h.gid_base, end.data(), sizeof(int64_t) * h.n,
                                          cudaMemcpyHostToDevice, st_));
            }
            DSPH_CUDA(cudaStreamSynchronize(st_));  // the staging vectors are reused
            flaw_used_ += nf;
            flaw_live_ += nf;
            h.flaws_on_device = true;
        }
    }

    void set_masks(const std::vector<int32_t>& mask, const std::vector<double>* dt,
                   const std::vector<double>* t_end) {
        int nimp = (int)imp_.size();
        if (nimp == 0) return;
        size_t bytes = sizeof(int32_t) * nimp + sizeof(double) * 2 * nimp + 64;
        if (mask_buf_bytes_ < bytes) {
            dfree(mask_buf_);
            mask_buf_bytes_ = bytes * 2;
            mask_buf_ = dalloc<char>(mask_buf_bytes_);
        }
        char* p = mask_buf_;
        int32_t* dm = (int32_t*)p;
        double* ddt = (double*)(p + ((sizeof(int32_t) * nimp + 15) / 16) * 16);
        double* dte = ddt + nimp;
        DSPH_CUDA(cudaMemcpyAsync(dm, mask.data(), sizeof(int32_t) * nimp, cudaMemcpyHostToDevice, st_));
        if (dt) DSPH_CUDA(cudaMemcpyAsync(ddt, dt->data(), sizeof(double) * nimp, cudaMemcpyHostToDevice, st_));
        if (t_end) DSPH_CUDA(cudaMemcpyAsync(dte, t_end->data(), sizeof(double) * nimp, cudaMemcpyHostToDevice, st_));
        launch_small(k_set_mask_dt, nimp, (const int32_t*)dm, dt ? (const double*)ddt : nullptr,
                     t_end ? (const double*)dte : nullptr);
        DSPH_CUDA(cudaStreamSynchronize(st_));  // host vectors are temporaries
    }

    void set_all_masks() {
        std::vector<int32_t> mask(imp_.size(), 0);
        for (size_t b = 0; b < imp_.size(); b++)
            if (imp_[b].used && imp_[b].alive && imp_[b].committed) mask[b] = 1;
        set_masks(mask, nullptr, nullptr);
    }

    int key_bits() const {
        int bits = 1;
        while ((1ll << bits) <= C_) bits++;
        return bits;
    }

    // Cell sort of all resident particles and gather of the carried state.
    void sort_reorder(bool count_changes) {
        if (N_ == 0 && !count_changes) return;
        if (G_ == 0) {  // no particle was ever added: nothing to order
            N_ = 0;
            grid_valid_ = true;
            return;
        }
        const int nimp = (int)imp_.size();
        DSPH_CUDA(cudaMemsetAsync(keys_by_gid_, 0xff, sizeof(uint32_t) * std::max<int64_t>(G_, 1), st_));
        DSPH_CUDA(cudaMemsetAsync(cell_cnt_, 0, sizeof(int32_t) * (C_ + 1), st_));
        const int keep_cls = cur_cls_;
        cls(KC_SORT);
        launch_small(k_impact_reset_omax, nimp);
        launch_n_raw(k_fine_keys<R>, N_, view(), keys_by_gid_, cell_cnt_, pf_tmp_, cpk_tmp_);
        prof_begin();
        launches_ += radix_sort_pairs(keys_by_gid_, nullptr, skeys_, sgid_, tkeys_, tgid_, G_,
                                      key_bits(), scratch_, st_);
        launches_ += exclusive_scan_i32(cell_cnt_, cell_cnt_, C_ + 1, scratch_, st_);
        prof_end();
        int64_t n_new = N_;
        if (count_changes) {
            DSPH_CUDA(cudaMemcpyAsync(flags_h_ + 2, cell_cnt_ + C_, sizeof(int32_t), cudaMemcpyDeviceToHost, st_));
            DSPH_CUDA(cudaStreamSynchronize(st_));
            n_new = flags_h_[2];
        }
        const int alt = cur_ ^ 1;
        if (n_new > 0) {
            launch_n_raw(k_make_src, n_new, n_new, (const int32_t*)sgid_, (const int32_t*)pos_of_gid_, src_);
            GatherCols g{};
            for (int c = 0; c < kND; c++) { g.din[c] = dcol_[cur_][c]; g.dout[c] = dcol_[alt][c]; }
            g.nr = kNR;
            for (int c = 0; c < kNR; c++) { g.rin[c] = rcol_[cur_][c]; g.rout[c] = rcol_[alt][c]; }
            g.b_in[0] = mat_[cur_]; g.b_out[0] = mat_[alt];
            g.b_in[1] = fixed_[cur_]; g.b_out[1] = fixed_[alt];
            g.imp_in = impc_[cur_]; g.imp_out = impc_[alt];
            g.gid_in = gid_[cur_]; g.gid_out = gid_[alt];
            g.pf_in = pf_tmp_; g.pf_out = pf_;
            g.cpk_in = cpk_tmp_; g.cpk_out = cpk_;
            g.lf_out = lf_; g.imps = tab_d_;
            launch_n_raw(k_gather<R>, n_new, n_new, (const int32_t*)src_, g);
        }
        cur_ = alt;
        N_ = n_new;
        launch_n_raw(k_post_sort<R>, N_, view(), pos_of_gid_);
        launch_small(k_impact_ranges, nimp, (const int32_t*)cell_cnt_);
        cls(keep_cls);
        grid_valid_ = true;
    }

    // Neighbour lists.  The step uses one superset list (see k_list_thread);
    // capacity overflow is handled by the consumers' traversal fallback, and
    // the capacity grows for later steps when host_check reads the overflow.
    template <int KIND>
    void build_list(bool host_check) {
        if (N_ <= 0) return;
        const int nimp = (int)imp_.size();
        const int keep = cur_cls_;
        cls(KC_OTHER);
        launch_small(k_impact_reset_slack, nimp);
        cls(keep);
        for (int attempt = 0; attempt < 8; attempt++) {
            DSPH_CUDA(cudaMemsetAsync(flags_d_, 0, sizeof(int32_t), st_));
            DSPH_CUDA(cudaMemsetAsync(flags_d_ + 2, 0, sizeof(int32_t), st_));
            DSPH_CUDA(cudaMemsetAsync(xcnt_, 0, sizeof(int32_t) * N_, st_));
            if (list_mode_ == 1 && !levels_active_) {  // graded impacts: the per-thread builder
                DSPH_CUDA(cudaMemsetAsync(ntask_, 0, sizeof(int32_t), st_));
                launch_n_raw(k_column_tasks<R>, N_, view(), tasks_, ntask_);
                const int grid = std::max(1, std::min<int>(nsm_ * 8, (int)((N_ / 16 + 255) / 256) + 1));
                prof_begin();
                k_list_warp<R><<<grid, 256, 0, st_>>>(view(), (const int32_t*)tasks_, (const int32_t*)ntask_);
                launched((const void*)k_list_warp<R>);
                prof_end();
                launches_++;
            } else if (list_mode_ == 2 && !levels_active_) {
                prof_begin();
                k_list_wpp<R><<<(unsigned)((N_ + 7) / 8), 256, 0, st_>>>(view());
                launched((const void*)k_list_wpp<R>);
                prof_end();
                launches_++;
            } else {
                launch_list_thread(0);
            }
            cls(KC_OTHER);
            launch_n_raw(k_sort_extra<R>, N_, view(), 0);
            cls(keep);
            if (!host_check) return;
            DSPH_CUDA(cudaMemcpyAsync(flags_h_, flags_d_, sizeof(int32_t), cudaMemcpyDeviceToHost, st_));
            DSPH_CUDA(cudaStreamSynchronize(st_));
            if (flags_h_[0] <= cap_nbr_) return;
            cap_nbr_ = (int)(flags_h_[0] * 1.25) + 8;
            alloc_lists();
        }
        throw SphError(SPH_ERR_CAPACITY, "neighbour list capacity could not be satisfied");
    }

    void launch_list_thread(int refresh) {
        const int bs = block_ > 0 ? block_ : 256;
        prof_begin();
        if (levels_active_) {
            k_list_thread<R, true><<<(unsigned)((N_ + bs - 1) / bs), bs, 0, st_>>>(view(), refresh);
            launched((const void*)k_list_thread<R, true>);
        } else if (any_periodic()) {
            k_list_thread<R, false, true><<<(unsigned)((N_ + bs - 1) / bs), bs, 0, st_>>>(view(), refresh);
            launched((const void*)k_list_thread<R, false, true>);
        } else {
            k_list_thread<R, false, false><<<(unsigned)((N_ + bs - 1) / bs), bs, 0, st_>>>(view(), refresh);
            launched((const void*)k_list_thread<R, false, false>);
        }
        prof_end();
        launches_++;
    }

    // Device-controlled counterpart of refresh_list_if_needed (captured
    // steps): impacts whose h outgrew the slack in this step's density rounds
    // rebuild their lists on the device, the others' kernels return at once,
    // so the force pass keeps list walks instead of the traversal fallback.
    void refresh_list_device() {
        if (N_ <= 0 || list_mode_ != 0) return;  // other builders: the consumers' fallback
        const int keep = cur_cls_;
        cls(KC_LIST_FORCE);
        launch_n(k_refresh_begin<R>, N_);
        launch_list_thread(1);
        launch_n_raw(k_sort_extra<R>, N_, view(), 1);
        launch_small(k_impact_end_refresh, (int)imp_.size());
        cls(keep);
    }

    // Rebuild the superset list when some h outgrew its slack (avoids the
    // consumers' slower traversal fallback).
    void refresh_list_if_needed() {
        DSPH_CUDA(cudaMemcpyAsync(flags_h_ + 3, flags_d_ + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        if (flags_h_[3]) {
            const int keep = cur_cls_;
            cls(KC_LIST_FORCE);
            build_list<kListSuperset>(false);
            cls(keep);
        }
    }

    void hmax_pass(int which) {
        int64_t n = N_;
        if (n <= 0) return;
        prof_begin();
        k_hmax<R><<<(unsigned)((n + 255) / 256), 256, 0, st_>>>(view(), which);
        launched((const void*)k_hmax<R>);
        prof_end();
        launches_++;
    }

    void density_rounds(int iters, bool host_sync) {
        const int nimp = (int)imp_.size();
        cls(KC_GRID);
        launch_small(k_impact_begin_round, nimp, 2);
        for (int round = 0; round < 4; round++) {
            cls(KC_GRID);
            if (round > 0) launch_small(k_impact_begin_round, nimp, 0);  // max h carried over
            else hmax_pass(0);
            launch_small(k_ref_grid, nimp);
            launch_n(k_ref_bins<R>, N_);
            cls(KC_DENSITY);
            if (iters > 0) {  // also reduces the new max h
                if (levels_active_) launch_n_raw(k_density<R, true>, N_, view(), iters);
                else if (any_periodic()) launch_n_raw(k_density<R, false, true>, N_, view(), iters);
                else launch_n_raw(k_density<R, false, false>, N_, view(), iters);
            }
            else hmax_pass(1);
            cls(KC_GRID);
            DSPH_CUDA(cudaMemsetAsync(flags_d_ + 1, 0, sizeof(int32_t), st_));
            launch_small(k_round_check, nimp, flags_d_);
            if (host_sync) {
                DSPH_CUDA(cudaMemcpyAsync(flags_h_ + 1, flags_d_ + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st_));
                DSPH_CUDA(cudaStreamSynchronize(st_));
                if (!flags_h_[1]) break;
            }
        }
        final_grid_build(true);
    }

    // Reference grid and bins for the force pass; after_rounds: the max h is the
    // one the last density pass reduced.
    void final_grid_build(bool after_rounds = false) {
        const int nimp = (int)imp_.size();
        cls(KC_GRID);
        launch_small(k_impact_begin_round, nimp, after_rounds ? 3 : 1);
        if (!after_rounds) hmax_pass(0);
        launch_small(k_ref_grid, nimp);
        launch_n(k_ref_bins<R>, N_);
    }

    void forces(bool host_check) {
        if (host_check) refresh_list_if_needed();
        cls(KC_EOS);
        launch_n(k_eos<R>, N_);
        cls(KC_FORCE);
        launch_force();
    }

    void dt_reduce() {
        launch_small(k_dt_begin, (int)imp_.size());
        launch_n(k_dt<R>, N_);
    }

    void grow_lists_after_overflow() {
        DSPH_CUDA(cudaMemcpyAsync(flags_h_, flags_d_, sizeof(int32_t), cudaMemcpyDeviceToHost, st_));
        DSPH_CUDA(cudaStreamSynchronize(st_));
        if (flags_h_[0] > cap_nbr_) {
            cap_nbr_ = (int)(flags_h_[0] * 1.25) + 8;
            alloc_lists();
        }
    }

    void record_phases() {
        DSPH_CUDA(cudaEventSynchronize(ev_[5]));
        for (int i = 0; i < 5; i++) {
            float ms = 0;
            DSPH_CUDA(cudaEventElapsedTime(&ms, ev_[i], ev_[i + 1]));
            phase_ms_[i] = ms;
        }
    }

    // ------------------------------------------------------------- members
    int dev_;
    cudaStream_t st_{};
    cudaStream_t copy_st_{};   // host <-> device copies of the batched field I/O
    cudaEvent_t copy_ev_{};
    cudaStream_t out_st_{};    // device -> host copies of step_fields (the other link direction)
    cudaEvent_t out_ev_{};
    cudaEvent_t late_ev_{};    // step_fields: the inputs first read by the EOS pass have landed
    std::vector<void*> allocs_, tmp_;
    std::vector<sph_material> mats_h_;
    MatT<R>* mats_d_ = nullptr;
    std::vector<ImpactH> imp_;
    std::vector<ImpactD> tab_;
    ImpactD* tab_d_ = nullptr;
    int tab_cap_ = 0;
    int64_t N_ = 0, cap_ = 0, G_ = 0, Gcap_ = 0, C_ = 0, Ccap_ = 0;
    std::vector<std::pair<int64_t, int64_t>> free_gids_;
    int cur_ = 0;
    double* dcol_[2][kND] = {};
    R* rcol_[2][kNR] = {};
    uint8_t* mat_[2] = {};
    uint8_t* fixed_[2] = {};
    uint16_t* impc_[2] = {};
    int32_t* gid_[2] = {};
    R* der_[kNDer] = {};
    float4* pf_ = nullptr;
    float4* pf_tmp_ = nullptr;     // offsets / cells in the pre-sort order
    uint32_t* cpk_tmp_ = nullptr;
    float2* pk_ = nullptr;
    float4* lf_ = nullptr;         // list-frame coordinates and h
    float4* fr_ = nullptr;         // mixed-form force-source records, six float4 per particle
    int32_t* tasks_ = nullptr;
    int32_t* ntask_ = nullptr;
    unsigned int* cell_hmax_ = nullptr;
    int nsm_ = 148;
    uint32_t* cpk_ = nullptr;
    unsigned long long* refbin_ = nullptr;
    int32_t* src_ = nullptr;
    uint32_t *keys_by_gid_ = nullptr, *skeys_ = nullptr, *tkeys_ = nullptr;
    int32_t *sgid_ = nullptr, *tgid_ = nullptr, *pos_of_gid_ = nullptr;
    int32_t* cell_cnt_ = nullptr;
    int32_t* nbr_ = nullptr;
    int32_t* nbr_cnt_ = nullptr;
    float* hlist_ = nullptr;
    int32_t* xnbr_ = nullptr;
    int32_t* xcnt_ = nullptr;
    double slack_ = 0.03;
    int cap_nbr_ = 160;
    int32_t* flags_d_ = nullptr;
    int32_t* wait_err_d_ = nullptr;   // set by a kernel whose bounded wait ran out
    std::vector<int64_t> alloc_bytes_;  // sizes of allocs_, in the same order
    int64_t dev_bytes_ = 0;
    int force_staging_ = 0;
    bool levels_ = false;          // traversal-grid levels for impacts with a wide h0 range
    bool levels_active_ = false;   // some resident impact has levels
    bool host_direct_ = false;     // field I/O reaches device-accessible host buffers directly
                                   // (option; measured no faster than the staging copies on GB300)
    bool pageable_access_ = false; // the device reads pageable host memory (host page tables)
    int32_t* flags_h_ = nullptr;
    void* scratch_ = nullptr;
    size_t scratch_bytes_ = 0;
    double* stage_d_ = nullptr;
    int64_t stage_cap_ = 0;
    char* mask_buf_ = nullptr;
    size_t mask_buf_bytes_ = 0;
    int64_t* flaw_beg_d_ = nullptr;  // per particle id: its thresholds in the pool
    int64_t* flaw_end_d_ = nullptr;
    int64_t flaw_gcap_ = 0;
    R* flaw_eps_d_ = nullptr;        // the pool of thresholds
    int64_t flaw_cap_ = 0, flaw_used_ = 0, flaw_live_ = 0;
    int block_ = 128;
    double cell_factor_ = 1.0;
    double cell_factor_z_ = 1.0;  // z cell height relative to the x / y width
    int list_mode_ = 0;   // 0: thread per particle, 1: warp per column run
    bool use_graphs_ = true;
    uint64_t layout_epoch_ = 1;
    // kGraphHead / kGraphTail: the two halves of a host-dt step (step_head,
    // step_tail), for step_fields' transfers between them
    enum { kGraphTwo = 0, kGraphOne = 1, kGraphHostDt = 2, kGraphHead = 3, kGraphTail = 4, kGraphKinds = 5 };
    cudaGraphExec_t graph_exec_[kGraphKinds][2] = {};
    uint64_t graph_key_[kGraphKinds][2] = {};
    int64_t graph_n_[kGraphKinds][2] = {{-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}, {-1, -1}};
    int64_t graph_launches_[kGraphKinds][2] = {};
    int64_t launches_ = 0;
    bool profiling_ = false;
    cudaEvent_t ev_[6]{};
    double phase_ms_[5];
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> prof_pool_;
    std::vector<int> prof_cls_;
    size_t np_ = 0;
    int cur_cls_ = 0;
    double kstat_ms_[KC_N] = {};
    int64_t kstat_n_[KC_N] = {};
    cudaEvent_t user_ev_[16]{};
    bool grid_valid_ = false;
};

}  // namespace dsph
