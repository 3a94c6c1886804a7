// engine_kernels.cuh -- the CUDA kernels of one SPH step over a batch of impacts.
//
// Data layout (HBM, structure of arrays, sorted by (impact, traversal cell,
// original id) at every step):
//   carried state      x y z u (FP64); vel, acc, dudt, mass, h, D, eps_act, h0,
//                      S[6], dSdt[6] (type R); mat, fixed (u8); impact (u16); gid (i32)
//   derived per step   rho P cs csig Pf dscale Rart sigmax eps_work,
//                      Pf/rho^2, dscale/rho^2, m/rho, new dudt, new dSdt[6]
//   geometry           pf = float4(offset from own traversal-cell origin, h),
//                      cpk = packed traversal-cell coordinates,
//                      refbin = packed reference-grid bins (sph.hpp:142-146)
//   neighbour lists    column-major nbr[t * stride + k], count per particle
//
// Reference semantics kept exactly: the neighbour criteria r < 2 h_i (density,
// self included, sph.hpp:193) and j != i, r < 2 hbar, r != 0 (sph.hpp:222,287),
// restricted to the 27-cell stencil of the reference grid of width
// ext / floor(ext / 2 h_max) (sph.hpp:147-182).  The traversal itself runs on a
// finer grid of width ~h_init and visits, per target, only the cell columns
// that intersect its search sphere.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "dsph_math.cuh"

namespace dsph {

constexpr uint32_t kInvalidKey = 0xffffffffu;
constexpr int kListDensity = 0;
constexpr int kListForce = 1;

// Per-impact parameters and per-step scalars, resident on the device.
struct ImpactD {
    double eta, h_init, alpha, beta, eps, alpha_u, cfl, eps_as;
    int32_t damage_on, multi_flaw, use_h0, mask;   // mask: takes part in this phase
    double dlo[3], dhi[3];
    int32_t per[3], active;                        // active: density round still running
    // traversal grid (fixed while the impact is resident)
    double glo[3], w[3], iw[3];
    float wf[3], Lf[3];
    int32_t nf[3], alive;
    int64_t cell_base, ncells;
    // reference grid of the last build (sph.hpp:147-157)
    int32_t nc[3], rounds;
    double cw[3];
    double h_max, hmax0;
    float hmax_f, margin;
    double inv_poly_eta;                           // 1 / W-polynomial at q = 1/eta
    float hcap;                                    // upper bound of h (2 max h0)
    int32_t pad0;
    // step scalars
    double dt, t, t_end;
    int64_t nsteps;
    int64_t off, n;                                // sorted particle range
    int64_t gid_base;
    unsigned long long hmax_bits, hm_bits, dt_bits;
    unsigned int omax_bits, pad1;
};

template <class R>
struct View {
    int64_t n;          // resident particles
    int64_t stride;     // neighbour list column stride
    int32_t cap;        // neighbour list capacity per particle
    int32_t pad;
    double *x, *y, *z, *u;
    R *vx, *vy, *vz, *ax, *ay, *az, *dudt, *mass, *hh, *D, *eps_act, *h0;
    R* S[6];
    R* dS[6];
    uint8_t *mat, *fixed;
    uint16_t* imp;
    int32_t* gid;
    R *rho, *P, *cs, *csig, *Pf, *dscale, *Rart, *sigmax, *epsw, *pfr2, *dsr2, *vol, *dudt_new;
    R* dS_new[6];
    float4* pf;
    uint32_t* cpk;
    unsigned long long* refbin;
    const int32_t* cell_ptr;
    int32_t* nbr;
    int32_t* nbr_cnt;
    int32_t* flags;     // [0] list overflow max, [1] any impact still in a density round
    ImpactD* imps;
    const MatT<R>* mats;
    const int64_t* flaw_ptr;   // by gid, multi-flaw extension
    const R* flaw_eps;
};

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }

__device__ __forceinline__ unsigned long long dbits(double v) {
    return (unsigned long long)__double_as_longlong(v);
}
__device__ __forceinline__ double bitsd(unsigned long long b) {
    return __longlong_as_double((long long)b);
}

// Per-impact atomic max / min on the bit pattern of a non-negative double (bit
// order equals value order there).  A full warp whose lanes all target the same
// impact combines in registers first and issues one atomic.
__device__ __forceinline__ bool warp_same_target(const void* addr) {
    unsigned act = __activemask();
    if (act != 0xffffffffu) return false;
    return __match_any_sync(act, (unsigned long long)addr) == act;
}

__device__ __forceinline__ void impact_atomic_max(unsigned long long* addr, double v) {
    unsigned long long b = dbits(v);
    if (warp_same_target(addr)) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
            b = x > b ? x : b;
        }
        if ((threadIdx.x & 31) == 0) atomicMax(addr, b);
    } else {
        atomicMax(addr, b);
    }
}

__device__ __forceinline__ void impact_atomic_min(unsigned long long* addr, double v) {
    unsigned long long b = dbits(v);
    if (warp_same_target(addr)) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
            b = x < b ? x : b;
        }
        if ((threadIdx.x & 31) == 0) atomicMin(addr, b);
    } else {
        atomicMin(addr, b);
    }
}

__device__ __forceinline__ void impact_atomic_max_u32(unsigned int* addr, unsigned int b) {
    if (warp_same_target(addr)) {
        b = __reduce_max_sync(0xffffffffu, b);
        if ((threadIdx.x & 31) == 0) atomicMax(addr, b);
    } else {
        atomicMax(addr, b);
    }
}

__device__ __forceinline__ int sat_int(double q) {
    if (q != q) return 0;
    if (q >= 2147483647.0) return 2147483647;
    if (q <= -2147483648.0) return (-2147483647 - 1);
    return (int)q;
}

// Reference-grid bin of one coordinate (sph.hpp:142-146), exact FP64.
__device__ __forceinline__ int ref_bin(const ImpactD& I, int a, double c) {
    int i = sat_int(__ddiv_rn(__dsub_rn(c, I.dlo[a]), I.cw[a]));
    if (i < 0) i = 0;
    if (i >= I.nc[a]) i = I.nc[a] - 1;
    return i;
}

// Is j's reference cell in i's 27-cell stencil (sph.hpp:166-177)?
__device__ __forceinline__ bool ref_member(unsigned long long bi, unsigned long long bj,
                                           const ImpactD& I) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int nc = I.nc[a];
        if (nc == 1) continue;
        int ia = (int)((bi >> (21 * a)) & 0x1fffffull);
        int ja = (int)((bj >> (21 * a)) & 0x1fffffull);
        int d = ja - ia;
        if (I.per[a]) {
            d = ((d % nc) + nc) % nc;
            if (!(d == 0 || d == 1 || d == nc - 1)) return false;
        } else if (d < -1 || d > 1) {
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void unpack_cell(uint32_t c, int& cx, int& cy, int& cz) {
    cx = (int)(c & 2047u);
    cy = (int)((c >> 11) & 2047u);
    cz = (int)(c >> 22);
}

// FP32 separation i - j from cell-relative offsets (the "FP64 cell origin +
// FP32 offset" representation), minimum image on periodic axes.
__device__ __forceinline__ void sep_f32(const ImpactD& I, float4 pi, uint32_t ci, float4 pj,
                                        uint32_t cj, float& dx, float& dy, float& dz) {
    int ix, iy, iz, jx, jy, jz;
    unpack_cell(ci, ix, iy, iz);
    unpack_cell(cj, jx, jy, jz);
    dx = (pi.x - pj.x) + (float)(ix - jx) * I.wf[0];
    dy = (pi.y - pj.y) + (float)(iy - jy) * I.wf[1];
    dz = (pi.z - pj.z) + (float)(iz - jz) * I.wf[2];
    if (I.per[0]) dx -= I.Lf[0] * rintf(dx / I.Lf[0]);
    if (I.per[1]) dy -= I.Lf[1] * rintf(dy / I.Lf[1]);
    if (I.per[2]) dz -= I.Lf[2] * rintf(dz / I.Lf[2]);
}

// Exact FP64 separation and distance in the reference's operation order
// (sph.hpp:130-136 and vec3.hpp norm): no contraction, IEEE divide and sqrt.
template <class R>
__device__ __forceinline__ double sep_exact(const View<R>& v, const ImpactD& I, int64_t i, int64_t j,
                                            double& dx, double& dy, double& dz) {
    dx = __dsub_rn(v.x[i], v.x[j]);
    dy = __dsub_rn(v.y[i], v.y[j]);
    dz = __dsub_rn(v.z[i], v.z[j]);
    if (I.per[0]) { double L = __dsub_rn(I.dhi[0], I.dlo[0]); dx = __dsub_rn(dx, __dmul_rn(L, round(__ddiv_rn(dx, L)))); }
    if (I.per[1]) { double L = __dsub_rn(I.dhi[1], I.dlo[1]); dy = __dsub_rn(dy, __dmul_rn(L, round(__ddiv_rn(dy, L)))); }
    if (I.per[2]) { double L = __dsub_rn(I.dhi[2], I.dlo[2]); dz = __dsub_rn(dz, __dmul_rn(L, round(__ddiv_rn(dz, L)))); }
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// Visit every traversal cell column that intersects the sphere of radius Rs
// around particle k (sorted index), cell by cell; calls f(j, dxc, dyc, dzc)
// where d?c are the FP32 cell-origin differences (i's cell minus j's cell).
template <class R, class F>
__device__ __forceinline__ void traverse(const View<R>& v, const ImpactD& I, float4 pi,
                                         uint32_t ci, float Rs, F&& f) {
    int c[3];
    unpack_cell(ci, c[0], c[1], c[2]);
    const float o[3] = {pi.x, pi.y, pi.z};
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float w = I.wf[a];
        int l = c[a] + (int)floorf((o[a] - Rs) / w);
        int h = c[a] + (int)floorf((o[a] + Rs) / w);
        int nf = I.nf[a];
        if (I.per[a]) {
            if (h - l + 1 > nf) { l = c[a] - nf / 2; h = l + nf - 1; }
        } else {  // clamped like the binning, so out-of-grid particles meet
            l = l < 0 ? 0 : (l > nf - 1 ? nf - 1 : l);
            h = h < 0 ? 0 : (h > nf - 1 ? nf - 1 : h);
        }
        lo[a] = l;
        hi[a] = h;
    }
    for (int ix = lo[0]; ix <= hi[0]; ix++) {
        int wx = ix;
        if (I.per[0]) wx = ((ix % I.nf[0]) + I.nf[0]) % I.nf[0];
        float dxc = (float)(c[0] - ix) * I.wf[0];
        for (int iy = lo[1]; iy <= hi[1]; iy++) {
            int wy = iy;
            if (I.per[1]) wy = ((iy % I.nf[1]) + I.nf[1]) % I.nf[1];
            float dyc = (float)(c[1] - iy) * I.wf[1];
            const int64_t colbase = I.cell_base + ((int64_t)wx * I.nf[1] + wy) * I.nf[2];
            if (!I.per[2]) {
                // z-cells of a column are contiguous in sorted order
                int64_t cz = lo[2];
                int32_t s = v.cell_ptr[colbase + lo[2]];
                const int32_t e = v.cell_ptr[colbase + hi[2] + 1];
                int32_t next = v.cell_ptr[colbase + cz + 1];
                float dzc = (float)(c[2] - (int)cz) * I.wf[2];
                for (int32_t j = s; j < e; j++) {
                    while (j >= next) {
                        cz++;
                        next = v.cell_ptr[colbase + cz + 1];
                        dzc = (float)(c[2] - (int)cz) * I.wf[2];
                    }
                    f(j, dxc, dyc, dzc);
                }
            } else {
                for (int iz = lo[2]; iz <= hi[2]; iz++) {
                    int wz = ((iz % I.nf[2]) + I.nf[2]) % I.nf[2];
                    float dzc = (float)(c[2] - iz) * I.wf[2];
                    int32_t s = v.cell_ptr[colbase + wz], e = v.cell_ptr[colbase + wz + 1];
                    for (int32_t j = s; j < e; j++) f(j, dxc, dyc, dzc);
                }
            }
        }
    }
}

// ---------------------------------------------------------------- kernels

// Kick (half step with the old acceleration) and drift (sph.hpp:360-361).
template <class R>
static __global__ void k_kick_drift(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask || v.fixed[k]) return;
    const double dt = I.dt;
    const R hd = (R)(0.5 * dt);
    R vx = v.vx[k] + v.ax[k] * hd;
    R vy = v.vy[k] + v.ay[k] * hd;
    R vz = v.vz[k] + v.az[k] * hd;
    v.vx[k] = vx;
    v.vy[k] = vy;
    v.vz[k] = vz;
    v.x[k] += (double)vx * dt;
    v.y[k] += (double)vy * dt;
    v.z[k] += (double)vz * dt;
}

__device__ __forceinline__ int fine_cell(const ImpactD& I, int a, double c, double& frac) {
    double q = (c - I.glo[a]) * I.iw[a];
    double fl = floor(q);
    int i = sat_int(fl);
    if (i < 0) i = 0;
    if (i >= I.nf[a]) i = I.nf[a] - 1;
    frac = q - (double)i;  // offset in cells from the (clamped) cell origin
    return i;
}

// Traversal-cell key of every resident particle, scattered into gid order,
// plus per-cell counts.
template <class R>
static __global__ void k_fine_keys(View<R> v, uint32_t* keys_by_gid, int32_t* cell_count) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.alive) return;  // leaves the arrays at this sort (key stays invalid)
    double f;
    int cx = fine_cell(I, 0, v.x[k], f);
    int cy = fine_cell(I, 1, v.y[k], f);
    int cz = fine_cell(I, 2, v.z[k], f);
    int64_t key = I.cell_base + ((int64_t)cx * I.nf[1] + cy) * I.nf[2] + cz;
    keys_by_gid[v.gid[k]] = (uint32_t)key;
    atomicAdd(&cell_count[key], 1);
}

static __global__ void k_make_src(int64_t n, const int32_t* sorted_gid, const int32_t* pos_of_gid,
                           int32_t* src) {
    int64_t k = gtid();
    if (k >= n) return;
    src[k] = pos_of_gid[sorted_gid[k]];
}

// Gather of all carried columns into sorted order.
struct GatherCols {
    const double* din[4];
    double* dout[4];
    const void* rin[24];
    void* rout[24];
    int nr;
    const uint8_t* b_in[2];
    uint8_t* b_out[2];
    const uint16_t* imp_in;
    uint16_t* imp_out;
    const int32_t* gid_in;
    int32_t* gid_out;
};

template <class R>
static __global__ void k_gather(int64_t n, const int32_t* src, GatherCols g) {
    int64_t k = gtid();
    if (k >= n) return;
    int64_t s = src[k];
#pragma unroll
    for (int c = 0; c < 4; c++) g.dout[c][k] = g.din[c][s];
    for (int c = 0; c < g.nr; c++) static_cast<R*>(g.rout[c])[k] = static_cast<const R*>(g.rin[c])[s];
    g.b_out[0][k] = g.b_in[0][s];
    g.b_out[1][k] = g.b_in[1][s];
    g.imp_out[k] = g.imp_in[s];
    g.gid_out[k] = g.gid_in[s];
}

// After the gather: inverse permutation, traversal-cell coordinates and FP32
// offsets from the cell origin, largest |offset| per impact.
template <class R>
static __global__ void k_post_sort(View<R> v, int32_t* pos_of_gid) {
    int64_t k = gtid();
    if (k >= v.n) return;
    pos_of_gid[v.gid[k]] = (int32_t)k;
    ImpactD& I = v.imps[v.imp[k]];
    double fx, fy, fz;
    int cx = fine_cell(I, 0, v.x[k], fx);
    int cy = fine_cell(I, 1, v.y[k], fy);
    int cz = fine_cell(I, 2, v.z[k], fz);
    float ox = (float)(fx * I.w[0]), oy = (float)(fy * I.w[1]), oz = (float)(fz * I.w[2]);
    v.pf[k] = make_float4(ox, oy, oz, (float)v.hh[k]);
    v.cpk[k] = (uint32_t)cx | ((uint32_t)cy << 11) | ((uint32_t)cz << 22);
    float om = fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz));
    impact_atomic_max_u32(&I.omax_bits, __float_as_uint(om));
}

// Per-impact sorted ranges from the cell pointer.
static __global__ void k_impact_ranges(ImpactD* imps, int nimp, const int32_t* cell_ptr) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    ImpactD& I = imps[b];
    if (!I.alive) { I.off = 0; I.n = 0; return; }
    int64_t s = cell_ptr[I.cell_base], e = cell_ptr[I.cell_base + I.ncells];
    I.off = s;
    I.n = e - s;
    // FP32 filter margin: bounds the rounding of offsets and cell-origin terms
    float om = __uint_as_float(I.omax_bits);
    float wmax = fmaxf(fmaxf(I.wf[0], I.wf[1]), I.wf[2]);
    I.margin = 1.0e-5f * (om + wmax) + 8.0e-5f * I.hcap + 1.0e-30f;
}

// Phase flags: 0 = clear reductions for masked impacts.
static __global__ void k_impact_begin_round(ImpactD* imps, int nimp, int set_active) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    ImpactD& I = imps[b];
    if (set_active) {
        I.active = I.mask;
        if (set_active == 2 && I.mask) I.rounds = 0;
    }
    if (I.mask && I.active) I.hmax_bits = 0x3bc79ca10c924223ull;  // bits of 1e-30 (> 0)
}

template <class R>
static __global__ void k_hmax(View<R> v, int which) {
    int64_t k = gtid();
    if (k >= v.n) return;
    ImpactD& I = v.imps[v.imp[k]];
    if (!(I.mask && I.active)) return;
    impact_atomic_max(which == 0 ? &I.hmax_bits : &I.hm_bits, (double)v.hh[k]);
}

// Reference grid of an impact (sph.hpp:147-157): h_max -> nc, cw.
static __global__ void k_ref_grid(ImpactD* imps, int nimp) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    ImpactD& I = imps[b];
    if (!(I.mask && I.active)) return;
    double hm = bitsd(I.hmax_bits);
    if (hm < 1e-30) hm = 1e-30;
    I.h_max = hm;
    I.hmax0 = hm;
    I.hmax_f = (float)hm;
    double rc = 2.0 * hm;
    for (int a = 0; a < 3; a++) {
        double ext = I.dhi[a] - I.dlo[a];
        if (ext <= 0) ext = rc;
        double q = __ddiv_rn(ext, rc);
        int m = q >= 2097151.0 ? 2097151 : (int)q;
        if (m < 1) m = 1;
        if (I.per[a] && m < 3) m = 1;
        I.nc[a] = m;
        I.cw[a] = __ddiv_rn(ext, (double)m);
    }
    I.hm_bits = 0x3bc79ca10c924223ull;
}

template <class R>
static __global__ void k_ref_bins(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!(I.mask && I.active)) return;
    unsigned long long b0 = (unsigned long long)ref_bin(I, 0, v.x[k]);
    unsigned long long b1 = (unsigned long long)ref_bin(I, 1, v.y[k]);
    unsigned long long b2 = (unsigned long long)ref_bin(I, 2, v.z[k]);
    v.refbin[k] = b0 | (b1 << 21) | (b2 << 42);
}

// End of an adaptive-h round (sph.hpp:203-205): keep going while max h grew > 2%.
static __global__ void k_round_check(ImpactD* imps, int nimp, int32_t* flags) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    ImpactD& I = imps[b];
    if (!(I.mask && I.active)) return;
    I.rounds++;
    double hm = bitsd(I.hm_bits);
    if (hm < 1e-30) hm = 1e-30;
    if (hm <= I.hmax0 * 1.02) {
        I.active = 0;
    } else {
        atomicOr(&flags[1], 1);
    }
}

// Neighbour-list build (FP32 filter; exact criteria applied by the consumer in
// the FP64 form, or as the criterion itself in the mixed form).
template <class R, int KIND>
static __global__ void k_list(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask || (KIND == kListDensity && !I.active)) return;
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    const unsigned long long bi = v.refbin[k];
    const bool exact = sizeof(R) == 8;
    const float m = exact ? I.margin : 0.0f;
    const float Rs = (KIND == kListDensity ? 2.0f * pi.w : pi.w + I.hmax_f) + m + (exact ? m : 0.0f);
    const float lim_d = 2.0f * pi.w + m;
    int cnt = 0;
    const int cap = v.cap;
    traverse(v, I, pi, ci, Rs, [&](int32_t j, float dxc, float dyc, float dzc) {
        float4 pj = v.pf[j];
        float dx = (pi.x - pj.x) + dxc;
        float dy = (pi.y - pj.y) + dyc;
        float dz = (pi.z - pj.z) + dzc;
        if (I.per[0]) dx -= I.Lf[0] * rintf(dx / I.Lf[0]);
        if (I.per[1]) dy -= I.Lf[1] * rintf(dy / I.Lf[1]);
        if (I.per[2]) dz -= I.Lf[2] * rintf(dz / I.Lf[2]);
        float r2 = dx * dx + dy * dy + dz * dz;
        float lim = KIND == kListDensity ? lim_d : (pi.w + pj.w + m);
        bool take = r2 < lim * lim;
        if (KIND == kListForce) take = take && (j != (int32_t)k) && (exact || r2 > 0.0f);
        if (take && ref_member(bi, v.refbin[j], I)) {
            if (cnt < cap) v.nbr[(int64_t)cnt * v.stride + k] = j;
            cnt++;
        }
    });
    v.nbr_cnt[k] = cnt;
    if (cnt > cap) atomicMax(&v.flags[0], cnt);
}

// Density sum and h update (sph.hpp:189-201).
template <class R>
static __global__ void k_density(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!(I.mask && I.active)) return;
    const R hi = v.hh[k];
    const R ihi = R(1) / hi;
    const int cnt = min(v.nbr_cnt[k], v.cap);
    R sum = R(0);
    if (sizeof(R) == 8) {
        const double two_h = 2.0 * (double)hi;
        for (int t = 0; t < cnt; t++) {
            int32_t j = v.nbr[(int64_t)t * v.stride + k];
            double dx, dy, dz;
            double r = sep_exact(v, I, k, j, dx, dy, dz);
            if (r < two_h) sum += v.mass[j] * kernel_W_ih<R>((R)r, ihi);
        }
    } else {
        const float4 pi = v.pf[k];
        const uint32_t ci = v.cpk[k];
        for (int t = 0; t < cnt; t++) {
            int32_t j = v.nbr[(int64_t)t * v.stride + k];
            float dx, dy, dz;
            sep_f32(I, pi, ci, v.pf[j], v.cpk[j], dx, dy, dz);
            float r = sqrtf(dx * dx + dy * dy + dz * dz);
            sum += v.mass[j] * kernel_W_ih<R>((R)r, ihi);
        }
    }
    R rho = rmax(sum, R(1e-30));
    v.rho[k] = rho;
    R h0 = I.use_h0 ? v.h0[k] : (R)I.h_init;
    R hn = rmin(R(2) * h0, rmax(R(0.5) * h0, (R)I.eta * rcbrt(v.mass[k] / rho)));
    v.hh[k] = hn;
    v.pf[k].w = (float)hn;
}

// EOS + damage pre-pass (sph.hpp:261-275) and per-particle factors reused by
// the pair loop.
template <class R>
static __global__ void k_eos(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask) return;
    const MatT<R> m = v.mats[v.mat[k]];
    const R rho = v.rho[k];
    const R u = (R)v.u[k];
    R P, cs;
    eos_P_cs(m, rho, u, P, cs);
    v.P[k] = P;
    v.cs[k] = cs;
    v.csig[k] = rsqrt_(cs * cs + (R(4) / R(3)) * m.G / rmax(rho, R(1e-30)));
    R pf = P, dsc = R(1);
    if (I.damage_on) {
        v.sigmax[k] = -P + eig_max(v.S[0][k], v.S[1][k], v.S[2][k], v.S[3][k], v.S[4][k], v.S[5][k]);
        dsc = R(1) - v.D[k];
        if (P < R(0)) pf = dsc * P;
    }
    v.Pf[k] = pf;
    v.dscale[k] = dsc;
    const R irho2 = R(1) / (rho * rho);
    v.Rart[k] = (I.eps_as > 0 && pf < R(0)) ? (R)I.eps_as * (-pf) * irho2 : R(0);
    v.pfr2[k] = pf * irho2;
    v.dsr2[k] = irho2 * dsc;
    v.vol[k] = v.mass[k] / rho;
}

template <class R>
struct Kahan {
    R s, c;
    __device__ __forceinline__ void init() { s = R(0); c = R(0); }
    __device__ __forceinline__ void add(R x) {
        R y = x - c;
        R t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ R value() const { return s; }
};
template <class R>
struct Plain {
    R s;
    __device__ __forceinline__ void init() { s = R(0); }
    __device__ __forceinline__ void add(R x) { s += x; }
    __device__ __forceinline__ R value() const { return s; }
};

// Velocity gradient -> Jaumann dS/dt and deviatoric power (sph.hpp:212-258)
// fused with the momentum / energy pair loop (sph.hpp:277-317).  Writes acc,
// the new dudt and dSdt, eps_work.
template <class R>
static __global__ void __launch_bounds__(128) k_force(View<R> v) {
    using Acc = typename std::conditional<sizeof(R) == 4, Kahan<R>, Plain<R>>::type;
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask) return;
    const R G = v.mats[v.mat[k]].G;
    const bool strength = G > R(0);
    const R alpha = (R)I.alpha, beta = (R)I.beta, eps = (R)I.eps, eps_as = (R)I.eps_as;
    const R alpha_u = (R)I.alpha_u;
    const R hi = v.hh[k], rhoi = v.rho[k], csi = v.csig[k], Pi_over = v.pfr2[k];
    const R dsri = v.dsr2[k], di = v.dscale[k], Rai = v.Rart[k];
    const R vxi = v.vx[k], vyi = v.vy[k], vzi = v.vz[k];
    const R sxx = v.S[0][k], syy = v.S[1][k], szz = v.S[2][k];
    const R sxy = v.S[3][k], sxz = v.S[4][k], syz = v.S[5][k];
    const R Pi = v.P[k], ui = (R)v.u[k];
    R L00 = 0, L01 = 0, L02 = 0, L10 = 0, L11 = 0, L12 = 0, L20 = 0, L21 = 0, L22 = 0;
    Acc ax, ay, az, du;
    ax.init(); ay.init(); az.init(); du.init();
    const int cnt = min(v.nbr_cnt[k], v.cap);
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    for (int t = 0; t < cnt; t++) {
        const int32_t j = v.nbr[(int64_t)t * v.stride + k];
        const R hj = v.hh[j];
        R rx, ry, rz, r;
        if (sizeof(R) == 8) {
            double dx, dy, dz;
            double rr = sep_exact(v, I, k, j, dx, dy, dz);
            double hsum = __dadd_rn((double)hi, (double)hj);
            if (rr >= hsum || rr == 0.0 || j == (int32_t)k) continue;
            rx = (R)dx; ry = (R)dy; rz = (R)dz; r = (R)rr;
        } else {
            float dx, dy, dz;
            sep_f32(I, pi, ci, v.pf[j], v.cpk[j], dx, dy, dz);
            rx = (R)dx; ry = (R)dy; rz = (R)dz;
            r = (R)sqrtf(dx * dx + dy * dy + dz * dz);
        }
        const R hbar = R(0.5) * (hi + hj);
        const R ihb = R(1) / hbar;
        const R ir = R(1) / r;
        const R dW = kernel_dW<R>(r, ihb);
        const R wg = dW * ir;
        const R gx = rx * wg, gy = ry * wg, gz = rz * wg;
        const R vxj = v.vx[j], vyj = v.vy[j], vzj = v.vz[j];
        const R vx = vxi - vxj, vy = vyi - vyj, vz = vzi - vzj;
        if (strength) {
            const R Vj = v.vol[j];
            const R ex = -vx * Vj, ey = -vy * Vj, ez = -vz * Vj;  // Vj (v_j - v_i)
            L00 += ex * gx; L01 += ex * gy; L02 += ex * gz;
            L10 += ey * gx; L11 += ey * gy; L12 += ey * gz;
            L20 += ez * gx; L21 += ez * gy; L22 += ez * gz;
        }
        const R rhoj = v.rho[j];
        const R dvr = vx * rx + vy * ry + vz * rz;
        R Pij = R(0);
        if (dvr < R(0)) {
            const R mu = hbar * dvr / (r * r + eps * hbar * hbar);
            const R cbar = R(0.5) * (csi + v.csig[j]);
            Pij = (-alpha * cbar * mu + beta * mu * mu) / (R(0.5) * (rhoi + rhoj));
        }
        const R mj = v.mass[j];
        const R term = Pi_over + v.pfr2[j] + Pij;
        du.add(R(0.5) * mj * term * (vx * gx + vy * gy + vz * gz));
        R mterm = term;
        if (eps_as > R(0)) {
            const R q = r * ihb;
            R poly;
            if (q < R(1)) poly = R(1) - R(1.5) * q * q + R(0.75) * q * q * q;
            else if (q < R(2)) { R tt = R(2) - q; poly = R(0.25) * tt * tt * tt; }
            else poly = R(0);
            R fr = poly * (R)I.inv_poly_eta;
            R fn = fr * fr;
            fn *= fn;
            mterm += (Rai + v.Rart[j]) * fn;
        }
        const R mm = mj * mterm;
        const R tjxx = v.S[0][j], tjyy = v.S[1][j], tjzz = v.S[2][j];
        const R tjxy = v.S[3][j], tjxz = v.S[4][j], tjyz = v.S[5][j];
        const R ci_ = dsri, cj_ = v.dsr2[j];
        const R stx = (sxx * gx + sxy * gy + sxz * gz) * ci_ + (tjxx * gx + tjxy * gy + tjxz * gz) * cj_;
        const R sty = (sxy * gx + syy * gy + syz * gz) * ci_ + (tjxy * gx + tjyy * gy + tjyz * gz) * cj_;
        const R stz = (sxz * gx + syz * gy + szz * gz) * ci_ + (tjxz * gx + tjyz * gy + tjzz * gz) * cj_;
        ax.add(stx * mj - gx * mm);
        ay.add(sty * mj - gy * mm);
        az.add(stz * mj - gz * mm);
        if (alpha_u > R(0)) {
            const R rbar = R(0.5) * (rhoi + rhoj);
            const R vsig = rsqrt_(rabs(Pi - v.P[j]) / rbar);
            du.add(alpha_u * mj * vsig * (ui - (R)v.u[j]) * dW / rbar);
        }
    }
    R epsw = R(0);
    if (strength) {
        const R exx = L00, eyy = L11, ezz = L22;
        const R exy = R(0.5) * (L01 + L10), exz = R(0.5) * (L02 + L20), eyz = R(0.5) * (L12 + L21);
        const R Rxy = R(0.5) * (L01 - L10), Rxz = R(0.5) * (L02 - L20), Ryz = R(0.5) * (L12 - L21);
        const R tr = (exx + eyy + ezz) / R(3);
        // Jaumann J = R S - S R with R = [[0,Rxy,Rxz],[-Rxy,0,Ryz],[-Rxz,-Ryz,0]]
        const R J00 = R(2) * (Rxy * sxy + Rxz * sxz);
        const R J11 = R(2) * (-Rxy * sxy + Ryz * syz);
        const R J22 = R(2) * (-Rxz * sxz - Ryz * syz);
        const R J01 = Rxy * syy + Rxz * syz - sxx * Rxy + sxz * Ryz;
        const R J02 = Rxy * syz + Rxz * szz - sxx * Rxz - sxy * Ryz;
        const R J12 = -Rxy * sxz + Ryz * szz - sxy * Rxz - syy * Ryz;
        const R twoG = R(2) * G;
        v.dS_new[0][k] = twoG * (exx - tr) + J00;
        v.dS_new[1][k] = twoG * (eyy - tr) + J11;
        v.dS_new[2][k] = twoG * (ezz - tr) + J22;
        v.dS_new[3][k] = twoG * exy + J01;
        v.dS_new[4][k] = twoG * exz + J02;
        v.dS_new[5][k] = twoG * eyz + J12;
        epsw = (sxx * exx + syy * eyy + szz * ezz + R(2) * (sxy * exy + sxz * exz + syz * eyz)) / rhoi;
    } else {
#pragma unroll
        for (int c = 0; c < 6; c++) v.dS_new[c][k] = R(0);
    }
    v.epsw[k] = epsw;
    v.ax[k] = ax.value();
    v.ay[k] = ay.value();
    v.az[k] = az.value();
    v.dudt_new[k] = du.value() + epsw * di;
}

// Crack growth (sph.hpp:336-348); multi-flaw extension by gid.
template <class R>
static __global__ void k_damage(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask || !I.damage_on) return;
    const MatT<R>& m = v.mats[v.mat[k]];
    const R D = v.D[k];
    if (m.Emod <= R(0) || D >= R(1)) return;
    const R sig = v.sigmax[k];
    const R eps_local = sig / m.Emod;
    if (!(sig > R(0) && eps_local > v.eps_act[k])) return;
    const R cg = R(0.4) * rsqrt_(m.Emod / rmax(v.rho[k], R(1e-30)));
    const R h0 = I.use_h0 ? v.h0[k] : (R)I.h_init;
    const R Rs = R(0.5) * h0 / (R)I.eta;
    const R dt = (R)I.dt;
    if (!I.multi_flaw) {
        R d13 = rcbrt(D) + (cg / Rs) * dt;
        v.D[k] = rmin(R(1), d13 * d13 * d13);
    } else {
        int64_t g = v.gid[k];
        int64_t b = v.flaw_ptr[g], e = v.flaw_ptr[g + 1];
        if (e <= b) return;
        int64_t nact = 0;
        for (int64_t q = b; q < e; q++)
            if (eps_local > v.flaw_eps[q]) nact++;
        R d13 = rcbrt(D) + rcbrt((R)nact) * (cg / Rs) * dt;
        R Dn = rmin((R)nact / (R)(e - b), d13 * d13 * d13);
        if (Dn > D) v.D[k] = Dn;
    }
}

// Second kick, trapezoidal u and S, u floor, yield (sph.hpp:365-376); the new
// derivatives become the carried ones for the next step's trapezoid.
template <class R>
static __global__ void k_finish(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask) return;
    const R dn = v.dudt_new[k];
    R dsn[6];
#pragma unroll
    for (int c = 0; c < 6; c++) dsn[c] = v.dS_new[c][k];
    if (!v.fixed[k]) {
        const double dt = I.dt;
        const R hd = (R)(0.5 * dt);
        v.vx[k] += v.ax[k] * hd;
        v.vy[k] += v.ay[k] * hd;
        v.vz[k] += v.az[k] * hd;
        double u = v.u[k] + (0.5 * dt) * ((double)v.dudt[k] + (double)dn);
        if (u < 1e-12) u = 1e-12;
        v.u[k] = u;
        R s[6];
#pragma unroll
        for (int c = 0; c < 6; c++) s[c] = v.S[c][k] + hd * (v.dS[c][k] + dsn[c]);
        const MatT<R>& m = v.mats[v.mat[k]];
        const R Y = yield_stress(m, v.P[k], v.D[k]);
        if (Y <= R(0)) {
#pragma unroll
            for (int c = 0; c < 6; c++) s[c] = R(0);
        } else {
            R J2 = R(0.5) * (s[0] * s[0] + s[1] * s[1] + s[2] * s[2]) + (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
            R vm = rsqrt_(R(3) * J2);
            if (vm > Y) {
                R f = Y / vm;
#pragma unroll
                for (int c = 0; c < 6; c++) s[c] *= f;
            }
        }
#pragma unroll
        for (int c = 0; c < 6; c++) v.S[c][k] = s[c];
    }
    v.dudt[k] = dn;
#pragma unroll
    for (int c = 0; c < 6; c++) v.dS[c][k] = dsn[c];
}

// Adopt freshly computed derivatives without integrating (end of init).
template <class R>
static __global__ void k_adopt_derivatives(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask) return;
    v.dudt[k] = v.dudt_new[k];
#pragma unroll
    for (int c = 0; c < 6; c++) v.dS[c][k] = v.dS_new[c][k];
}

static __global__ void k_dt_begin(ImpactD* imps, int nimp) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    if (imps[b].mask) imps[b].dt_bits = 0x7ff0000000000000ull;  // +inf
}

// CFL step (sph.hpp:350-355): per-impact min of cfl h / (csig (1 + alpha) + 1e-30).
template <class R>
static __global__ void k_dt(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask) return;
    double d = I.cfl * (double)v.hh[k] / ((double)v.csig[k] * (1.0 + I.alpha) + 1e-30);
    impact_atomic_min(&I.dt_bits, d);
}

// Device-side step control for batched runs: dt = min(CFL dt, t_end - t);
// impacts at t_end drop out of the mask.
static __global__ void k_run_control(ImpactD* imps, int nimp, int phase) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    ImpactD& I = imps[b];
    if (!I.alive) { I.mask = 0; return; }
    if (phase == 0) {  // before a step
        if (I.t_end > 0 && I.t >= I.t_end) { I.mask = 0; return; }
        double dt = bitsd(I.dt_bits);
        if (I.t_end > 0 && I.t + dt > I.t_end) dt = I.t_end - I.t;
        I.dt = dt;
    } else {  // after a step
        if (I.mask) {
            I.t += I.dt;
            I.nsteps++;
        }
    }
}

}  // namespace dsph
