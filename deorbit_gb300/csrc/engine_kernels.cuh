// engine_kernels.cuh -- the CUDA kernels of one SPH step over a batch of impacts.
//
// Data layout (HBM, structure of arrays, sorted by (impact, traversal cell,
// original id) at every step):
//   carried state      x y z u vx vy vz (FP64); acc, dudt, mass, h, D, eps_act,
//                      h0, S[6], dSdt[6] (type R); mat, fixed (u8); impact (u16); gid (i32)
//   derived per step   rho P cs csig Pf dscale Rart sigmax eps_work,
//                      Pf/rho^2, dscale/rho^2, m/rho, new dudt, new dSdt[6]
//   geometry           pf = float4(offset from own traversal-cell origin, h),
//                      cpk = packed traversal-cell coordinates,
//                      refbin = packed reference-grid bins (sph.hpp:142-146)
//   neighbour lists    4-entry blocks, entry-major: entries 4b..4b+3 of particle k are
//                      the int4 at nbr[(b * ls + k) * 4] (ls = particle capacity)
//
// Reference semantics kept exactly: the neighbour criteria r < 2 h_i (density,
// self included, sph.hpp:193) and j != i, r < 2 hbar, r != 0 (sph.hpp:222,287),
// restricted to the 27-cell stencil of the reference grid of width
// ext / floor(ext / 2 h_max) (sph.hpp:147-182).  The traversal itself runs on a
// finer grid of width ~h_init and visits, per target, only the cell columns
// that intersect its search sphere.
#pragma once

#include <climits>
#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "dsph_math.cuh"

namespace dsph {

constexpr uint32_t kInvalidKey = 0xffffffffu;
constexpr int kListDensity = 0;
constexpr int kListForce = 1;
constexpr int kListSuperset = 2;
constexpr int kExtraCap = 32;   // reverse-pair entries per particle
constexpr int kMaxLevels = 4;   // traversal-grid levels of an impact (graded lattices)

// Per-impact parameters and per-step scalars, resident on the device.
struct ImpactD {
    double eta, h_init, alpha, beta, eps, alpha_u, cfl, eps_as;
    int32_t damage_on, multi_flaw, use_h0, mask;   // mask: takes part in this phase
    double dlo[3], dhi[3];
    int32_t per[3], active;                        // active: density round still running
    // traversal grid (fixed while the impact is resident)
    double glo[3], w[3], iw[3];
    float wf[3], Lf[3], iwf[3];
    int32_t nf[3], alive;
    int64_t cell_base, ncells;
    // reference grid of the last build (sph.hpp:147-157)
    int32_t nc[3], rounds;
    double cw[3], icw[3];                          // cell widths and their reciprocals
    int32_t bins_ok, pad2;                         // refbin matches this grid and the positions
    double h_max, hmax0;
    float hmax_f, margin;
    double inv_poly_eta;                           // 1 / W-polynomial at q = 1/eta
    float inv_poly_eta_f;                          // the same in FP32 (no conversion in pair loops)
    float lmargin;                                 // list-frame rounding bound on r (list radii)
    float hcap;                                    // upper bound of h (2 max h0)
    float cwmin;                                   // smallest reference cell width (nc > 1)
    float slack;                                   // superset-list radius slack
    int32_t slack_flag;                            // some h outgrew the list slack
    // step scalars
    double dt, t, t_end;
    int64_t nsteps, max_steps;   // max_steps > 0: the impact stops after that many steps
    int64_t off, n;                                // sorted particle range
    int64_t gid_base;
    unsigned long long hmax_bits, hm_bits, dt_bits;
    unsigned int omax_bits, pad1;                  // max |offset from the cell origin|
    // Traversal-grid levels (graded lattices; nlev = 1 otherwise): level L holds
    // the particles with lev_h0[L] <= h0 < lev_h0[L + 1]; its cells are 2^L base
    // cells wide on every axis and cover the box lev_lo .. lev_lo + lev_nf - 1
    // (in level cells); its cell ids start at cell_base + lev_base[L].  Particles
    // keep base-grid coordinates of their cell's origin, so pair separations
    // are formed exactly as on one grid.
    int32_t nlev, lev_esc;                         // lev_esc bit L: level L had clamped particles
    unsigned int lev_esc_next, pad3;               // gathered by the key pass for the next traversals
    float lev_h0[kMaxLevels];
    int32_t lev_lo[kMaxLevels][3], lev_nf[kMaxLevels][3];
    int64_t lev_base[kMaxLevels];
};

template <class R>
struct View {
    int64_t n;          // resident particles
    int32_t cap;        // neighbour list capacity per particle
    int32_t pad;
    double *x, *y, *z, *u, *vx, *vy, *vz;
    R *ax, *ay, *az, *dudt, *mass, *hh, *D, *eps_act, *h0;
    R* S[6];
    R* dS[6];
    uint8_t *mat, *fixed;
    uint16_t* imp;
    int32_t* gid;
    R *rho, *P, *cs, *csig, *Pf, *dscale, *Rart, *sigmax, *epsw, *pfr2, *dsr2, *vol, *dudt_new;
    R* rho_lo;          // mixed form: low part of the compensated density sum (0 in FP64)
    R* dS_new[6];
    float4* pf;
    float2* pk;          // mixed form: (mass, packed cell) per particle, for density gathers
    float4* lf;          // list frame: FP32 coordinates relative to the traversal-grid origin,
                         // and h; the list builders' pair distances (one load per candidate)
    float4* fr;          // mixed form: 96-byte force-source record of particle k at fr[6k..6k+5]:
                         // [0] offsets + h, [1] FP32 hi part of the FP64 velocity + mass,
                         // [2] lo part + packed cell, [3] (m/rho, rho, csig, Pf/rho^2),
                         // [4] (dscale/rho^2, Rart, S4, S5), [5] (S0..S3); read as three
                         // 32-byte loads
    uint32_t* cpk;
    unsigned long long* refbin;
    const int32_t* cell_ptr;
    int32_t* nbr;       // own list, 4-entry blocks: entry t of k at nbr_slot(t, ls) + 4k
    int64_t ls;         // list stride (particle capacity): a warp reads a block of 32
                        // consecutive particles as one contiguous 512-byte run
    int32_t* nbr_cnt;
    float* hlist;       // h of each particle when its list was built
    int32_t* xnbr;      // extra (reverse) list, entry-major [t * ls + k], t < kExtraCap
    int32_t* xcnt;
    int32_t* flags;     // [0] list overflow max, [1] any impact still in a density round
    ImpactD* imps;
    const MatT<R>* mats;
    const int64_t* flaw_beg;   // by gid: first / past-last threshold in flaw_eps (multi-flaw extension)
    const int64_t* flaw_end;
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

// Per-impact atomic max on the bit pattern of a non-negative double (bit order
// equals value order there).  A full warp whose lanes all target the same
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

// Block-wide combine before a per-impact atomic on ordered bits: when every
// thread of the block targets the same address, the block's extreme leaves as
// one atomic (a kernel-wide reduction then issues one atomic per block, not per
// warp); otherwise each thread with a value issues its own.  Every thread of
// the block must call it.
template <bool MAX, class U>
__device__ __forceinline__ void block_atomic_ext(U* addr, U b, bool has) {
    __shared__ U part[32];
    __shared__ U* first;
    const U none = MAX ? U(0) : ~U(0);
    if (!has) b = none;
    if (threadIdx.x == 0) first = addr;
    __syncthreads();
    const bool same = __syncthreads_and(addr == first);
    if (!same) {
        if (has) { if (MAX) atomicMax(addr, b); else atomicMin(addr, b); }
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        const U x = __shfl_xor_sync(0xffffffffu, b, o);
        b = MAX ? (x > b ? x : b) : (x < b ? x : b);
    }
    if (lane == 0) part[warp] = b;
    __syncthreads();
    if (warp == 0) {
        b = lane < (int)((blockDim.x + 31) >> 5) ? part[lane] : none;
        for (int o = 16; o > 0; o >>= 1) {
            const U x = __shfl_xor_sync(0xffffffffu, b, o);
            b = MAX ? (x > b ? x : b) : (x < b ? x : b);
        }
        if (lane == 0 && b != none) { if (MAX) atomicMax(addr, b); else atomicMin(addr, b); }
    }
}

__device__ __forceinline__ int sat_int(double q) {
    if (q != q) return 0;
    if (q >= 2147483647.0) return 2147483647;
    if (q <= -2147483648.0) return (-2147483647 - 1);
    return (int)q;
}

// Reference-grid bin of one coordinate (sph.hpp:142-146), exact FP64: the
// truncation of the IEEE quotient (c - lo) / cw.  The quotient is formed with
// the reciprocal (one multiply instead of a division, which is slow in FP64);
// it is within 2 ulp of the IEEE quotient, so the truncations agree unless an
// integer lies within a few ulp of it -- then the division decides.
//
// Cheaper still: the quotient in FP32 is within 4e-7 |q| of the exact one, so
// when it lies farther than 1e-6 (|q| + 1) from every integer its truncation is
// the exact bin; only the rest take the FP64 route.
__device__ __forceinline__ int ref_bin(const ImpactD& I, int a, double c) {
    const double d = __dsub_rn(c, I.dlo[a]);
    int i;
    const float qf = (float)d * (float)I.icw[a];
    if (fabsf(qf) < 1.0e6f && fabsf(qf - rintf(qf)) > 1.0e-6f * (fabsf(qf) + 1.0f)) {
        i = (int)qf;
    } else {
        double q = __dmul_rn(d, I.icw[a]);
        if (fabs(q - rint(q)) <= fabs(q) * 0x1p-49 + 0x1p-1000) q = __ddiv_rn(d, I.cw[a]);
        i = sat_int(q);
    }
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
// FP32 offset" representation), minimum image on periodic axes.  PER false:
// the caller knows that no resident impact has a periodic axis.
template <bool PER = true>
__device__ __forceinline__ void sep_f32(const ImpactD& I, float4 pi, uint32_t ci, float4 pj,
                                        uint32_t cj, float& dx, float& dy, float& dz) {
    int ix, iy, iz, jx, jy, jz;
    unpack_cell(ci, ix, iy, iz);
    unpack_cell(cj, jx, jy, jz);
    dx = (pi.x - pj.x) + (float)(ix - jx) * I.wf[0];
    dy = (pi.y - pj.y) + (float)(iy - jy) * I.wf[1];
    dz = (pi.z - pj.z) + (float)(iz - jz) * I.wf[2];
    if constexpr (PER) {
        if (I.per[0]) dx -= I.Lf[0] * rintf(dx / I.Lf[0]);
        if (I.per[1]) dy -= I.Lf[1] * rintf(dy / I.Lf[1]);
        if (I.per[2]) dz -= I.Lf[2] * rintf(dz / I.Lf[2]);
    }
}

// Exact FP64 separation and distance in the reference's operation order
// (sph.hpp:130-136 and vec3.hpp norm): no contraction, IEEE divide and sqrt.
template <bool PER = true, class R>
__device__ __forceinline__ double sep_exact(const View<R>& v, const ImpactD& I, int64_t i, int64_t j,
                                            double& dx, double& dy, double& dz) {
    dx = __dsub_rn(v.x[i], v.x[j]);
    dy = __dsub_rn(v.y[i], v.y[j]);
    dz = __dsub_rn(v.z[i], v.z[j]);
    if constexpr (PER) {
        if (I.per[0]) { double L = __dsub_rn(I.dhi[0], I.dlo[0]); dx = __dsub_rn(dx, __dmul_rn(L, round(__ddiv_rn(dx, L)))); }
        if (I.per[1]) { double L = __dsub_rn(I.dhi[1], I.dlo[1]); dy = __dsub_rn(dy, __dmul_rn(L, round(__ddiv_rn(dy, L)))); }
        if (I.per[2]) { double L = __dsub_rn(I.dhi[2], I.dlo[2]); dz = __dsub_rn(dz, __dmul_rn(L, round(__ddiv_rn(dz, L)))); }
    }
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

// traverse_sphere() on the levels of a graded impact (non-periodic): for every
// level, the cell columns of its box that meet the sphere of radius Rs and, per
// column, the level cells of the sphere's chord.  Ranges are formed in base
// cells relative to the particle's own cell (as on one grid) and shifted to the
// level, widened by 1e-5 base cells: a range may gain a cell, never lose one.
// A level none of whose particles was clamped into its box is skipped when the
// sphere's range misses the box; box border columns are never pruned, so
// clamped particles are met as on one grid.  f(j, dxc, dyc, dzc) as in
// traverse(), with the cell-origin differences in base cells.
template <class R, class F>
__device__ __forceinline__ void traverse_levels(const View<R>& v, const ImpactD& I, float4 pi, uint32_t ci,
                                             float Rs, F&& f) {
    constexpr float kWiden = 1.0e-5f;
    int c[3];
    unpack_cell(ci, c[0], c[1], c[2]);
    const float o[3] = {pi.x, pi.y, pi.z};
    int blo[3], bhi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        blo[a] = c[a] + (int)floorf((o[a] - Rs) * I.iwf[a] - kWiden);
        bhi[a] = c[a] + (int)floorf((o[a] + Rs) * I.iwf[a] + kWiden);
    }
    const float R2 = Rs * Rs;
    const float w0 = I.wf[0], w1 = I.wf[1], w2 = I.wf[2];
    for (int L = 0; L < I.nlev; L++) {
        const int lo0 = I.lev_lo[L][0], lo1 = I.lev_lo[L][1], lo2 = I.lev_lo[L][2];
        const int e0 = lo0 + I.lev_nf[L][0] - 1, e1 = lo1 + I.lev_nf[L][1] - 1, e2 = lo2 + I.lev_nf[L][2] - 1;
        int l0 = blo[0] >> L, h0 = bhi[0] >> L, l1 = blo[1] >> L, h1 = bhi[1] >> L;
        const int l2 = blo[2] >> L, h2 = bhi[2] >> L;
        if (!((I.lev_esc >> L) & 1) &&
            (h0 < lo0 || l0 > e0 || h1 < lo1 || l1 > e1 || h2 < lo2 || l2 > e2))
            continue;  // no particle of this level can be within Rs
        l0 = l0 < lo0 ? lo0 : (l0 > e0 ? e0 : l0);
        h0 = h0 < lo0 ? lo0 : (h0 > e0 ? e0 : h0);
        l1 = l1 < lo1 ? lo1 : (l1 > e1 ? e1 : l1);
        h1 = h1 < lo1 ? lo1 : (h1 > e1 ? e1 : h1);
        const float wl0 = w0 * (float)(1 << L), wl1 = w1 * (float)(1 << L);
        const int n1 = I.lev_nf[L][1], n2 = I.lev_nf[L][2];
        const int64_t lbase = I.cell_base + I.lev_base[L] - lo2;
        for (int ix = l0; ix <= h0; ix++) {
            const float xa = (float)((ix << L) - c[0]) * w0 - o[0];  // column x-interval [xa, xa + wl0) rel. to i
            float bx = xa > 0.0f ? xa : (xa + wl0 < 0.0f ? -(xa + wl0) : 0.0f);
            if (ix == lo0 || ix == e0) bx = 0.0f;
            const float dxc = (float)(c[0] - (ix << L)) * w0;
            for (int iy = l1; iy <= h1; iy++) {
                const float ya = (float)((iy << L) - c[1]) * w1 - o[1];
                float by = ya > 0.0f ? ya : (ya + wl1 < 0.0f ? -(ya + wl1) : 0.0f);
                if (iy == lo1 || iy == e1) by = 0.0f;
                const float d2 = bx * bx + by * by;
                if (d2 >= R2) continue;
                const float hz = sqrtf(R2 - d2);
                int zl = (c[2] + (int)floorf((o[2] - hz) * I.iwf[2] - kWiden)) >> L;
                int zh = (c[2] + (int)floorf((o[2] + hz) * I.iwf[2] + kWiden)) >> L;
                zl = zl < lo2 ? lo2 : (zl > e2 ? e2 : zl);
                zh = zh < lo2 ? lo2 : (zh > e2 ? e2 : zh);
                const float dyc = (float)(c[1] - (iy << L)) * w1;
                const int64_t colbase = lbase + ((int64_t)(ix - lo0) * n1 + (iy - lo1)) * n2;
                int cz = zl;
                const int32_t s0 = v.cell_ptr[colbase + zl];
                const int32_t e = v.cell_ptr[colbase + zh + 1];
                int32_t next = v.cell_ptr[colbase + cz + 1];
                float dzc = (float)(c[2] - (cz << L)) * w2;
                for (int32_t j = s0; j < e; j++) {
                    while (j >= next) {
                        cz++;
                        next = v.cell_ptr[colbase + cz + 1];
                        dzc = (float)(c[2] - (cz << L)) * w2;
                    }
                    f(j, dxc, dyc, dzc);
                }
            }
        }
    }
}

// Visit every traversal cell column that intersects the sphere of radius Rs
// around particle k (sorted index), cell by cell; calls f(j, dxc, dyc, dzc)
// where d?c are the FP32 cell-origin differences (i's cell minus j's cell).
// LV: the kernel also serves impacts with traversal-grid levels (instantiated
// only where a resident impact has them, so that the one-grid kernels keep
// their register allocation).
template <class R, bool LV = false, class F>
__device__ __forceinline__ void traverse(const View<R>& v, const ImpactD& I, float4 pi,
                                         uint32_t ci, float Rs, F&& f) {
    if constexpr (LV) {
        if (I.nlev > 1) {  // graded impacts (never periodic)
            traverse_levels(v, I, pi, ci, Rs, f);
            return;
        }
    }
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

// Like traverse(), but visits only the cell columns whose footprint meets the
// sphere and, per column, only the z-cells within the sphere's chord there
// (non-periodic impacts; periodic ones use the full box).  Border columns are
// never pruned by x / y because clamped particles may lie outside their cell.
template <class R, bool LV = false, bool PER = true, class F>
__device__ __forceinline__ void traverse_sphere(const View<R>& v, const ImpactD& I, float4 pi,
                                                uint32_t ci, float Rs, F&& f) {
    if constexpr (PER) {
        if (I.per[0] | I.per[1] | I.per[2]) {
            traverse(v, I, pi, ci, Rs, f);
            return;
        }
    }
    if constexpr (LV) {
        if (I.nlev > 1) {
            traverse_levels(v, I, pi, ci, Rs, f);
            return;
        }
    }
    int c[3];
    unpack_cell(ci, c[0], c[1], c[2]);
    const float o[3] = {pi.x, pi.y, pi.z};
    int lo[2], hi[2];
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const float w = I.wf[a];
        const int nf = I.nf[a];
        int l = c[a] + (int)floorf((o[a] - Rs) / w);
        int h = c[a] + (int)floorf((o[a] + Rs) / w);
        lo[a] = l < 0 ? 0 : (l > nf - 1 ? nf - 1 : l);
        hi[a] = h < 0 ? 0 : (h > nf - 1 ? nf - 1 : h);
    }
    const float R2 = Rs * Rs;
    const float w0 = I.wf[0], w1 = I.wf[1], w2 = I.wf[2];
    const int nf2 = I.nf[2];
    for (int ix = lo[0]; ix <= hi[0]; ix++) {
        const float xa = (float)(ix - c[0]) * w0 - o[0];   // column x-interval [xa, xa + w0) rel. to i
        float bx = xa > 0.0f ? xa : (xa + w0 < 0.0f ? -(xa + w0) : 0.0f);
        if (ix == 0 || ix == I.nf[0] - 1) bx = 0.0f;
        const float dxc = (float)(c[0] - ix) * w0;
        for (int iy = lo[1]; iy <= hi[1]; iy++) {
            const float ya = (float)(iy - c[1]) * w1 - o[1];
            float by = ya > 0.0f ? ya : (ya + w1 < 0.0f ? -(ya + w1) : 0.0f);
            if (iy == 0 || iy == I.nf[1] - 1) by = 0.0f;
            const float d2 = bx * bx + by * by;
            if (d2 >= R2) continue;
            const float hz = sqrtf(R2 - d2);
            int zl = c[2] + (int)floorf((o[2] - hz) / w2);
            int zh = c[2] + (int)floorf((o[2] + hz) / w2);
            zl = zl < 0 ? 0 : (zl > nf2 - 1 ? nf2 - 1 : zl);
            zh = zh < 0 ? 0 : (zh > nf2 - 1 ? nf2 - 1 : zh);
            const float dyc = (float)(c[1] - iy) * w1;
            const int64_t colbase = I.cell_base + ((int64_t)ix * I.nf[1] + iy) * nf2;
            int cz = zl;
            const int32_t s = v.cell_ptr[colbase + zl];
            const int32_t e = v.cell_ptr[colbase + zh + 1];
            int32_t next = v.cell_ptr[colbase + cz + 1];
            float dzc = (float)(c[2] - cz) * w2;
            for (int32_t j = s; j < e; j++) {
                while (j >= next) {
                    cz++;
                    next = v.cell_ptr[colbase + cz + 1];
                    dzc = (float)(c[2] - cz) * w2;
                }
                f(j, dxc, dyc, dzc);
            }
        }
    }
}

// One 32-byte load (two float4 halves) of a 32-byte-aligned record that no
// thread of the kernel writes: sm_100-class GPUs load 256 bits per thread in one
// instruction, here through the read-only path.
__device__ __forceinline__ void ld_f32x8_ro(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// ---- bulk-copy staging (cp.async.bulk through the TMA engine, mbarrier completion)
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes initialised barriers visible to the bulk-copy (async) proxy
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}
// this thread's arrival on the barrier's current phase, announcing `bytes` of
// bulk copies that will complete on it
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the barrier phase of the given parity, at most `limit` polls
// (each poll may suspend the thread for a bounded, hardware-chosen time);
// false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit) {
    for (int i = 0; i < limit; i++)
        if (mbar_test(bar, parity)) return true;
    return false;
}
// global -> shared bulk copy of `bytes` (multiple of 16, both addresses 16-byte
// aligned), completing as transaction bytes on the barrier
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// global -> shared 16-byte asynchronous copy through L1 (cp.async.ca), and the
// arrival on a barrier once every cp.async this thread issued before it has
// landed (the barrier's expected count includes this arrival)
__device__ __forceinline__ void async16_g2s(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void async_arrive(uint64_t* bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Own-list addressing: entry t of particle k lives at nbr[4k + nbr_slot(t, ls)],
// i.e. 4-entry blocks stored block-major, so one int4 load brings a lane four
// entries and a warp's block loads are contiguous.
__device__ __forceinline__ int64_t nbr_slot(int t, int64_t ls) {
    return (((int64_t)(t >> 2) * ls) << 2) + (t & 3);
}

// f(j) for entries 0..cnt-1 of particle k's own list, in list order.
// The next index block is loaded one block ahead, so its (usually uncached)
// read overlaps the current block's entries.
template <class F>
__device__ __forceinline__ void walk_list(const int32_t* nbr, int64_t ls, int64_t k, int cnt, F&& f) {
    const int4* p = reinterpret_cast<const int4*>(nbr) + k;
    int4 q = cnt > 0 ? *p : make_int4(0, 0, 0, 0);
    for (int t = 0; t < cnt; t += 4) {
        p += ls;
        const int4 qn = t + 4 < cnt ? *p : q;
        const int m = min(4, cnt - t);
#pragma unroll 1
        for (int i = 0; i < m; i++) f(i == 0 ? q.x : i == 1 ? q.y : i == 2 ? q.z : q.w);
        q = qn;
    }
}

// walk_list with the entries handed over two at a time where a block allows
// (f2(j0, j1) must apply them in that order; f1 takes a lone entry).
template <class F1, class F2>
__device__ __forceinline__ void walk_list_pairs(const int32_t* nbr, int64_t ls, int64_t k, int cnt, F1&& f1,
                                                F2&& f2) {
    const int4* p = reinterpret_cast<const int4*>(nbr) + k;
    int4 q = cnt > 0 ? *p : make_int4(0, 0, 0, 0);
    for (int t = 0; t < cnt; t += 4) {
        p += ls;
        const int4 qn = t + 4 < cnt ? *p : q;
        const int m = min(4, cnt - t);
        if (m >= 2) f2(q.x, q.y); else f1(q.x);
        if (m == 4) f2(q.z, q.w); else if (m == 3) f1(q.z);
        q = qn;
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
    const double hd = 0.5 * dt;
    // all loads before the stores (the columns may alias as far as the compiler knows)
    const double x = v.x[k], y = v.y[k], z = v.z[k];
    const double vx = v.vx[k] + (double)v.ax[k] * hd;
    const double vy = v.vy[k] + (double)v.ay[k] * hd;
    const double vz = v.vz[k] + (double)v.az[k] * hd;
    v.vx[k] = vx;
    v.vy[k] = vy;
    v.vz[k] = vz;
    v.x[k] = x + vx * dt;
    v.y[k] = y + vy * dt;
    v.z[k] = z + vz * dt;
}

// Traversal cell along axis a and the FP32 offset from its origin.  The cell
// may be chosen from the FP32 quotient (any cell works as long as the offset is
// taken from that cell's origin); the offset itself is one FP64 fused
// multiply-add, rounded once to FP32.
__device__ __forceinline__ int fine_cell(const ImpactD& I, int a, double c, float& off) {
    const double d = c - I.glo[a];
    const float qf = (float)d * I.iwf[a];
    int i = qf >= 2147483520.0f ? 2147483647 : (qf == qf ? (int)floorf(qf) : 0);
    if (i < 0) i = 0;
    if (i >= I.nf[a]) i = I.nf[a] - 1;
    off = (float)fma(-(double)i, I.w[a], d);
    return i;
}

// One particle's key, counts, offsets and packed cell; returns the bits of its
// largest |offset| (ordered as the non-negative floats).
template <class R>
__device__ __forceinline__ unsigned int fine_keys_one(const View<R>& v, const ImpactD& I, int64_t k,
                                                      uint32_t* keys_by_gid, int32_t* cell_count, float4* pf_out,
                                                      uint32_t* cpk_out) {
    const float h = (float)v.hh[k];  // loaded before the stores below
    const int32_t gid = v.gid[k];
    float ox, oy, oz;
    int cx, cy, cz;
    int64_t key;
    if (I.nlev <= 1) {
        cx = fine_cell(I, 0, v.x[k], ox);
        cy = fine_cell(I, 1, v.y[k], oy);
        cz = fine_cell(I, 2, v.z[k], oz);
        key = I.cell_base + ((int64_t)cx * I.nf[1] + cy) * I.nf[2] + cz;
    } else {
        // the particle's level from its reference smoothing length, its cell in
        // that level's box (clamped, noted), and the cell's origin in base cells
        const float h0 = (float)v.h0[k];
        int L = 0;
        while (L + 1 < I.nlev && h0 >= I.lev_h0[L + 1]) L++;
        const double pc[3] = {v.x[k], v.y[k], v.z[k]};
        int cb[3];
        float off[3];
        bool clamped = false;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double d = pc[a] - I.glo[a];
            const float qf = (float)d * I.iwf[a];
            int ib = qf >= 2147483520.0f ? 2147483647 : (qf == qf ? (int)floorf(qf) : 0);
            if (ib < 0) { ib = 0; clamped = true; }
            if (ib >= I.nf[a]) { ib = I.nf[a] - 1; clamped = true; }
            int il = ib >> L;
            const int lo = I.lev_lo[L][a], hi = lo + I.lev_nf[L][a] - 1;
            if (il < lo) { il = lo; clamped = true; }
            if (il > hi) { il = hi; clamped = true; }
            cb[a] = il << L;
            off[a] = (float)fma(-(double)cb[a], I.w[a], d);
        }
        if (clamped) atomicOr(const_cast<unsigned int*>(&I.lev_esc_next), 1u << L);
        cx = cb[0]; cy = cb[1]; cz = cb[2];
        ox = off[0]; oy = off[1]; oz = off[2];
        key = I.cell_base + I.lev_base[L] +
              ((int64_t)((cx >> L) - I.lev_lo[L][0]) * I.lev_nf[L][1] + ((cy >> L) - I.lev_lo[L][1])) *
                  I.lev_nf[L][2] +
              ((cz >> L) - I.lev_lo[L][2]);
    }
    keys_by_gid[gid] = (uint32_t)key;
    atomicAdd(&cell_count[key], 1);
    pf_out[k] = make_float4(ox, oy, oz, h);
    cpk_out[k] = (uint32_t)cx | ((uint32_t)cy << 11) | ((uint32_t)cz << 22);
    return __float_as_uint(fmaxf(fmaxf(fabsf(ox), fabsf(oy)), fabsf(oz)));
}

// Traversal-cell key of every resident particle, scattered into gid order,
// per-cell counts, and (in the current order, for the gather to carry) the
// FP32 offset from the cell origin with h, the packed cell coordinates and the
// per-impact largest |offset|.
template <class R>
static __global__ void k_fine_keys(View<R> v, uint32_t* keys_by_gid, int32_t* cell_count, float4* pf_out,
                                   uint32_t* cpk_out) {
    const int64_t k0 = gtid();
    const bool inb = k0 < v.n;
    const int64_t k = inb ? k0 : v.n - 1;
    ImpactD& I = v.imps[v.imp[k]];
    const bool live = inb && I.alive;  // a dead impact's particles leave at this sort (key stays invalid)
    unsigned int om = 0u;
    if (live) om = fine_keys_one(v, I, k, keys_by_gid, cell_count, pf_out, cpk_out);
    block_atomic_ext<true>(&I.omax_bits, om, live);
}

static __global__ void k_make_src(int64_t n, const int32_t* sorted_gid, const int32_t* pos_of_gid,
                           int32_t* src) {
    int64_t k = gtid();
    if (k >= n) return;
    src[k] = pos_of_gid[sorted_gid[k]];
}

// Gather of all carried columns into sorted order.
struct GatherCols {
    const double* din[7];
    double* dout[7];
    const void* rin[24];
    void* rout[24];
    int nr;
    const uint8_t* b_in[2];
    uint8_t* b_out[2];
    const uint16_t* imp_in;
    uint16_t* imp_out;
    const int32_t* gid_in;
    int32_t* gid_out;
    const float4* pf_in;     // offsets + h and packed cells made by k_fine_keys
    float4* pf_out;
    const uint32_t* cpk_in;
    uint32_t* cpk_out;
    float4* lf_out;          // list frame, formed from the cell and the offset
    const ImpactD* imps;
};

template <class R>
static __global__ void k_gather(int64_t n, const int32_t* src, GatherCols g) {
    int64_t k = gtid();
    if (k >= n) return;
    int64_t s = src[k];
    // every load first, then every store: the column pointers may alias as far
    // as the compiler knows, so interleaved copies would wait for each load in turn
    double dv[7];
    R rv[24];
#pragma unroll
    for (int c = 0; c < 7; c++) dv[c] = g.din[c][s];
#pragma unroll
    for (int c = 0; c < 24; c++)
        if (c < g.nr) rv[c] = static_cast<const R*>(g.rin[c])[s];
    const uint8_t b0 = g.b_in[0][s], b1 = g.b_in[1][s];
    const uint16_t ib = g.imp_in[s];
    const int32_t gid = g.gid_in[s];
    const float4 p = g.pf_in[s];
    const uint32_t c = g.cpk_in[s];
#pragma unroll
    for (int q = 0; q < 7; q++) g.dout[q][k] = dv[q];
#pragma unroll
    for (int q = 0; q < 24; q++)
        if (q < g.nr) static_cast<R*>(g.rout[q])[k] = rv[q];
    g.b_out[0][k] = b0;
    g.b_out[1][k] = b1;
    g.imp_out[k] = ib;
    g.gid_out[k] = gid;
    g.pf_out[k] = p;
    g.cpk_out[k] = c;
    // one FP32 coordinate per particle (all its pairs use the same value):
    // |lf - (x - glo)| <= 2 roundings of a value below nf w + max |offset|
    const ImpactD& I = g.imps[ib];
    g.lf_out[k] = make_float4((float)(c & 2047u) * I.wf[0] + p.x, (float)((c >> 11) & 2047u) * I.wf[1] + p.y,
                              (float)(c >> 22) * I.wf[2] + p.z, p.w);
}

// After the gather: inverse permutation (gid -> sorted position) and, in the
// mixed form, the (mass, packed cell) records of the density gathers.
template <class R>
static __global__ void k_post_sort(View<R> v, int32_t* pos_of_gid) {
    int64_t k = gtid();
    if (k >= v.n) return;
    pos_of_gid[v.gid[k]] = (int32_t)k;
    if (sizeof(R) == 4) v.pk[k] = make_float2((float)v.mass[k], __uint_as_float(v.cpk[k]));
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
    I.lev_esc = (int32_t)I.lev_esc_next;  // the key pass of this sort
    I.lev_esc_next = 0u;
    // FP32 filter margin: bounds the rounding of offsets and cell-origin terms
    float om = __uint_as_float(I.omax_bits);
    float wmax = fmaxf(fmaxf(I.wf[0], I.wf[1]), I.wf[2]);
    I.margin = 1.0e-5f * (om + wmax) + 8.0e-5f * I.hcap + 1.0e-30f;
    // list-frame r: each coordinate within two FP32 roundings of a value below
    // c_max = max (nf w) + max |offset|, differences and r^2 rounded in FP32
    // (<= 2^-23 r): the error of r stays below 1e-6 (c_max + 4 hcap)
    const float cmax = fmaxf(fmaxf(I.wf[0] * I.nf[0], I.wf[1] * I.nf[1]), I.wf[2] * I.nf[2]) + om;
    I.lmargin = 1.0e-6f * (cmax + 4.0f * I.hcap) + 1.0e-30f;
}

// Start of an on-device list rebuild: empty the extra lists of the impacts
// whose h outgrew the slack.
template <class R>
static __global__ void k_refresh_begin(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (I.mask && I.slack_flag) v.xcnt[k] = 0;
}

// End of an on-device list rebuild: the rebuilt lists cover the new h.
static __global__ void k_impact_end_refresh(ImpactD* imps, int nimp) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nimp && imps[b].mask) imps[b].slack_flag = 0;
}

// Phase flags: 0 = clear reductions for masked impacts.
static __global__ void k_impact_reset_slack(ImpactD* imps, int nimp) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < nimp && imps[b].mask) imps[b].slack_flag = 0;
}

// set_active: 2 first round of a step, 0 a later round, 1 a grid build outside
// the rounds, 3 the grid build after the rounds.  The max h at a round's start
// (and at the build after the rounds) is the max the previous round's density
// pass reduced (h does not change in between); otherwise it is reduced anew.
static __global__ void k_impact_begin_round(ImpactD* imps, int nimp, int set_active) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nimp) return;
    ImpactD& I = imps[b];
    if (set_active) {
        I.active = I.mask;
        if (set_active == 2 && I.mask) {
            I.rounds = 0;
            I.bins_ok = 0;
        }
    }
    if (I.mask && I.active)
        I.hmax_bits = (set_active == 0 || set_active == 3) ? I.hm_bits
                                                           : 0x3bc79ca10c924223ull;  // bits of 1e-30 (> 0)
}

template <class R>
static __global__ void k_hmax(View<R> v, int which) {
    const int64_t k0 = gtid();
    const bool inb = k0 < v.n;
    const int64_t k = inb ? k0 : v.n - 1;
    ImpactD& I = v.imps[v.imp[k]];
    const bool has = inb && I.mask && I.active;
    block_atomic_ext<true>(which == 0 ? &I.hmax_bits : &I.hm_bits, dbits((double)v.hh[k]), has);
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
    bool same = I.bins_ok != 0;
    for (int a = 0; a < 3; a++) {
        double ext = I.dhi[a] - I.dlo[a];
        if (ext <= 0) ext = rc;
        double q = __ddiv_rn(ext, rc);
        int m = q >= 2097151.0 ? 2097151 : (int)q;
        if (m < 1) m = 1;
        if (I.per[a] && m < 3) m = 1;
        const double cw = __ddiv_rn(ext, (double)m);
        same = same && m == I.nc[a] && cw == I.cw[a];
        I.nc[a] = m;
        I.cw[a] = cw;
        I.icw[a] = __ddiv_rn(1.0, cw);
    }
    I.bins_ok = same ? 1 : 0;  // same grid, positions unchanged since the bins were made
    float cwm = 3.0e38f;
    for (int a = 0; a < 3; a++)
        if (I.nc[a] > 1) cwm = fminf(cwm, (float)I.cw[a]);
    I.cwmin = cwm;
    I.hm_bits = 0x3bc79ca10c924223ull;
}

template <class R>
static __global__ void k_ref_bins(View<R> v) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!(I.mask && I.active) || I.bins_ok) return;
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
    I.bins_ok = 1;  // this round's bins exist
    I.rounds++;
    double hm = bitsd(I.hm_bits);
    if (hm < 1e-30) hm = 1e-30;
    if (hm <= I.hmax0 * 1.02) {
        I.active = 0;
    } else {
        atomicOr(&flags[1], 1);
    }
}

// Pair distance^2 of the list builders on non-periodic impacts, from the list
// frame: IEEE differences are exactly antisymmetric, so both sides of a pair
// get the same r^2 bit for bit and the own / reverse tests partition the pairs
// exactly.  Periodic impacts use the cell-relative offsets (minimum image).
__device__ __forceinline__ float list_r2(float4 a, float4 b) {
    const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return dx * dx + dy * dy + dz * dz;
}

// One particle's list by its own traversal (periodic impacts, and warps that
// straddle two impacts).
template <class R, bool LV = false, bool PER = true>
__device__ __forceinline__ void list_one(const View<R>& v, const ImpactD& I, int64_t k) {
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    const float4 li = v.lf[k];
    const bool periodic = PER && (I.per[0] | I.per[1] | I.per[2]);
    const float m = (sizeof(R) == 8 ? I.margin : 0.0f) + I.lmargin;
    const float sl = 1.0f + I.slack;
    const float ri = 2.0f * pi.w * sl + m;
    const float ri2 = ri * ri;
    int cnt = 0;
    const int cap = v.cap;
    int32_t* out = v.nbr + 4 * k;  // entry t at out[nbr_slot(t, ls)]
    traverse_sphere<R, LV, PER>(v, I, pi, ci, ri + m, [&](int32_t j, float dxc, float dyc, float dzc) {
        float r2, hj;
        if (!periodic) {
            const float4 lj = v.lf[j];
            r2 = list_r2(li, lj);
            hj = lj.w;
        } else {
            const float4 pj = v.pf[j];
            float dx = (pi.x - pj.x) + dxc;
            float dy = (pi.y - pj.y) + dyc;
            float dz = (pi.z - pj.z) + dzc;
            if (I.per[0]) dx -= I.Lf[0] * rintf(dx / I.Lf[0]);
            if (I.per[1]) dy -= I.Lf[1] * rintf(dy / I.Lf[1]);
            if (I.per[2]) dz -= I.Lf[2] * rintf(dz / I.Lf[2]);
            r2 = dx * dx + dy * dy + dz * dz;
            hj = pj.w;
        }
        if (r2 < ri2) {
            if (cnt < cap) out[nbr_slot(cnt, v.ls)] = j;
            cnt++;
            // does j's own search miss k although the pair can interact?
            const float rj = 2.0f * hj * sl + m;
            const float rb = (pi.w + hj) * sl + m;
            if (!(r2 < rj * rj) && r2 < rb * rb) {
                const int slot = atomicAdd(&v.xcnt[j], 1);
                if (slot < kExtraCap) v.xnbr[(int64_t)slot * v.ls + j] = (int32_t)k;
            }
        }
    });
    v.nbr_cnt[k] = cnt;
    v.hlist[k] = pi.w;
    if (cnt > cap) atomicMax(&v.flags[0], cnt);
}

// The warp-union walk of the list build on the levels of a graded impact
// (all 32 lanes in one impact, non-periodic): level by level, the warp walks
// the union of its lanes' level-cell column boxes; each lane takes the columns
// of its own box that meet its sphere, over the level cells of its own chord,
// and run(s, len) tests the lane's candidates s .. s + len - 1 (len = 0 where
// the lane takes nothing; run reduces over the warp).  Every lane meets the
// columns and cells of traverse_levels() in its order, so the lists equal
// those of the per-thread build entry for entry.
template <class R, class Run>
__device__ __forceinline__ void warp_walk_levels(const View<R>& v, const ImpactD& I, bool act, float4 pi,
                                                 uint32_t ci, float Rs, Run&& run) {
    const unsigned full = 0xffffffffu;
    constexpr float kWiden = 1.0e-5f;
    int c[3];
    unpack_cell(ci, c[0], c[1], c[2]);
    const float o[3] = {pi.x, pi.y, pi.z};
    int blo[3], bhi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        blo[a] = c[a] + (int)floorf((o[a] - Rs) * I.iwf[a] - kWiden);
        bhi[a] = c[a] + (int)floorf((o[a] + Rs) * I.iwf[a] + kWiden);
    }
    const float R2 = Rs * Rs;
    const float w0 = I.wf[0], w1 = I.wf[1];
    const int nlev = I.nlev;
    for (int L = 0; L < nlev; L++) {
        const int lo0 = I.lev_lo[L][0], lo1 = I.lev_lo[L][1], lo2 = I.lev_lo[L][2];
        const int e0 = lo0 + I.lev_nf[L][0] - 1, e1 = lo1 + I.lev_nf[L][1] - 1, e2 = lo2 + I.lev_nf[L][2] - 1;
        int l0 = blo[0] >> L, h0 = bhi[0] >> L, l1 = blo[1] >> L, h1 = bhi[1] >> L;
        const int l2 = blo[2] >> L, h2 = bhi[2] >> L;
        const bool lane = act && (((I.lev_esc >> L) & 1) ||
                                  !(h0 < lo0 || l0 > e0 || h1 < lo1 || l1 > e1 || h2 < lo2 || l2 > e2));
        l0 = l0 < lo0 ? lo0 : (l0 > e0 ? e0 : l0);
        h0 = h0 < lo0 ? lo0 : (h0 > e0 ? e0 : h0);
        l1 = l1 < lo1 ? lo1 : (l1 > e1 ? e1 : l1);
        h1 = h1 < lo1 ? lo1 : (h1 > e1 ? e1 : h1);
        const int ul0 = __reduce_min_sync(full, lane ? l0 : INT_MAX), uh0 = __reduce_max_sync(full, lane ? h0 : INT_MIN);
        const int ul1 = __reduce_min_sync(full, lane ? l1 : INT_MAX), uh1 = __reduce_max_sync(full, lane ? h1 : INT_MIN);
        const float wl0 = w0 * (float)(1 << L), wl1 = w1 * (float)(1 << L);
        const int n1 = I.lev_nf[L][1], n2 = I.lev_nf[L][2];
        const int64_t lbase = I.cell_base + I.lev_base[L] - lo2;
        for (int ix = ul0; ix <= uh0; ix++) {  // empty when no lane meets this level
            const float xa = (float)((ix << L) - c[0]) * w0 - o[0];
            float bx = xa > 0.0f ? xa : (xa + wl0 < 0.0f ? -(xa + wl0) : 0.0f);
            if (ix == lo0 || ix == e0) bx = 0.0f;
            const bool in_x = lane && ix >= l0 && ix <= h0;
            for (int iy = ul1; iy <= uh1; iy++) {
                const float ya = (float)((iy << L) - c[1]) * w1 - o[1];
                float by = ya > 0.0f ? ya : (ya + wl1 < 0.0f ? -(ya + wl1) : 0.0f);
                if (iy == lo1 || iy == e1) by = 0.0f;
                const float d2 = bx * bx + by * by;
                int32_t s = 0, len = 0;
                if (in_x && iy >= l1 && iy <= h1 && d2 < R2) {
                    const float hz = sqrtf(R2 - d2);
                    int zl = (c[2] + (int)floorf((o[2] - hz) * I.iwf[2] - kWiden)) >> L;
                    int zh = (c[2] + (int)floorf((o[2] + hz) * I.iwf[2] + kWiden)) >> L;
                    zl = zl < lo2 ? lo2 : (zl > e2 ? e2 : zl);
                    zh = zh < lo2 ? lo2 : (zh > e2 ? e2 : zh);
                    const int64_t colbase = lbase + ((int64_t)(ix - lo0) * n1 + (iy - lo1)) * n2;
                    s = v.cell_ptr[colbase + zl];
                    len = v.cell_ptr[colbase + zh + 1] - s;
                }
                run(s, len);
            }
        }
    }
}

// Neighbour-list build, one thread per particle k.  Each particle searches only
// its own sphere of radius 2 h_k (1 + slack) and records
//   own list   every j with r < 2 h_k (1 + s)  -- a superset of the density set
//              {r < 2 h_k} and of the force pairs with h_j <= h_k;
//   extra list of j: k itself, when j's own search misses k (r >= 2 h_j (1 + s))
//              but the pair can interact (r < (h_j + h_k)(1 + s)); such a k is
//              always inside k's own sphere, so every force pair is found once.
// The FP32 pair distance comes from the list frame (list_r2) and is the same
// bit for bit from either side, so the two tests partition the pairs exactly;
// every radius carries the frame's rounding bound, and the FP64 form adds its
// margin m as well.  Extra lists are appended with atomics and sorted afterwards, so
// list contents and order depend only on the state.  Consumers apply the exact
// criteria, the reference-stencil restriction, and fall back to a traversal
// for a particle whose h outgrew the slack or whose list overflowed.
//
// Loop shape: the 32 particles of a warp are consecutive in sorted order, so
// they sit in one or two cell columns and search nearly the same columns.  The
// warp walks the union of its lanes' column boxes in a fixed order; each lane
// takes the columns of its own box that meet its sphere, over the z-range of
// its own chord, and the candidate loop runs to the longest chord of the warp
// with the other lanes predicated off; a candidate costs one 16-byte load of
// its list-frame record.  Every lane visits the same candidates in the same
// order as traverse_sphere(), so the lists equal those of a per-thread
// traversal entry for entry.
//
// refresh != 0: rebuild only the lists of impacts whose h outgrew the slack in
// this step's density rounds (the others return at once).
template <class R, bool LV = false, bool PER = true>
static __global__ void k_list_thread(View<R> v, int refresh) {
    const unsigned full = 0xffffffffu;
    const int64_t k0 = gtid();
    const bool inb = k0 < v.n;
    const int64_t k = inb ? k0 : v.n - 1;
    const int ib = v.imp[k];
    const ImpactD& I = v.imps[ib];
    const bool wanted = I.mask && (!refresh || I.slack_flag);
    const bool one_impact = __all_sync(full, ib == __shfl_sync(full, ib, 0));
    if (!one_impact || (PER && (I.per[0] | I.per[1] | I.per[2]))) {
        if (inb && wanted) list_one<R, LV, PER>(v, I, k);
        return;
    }
    if (!wanted) return;  // warp-uniform: one impact
    const bool act = inb;
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    const float4 li = v.lf[k];
    const float m = (sizeof(R) == 8 ? I.margin : 0.0f) + I.lmargin;
    const float sl = 1.0f + I.slack;
    const float ri = 2.0f * pi.w * sl + m;
    const float ri2 = ri * ri;
    const float Rs = ri + m;
    const float R2 = Rs * Rs;
    int cnt = 0;
    const int cap = v.cap;
    int32_t* out = v.nbr + 4 * k;  // entry t at out[nbr_slot(t, ls)]
    auto take = [&](int32_t j, float4 lj, float r2) {
        if (cnt < cap) out[nbr_slot(cnt, v.ls)] = j;
        cnt++;
        const float rj = 2.0f * lj.w * sl + m;
        const float rb = (pi.w + lj.w) * sl + m;
        if (!(r2 < rj * rj) && r2 < rb * rb) {
            const int slot = atomicAdd(&v.xcnt[j], 1);
            if (slot < kExtraCap) v.xnbr[(int64_t)slot * v.ls + j] = (int32_t)k;
        }
    };
    // two candidates per trip: independent load / distance chains, appended
    // in candidate order (four per trip was slower: the chords are short and
    // the tail trips run mostly predicated off)
    auto run = [&](int32_t s, int32_t len) {
        const int maxlen = __reduce_max_sync(full, len);
        for (int t = 0; t < maxlen; t += 2) {
            const bool ok0 = t < len, ok1 = t + 1 < len;
            const int32_t j0 = ok0 ? s + t : (int32_t)k, j1 = ok1 ? s + t + 1 : (int32_t)k;
            const float4 l0 = v.lf[j0], l1 = v.lf[j1];
            const float r20 = list_r2(li, l0), r21 = list_r2(li, l1);
            if (ok0 && r20 < ri2) take(j0, l0, r20);
            if (ok1 && r21 < ri2) take(j1, l1, r21);
        }
    };
    if constexpr (LV) {
        if (I.nlev > 1) {  // warp-uniform: graded impact with traversal-grid levels
            warp_walk_levels(v, I, act, pi, ci, Rs, run);
            if (act) {
                v.nbr_cnt[k] = cnt;
                v.hlist[k] = pi.w;
                if (cnt > cap) atomicMax(&v.flags[0], cnt);
            }
            return;
        }
    }
    int c[3];
    unpack_cell(ci, c[0], c[1], c[2]);
    const float w0 = I.wf[0], w1 = I.wf[1];
    const float iw0 = I.iwf[0], iw1 = I.iwf[1], iw2 = I.iwf[2];
    const int nf0 = I.nf[0], nf1 = I.nf[1], nf2 = I.nf[2];
    // cell ranges by reciprocal multiplies, widened by 1e-5 cell (far above
    // their rounding): a range may gain a cell whose candidates all fail the
    // distance test, never lose one
    constexpr float kWiden = 1.0e-5f;
    int lo0 = c[0] + (int)floorf((pi.x - Rs) * iw0 - kWiden), hi0 = c[0] + (int)floorf((pi.x + Rs) * iw0 + kWiden);
    int lo1 = c[1] + (int)floorf((pi.y - Rs) * iw1 - kWiden), hi1 = c[1] + (int)floorf((pi.y + Rs) * iw1 + kWiden);
    lo0 = lo0 < 0 ? 0 : (lo0 > nf0 - 1 ? nf0 - 1 : lo0);
    hi0 = hi0 < 0 ? 0 : (hi0 > nf0 - 1 ? nf0 - 1 : hi0);
    lo1 = lo1 < 0 ? 0 : (lo1 > nf1 - 1 ? nf1 - 1 : lo1);
    hi1 = hi1 < 0 ? 0 : (hi1 > nf1 - 1 ? nf1 - 1 : hi1);
    const int ulo0 = __reduce_min_sync(full, act ? lo0 : INT_MAX), uhi0 = __reduce_max_sync(full, act ? hi0 : INT_MIN);
    const int ulo1 = __reduce_min_sync(full, act ? lo1 : INT_MAX), uhi1 = __reduce_max_sync(full, act ? hi1 : INT_MIN);
    for (int ix = ulo0; ix <= uhi0; ix++) {
        const float xa = (float)(ix - c[0]) * w0 - pi.x;
        float bx = xa > 0.0f ? xa : (xa + w0 < 0.0f ? -(xa + w0) : 0.0f);
        if (ix == 0 || ix == nf0 - 1) bx = 0.0f;
        const bool in_x = act && ix >= lo0 && ix <= hi0;
        for (int iy = ulo1; iy <= uhi1; iy++) {
            const float ya = (float)(iy - c[1]) * w1 - pi.y;
            float by = ya > 0.0f ? ya : (ya + w1 < 0.0f ? -(ya + w1) : 0.0f);
            if (iy == 0 || iy == nf1 - 1) by = 0.0f;
            const float d2 = bx * bx + by * by;
            int32_t s = 0, len = 0;
            if (in_x && iy >= lo1 && iy <= hi1 && d2 < R2) {
                const float q = R2 - d2;
                const float hz = q * rsqrtf(q) * (1.0f + 1.0e-6f);  // hardware 1/sqrt (2 ulp), widened
                int zl = c[2] + (int)floorf((pi.z - hz) * iw2 - kWiden);
                int zh = c[2] + (int)floorf((pi.z + hz) * iw2 + kWiden);
                zl = zl < 0 ? 0 : (zl > nf2 - 1 ? nf2 - 1 : zl);
                zh = zh < 0 ? 0 : (zh > nf2 - 1 ? nf2 - 1 : zh);
                const int64_t colbase = I.cell_base + ((int64_t)ix * nf1 + iy) * nf2;
                s = v.cell_ptr[colbase + zl];
                len = v.cell_ptr[colbase + zh + 1] - s;
            }
            run(s, len);
        }
    }
    if (act) {
        v.nbr_cnt[k] = cnt;
        v.hlist[k] = pi.w;
        if (cnt > cap) atomicMax(&v.flags[0], cnt);
    }
}

// Work list for the warp-converged list build: one task per run of up to 32
// consecutive sorted particles inside one traversal-cell column of one impact.
template <class R>
static __global__ void k_column_tasks(View<R> v, int32_t* tasks, int32_t* ntask) {
    int64_t k = gtid();
    if (k >= v.n) return;
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask) return;
    int cx, cy, cz;
    unpack_cell(v.cpk[k], cx, cy, cz);
    const int64_t colbase = I.cell_base + ((int64_t)cx * I.nf[1] + cy) * I.nf[2];
    const int32_t cs = v.cell_ptr[colbase];
    if (((int32_t)k - cs) % 32 == 0) tasks[atomicAdd(ntask, 1)] = (int32_t)k;
}

__device__ __forceinline__ float warp_min(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fminf(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}
__device__ __forceinline__ float warp_max(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

// Neighbour-list build, one warp per column task (same lists as k_list_thread,
// bit for bit: each lane appends its candidates in ascending sorted index).
// The warp walks the union of its lanes' sphere chords column by column; every
// candidate is loaded once (broadcast) and tested by all lanes, so the loops
// are warp-uniform.  Periodic impacts take the per-lane path.
template <class R>
static __global__ void __launch_bounds__(256) k_list_warp(View<R> v, const int32_t* tasks, const int32_t* ntask) {
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    const int nt_all = *ntask;
    for (int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < nt_all; q += nwarps) {
        const int32_t t0 = tasks[q];
        const ImpactD& I = v.imps[v.imp[t0]];
        int cx, cy, cz0;
        unpack_cell(v.cpk[t0], cx, cy, cz0);
        const int64_t colbase0 = I.cell_base + ((int64_t)cx * I.nf[1] + cy) * I.nf[2];
        const int32_t cend = v.cell_ptr[colbase0 + I.nf[2]];
        const int nt = min(32, (int)(cend - t0));
        const bool active = lane < nt;
        const int64_t k = t0 + (active ? lane : 0);
        const float4 pi = v.pf[k];
        const uint32_t ci = v.cpk[k];
        const float4 li = v.lf[k];
        const float m = (sizeof(R) == 8 ? I.margin : 0.0f) + I.lmargin;
        const float sl = 1.0f + I.slack;
        const float ri = 2.0f * pi.w * sl + m;
        const float ri2 = ri * ri;
        const float Rs = ri + m;
        int cnt = 0;
        const int cap = v.cap;
        int32_t* out = v.nbr + 4 * k;  // entry t at out[nbr_slot(t, ls)]
        int icx, icy, icz;
        unpack_cell(ci, icx, icy, icz);
        if (I.per[0] | I.per[1] | I.per[2]) {
            if (active) {
                traverse(v, I, pi, ci, Rs, [&](int32_t j, float dxc, float dyc, float dzc) {
                    const float4 pj = v.pf[j];
                    float dx = (pi.x - pj.x) + dxc, dy = (pi.y - pj.y) + dyc, dz = (pi.z - pj.z) + dzc;
                    if (I.per[0]) dx -= I.Lf[0] * rintf(dx / I.Lf[0]);
                    if (I.per[1]) dy -= I.Lf[1] * rintf(dy / I.Lf[1]);
                    if (I.per[2]) dz -= I.Lf[2] * rintf(dz / I.Lf[2]);
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 < ri2) {
                        if (cnt < cap) out[nbr_slot(cnt, v.ls)] = j;
                        cnt++;
                        const float rj = 2.0f * pj.w * sl + m, rb = (pi.w + pj.w) * sl + m;
                        if (!(r2 < rj * rj) && r2 < rb * rb) {
                            const int slot = atomicAdd(&v.xcnt[j], 1);
                            if (slot < kExtraCap) v.xnbr[(int64_t)slot * v.ls + j] = (int32_t)k;
                        }
                    }
                });
            }
        } else {
            const float w0 = I.wf[0], w1 = I.wf[1], w2 = I.wf[2];
            // union x / y column range of the warp (positions relative to the shared column)
            const float xl = warp_min(active ? pi.x - Rs : 3e38f), xh = warp_max(active ? pi.x + Rs : -3e38f);
            const float yl = warp_min(active ? pi.y - Rs : 3e38f), yh = warp_max(active ? pi.y + Rs : -3e38f);
            int lox = cx + (int)floorf(xl / w0), hix = cx + (int)floorf(xh / w0);
            int loy = cy + (int)floorf(yl / w1), hiy = cy + (int)floorf(yh / w1);
            lox = max(0, min(I.nf[0] - 1, lox)); hix = max(0, min(I.nf[0] - 1, hix));
            loy = max(0, min(I.nf[1] - 1, loy)); hiy = max(0, min(I.nf[1] - 1, hiy));
            const float zi = (float)icz * w2 + pi.z;   // lane z in the column frame (range use only)
            const int nf2 = I.nf[2];
            for (int ix = lox; ix <= hix; ix++) {
                const float xa = (float)(ix - icx) * w0 - pi.x;
                float bx = xa > 0.0f ? xa : (xa + w0 < 0.0f ? -(xa + w0) : 0.0f);
                if (ix == 0 || ix == I.nf[0] - 1) bx = 0.0f;
                for (int iy = loy; iy <= hiy; iy++) {
                    const float ya = (float)(iy - icy) * w1 - pi.y;
                    float by = ya > 0.0f ? ya : (ya + w1 < 0.0f ? -(ya + w1) : 0.0f);
                    if (iy == 0 || iy == I.nf[1] - 1) by = 0.0f;
                    const float d2 = bx * bx + by * by;
                    float zlo = 3e38f, zhi = -3e38f;
                    if (active && d2 < Rs * Rs) {
                        const float hz = sqrtf(Rs * Rs - d2);
                        zlo = zi - hz;
                        zhi = zi + hz;
                    }
                    zlo = warp_min(zlo);
                    zhi = warp_max(zhi);
                    if (zlo > zhi) continue;
                    zlo -= 1e-3f * w2;  // covers rounding of the column-frame z
                    zhi += 1e-3f * w2;
                    int zl = (int)floorf(zlo / w2), zh = (int)floorf(zhi / w2);
                    zl = max(0, min(nf2 - 1, zl));
                    zh = max(0, min(nf2 - 1, zh));
                    const int64_t colbase = I.cell_base + ((int64_t)ix * I.nf[1] + iy) * nf2;
                    const int32_t s = v.cell_ptr[colbase + zl];
                    const int32_t e = v.cell_ptr[colbase + zh + 1];
                    for (int32_t j = s; j < e; j++) {
                        const float4 lj = v.lf[j];
                        const float r2 = list_r2(li, lj);
                        if (active && r2 < ri2) {
                            if (cnt < cap) out[nbr_slot(cnt, v.ls)] = j;
                            cnt++;
                            const float rj = 2.0f * lj.w * sl + m, rb = (pi.w + lj.w) * sl + m;
                            if (!(r2 < rj * rj) && r2 < rb * rb) {
                                const int slot = atomicAdd(&v.xcnt[j], 1);
                                if (slot < kExtraCap) v.xnbr[(int64_t)slot * v.ls + j] = (int32_t)k;
                            }
                        }
                    }
                }
            }
        }
        if (active) {
            v.nbr_cnt[k] = cnt;
            v.hlist[k] = pi.w;
            if (cnt > cap) atomicMax(&v.flags[0], cnt);
        }
    }
}

// Neighbour-list build, one warp per particle.  The lanes take the cell
// columns that meet the particle's search sphere, 32 at a time, and walk them
// cell by cell in step; the hits of a step are compacted with a ballot, so the
// list is written in coalesced runs and the loops stay converged.  Same sets
// and the same extra-list entries as k_list_thread (the pair test is the same
// expression); entries are ordered by step, then by column.
__device__ __forceinline__ int wrap_cell(int i, int nf, int per) {
    return per ? ((i % nf) + nf) % nf : i;
}

template <class R>
static __global__ void __launch_bounds__(256) k_list_wpp(View<R> v) {
    const int lane = threadIdx.x & 31;
    const int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= v.n) return;  // warp-uniform
    const ImpactD& I = v.imps[v.imp[k]];
    if (!I.mask) return;
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    const float4 li = v.lf[k];
    const float m = (sizeof(R) == 8 ? I.margin : 0.0f) + I.lmargin;
    const float sl = 1.0f + I.slack;
    const float ri = 2.0f * pi.w * sl + m;
    const float ri2 = ri * ri;
    const float Rs = ri + m;
    const int cap = v.cap;
    int32_t* out = v.nbr + 4 * k;  // entry t at out[nbr_slot(t, ls)]
    int c[3];
    unpack_cell(ci, c[0], c[1], c[2]);
    const float o[3] = {pi.x, pi.y, pi.z};
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {  // the cell box of traverse()
        const float w = I.wf[a];
        int l = c[a] + (int)floorf((o[a] - Rs) / w);
        int h = c[a] + (int)floorf((o[a] + Rs) / w);
        const int nf = I.nf[a];
        if (I.per[a]) {
            if (h - l + 1 > nf) { l = c[a] - nf / 2; h = l + nf - 1; }
        } else {
            l = l < 0 ? 0 : (l > nf - 1 ? nf - 1 : l);
            h = h < 0 ? 0 : (h > nf - 1 ? nf - 1 : h);
        }
        lo[a] = l;
        hi[a] = h;
    }
    const bool sphere = !(I.per[0] | I.per[1] | I.per[2]);
    const float w0 = I.wf[0], w1 = I.wf[1], w2 = I.wf[2];
    const int nf0 = I.nf[0], nf1 = I.nf[1], nf2 = I.nf[2];
    const int ncy = hi[1] - lo[1] + 1;
    const int ncol = (hi[0] - lo[0] + 1) * ncy;
    const float R2 = Rs * Rs;
    const unsigned below = (1u << lane) - 1u;
    int cnt = 0;
    for (int base = 0; base < ncol; base += 32) {
        const int q = base + lane;
        int iz = 0, izh = -1;
        int32_t j = 0, e = 0;
        float dxc = 0.0f, dyc = 0.0f, dzc = 0.0f;
        int64_t colbase = 0;
        if (q < ncol) {
            const int ix = lo[0] + q / ncy, iy = lo[1] + q % ncy;
            dxc = (float)(c[0] - ix) * w0;
            dyc = (float)(c[1] - iy) * w1;
            colbase = I.cell_base + ((int64_t)wrap_cell(ix, nf0, I.per[0]) * nf1 + wrap_cell(iy, nf1, I.per[1])) * nf2;
            iz = lo[2];
            izh = hi[2];
            if (sphere) {  // the column pruning and z chord of traverse_sphere()
                const float xa = (float)(ix - c[0]) * w0 - o[0];
                float bx = xa > 0.0f ? xa : (xa + w0 < 0.0f ? -(xa + w0) : 0.0f);
                if (ix == 0 || ix == nf0 - 1) bx = 0.0f;
                const float ya = (float)(iy - c[1]) * w1 - o[1];
                float by = ya > 0.0f ? ya : (ya + w1 < 0.0f ? -(ya + w1) : 0.0f);
                if (iy == 0 || iy == nf1 - 1) by = 0.0f;
                const float d2 = bx * bx + by * by;
                if (d2 < R2) {
                    const float hz = sqrtf(R2 - d2);
                    int zl = c[2] + (int)floorf((o[2] - hz) / w2);
                    int zh = c[2] + (int)floorf((o[2] + hz) / w2);
                    iz = zl < 0 ? 0 : (zl > nf2 - 1 ? nf2 - 1 : zl);
                    izh = zh < 0 ? 0 : (zh > nf2 - 1 ? nf2 - 1 : zh);
                } else {
                    izh = iz - 1;
                }
            }
            if (iz <= izh) {
                const int wz = wrap_cell(iz, nf2, I.per[2]);
                j = v.cell_ptr[colbase + wz];
                e = v.cell_ptr[colbase + wz + 1];
                dzc = (float)(c[2] - iz) * w2;
            }
        }
        while (true) {
            while (j >= e && iz < izh) {  // next non-empty cell of this lane's column
                iz++;
                const int wz = wrap_cell(iz, nf2, I.per[2]);
                j = v.cell_ptr[colbase + wz];
                e = v.cell_ptr[colbase + wz + 1];
                dzc = (float)(c[2] - iz) * w2;
            }
            const bool have = j < e;
            if (!__any_sync(0xffffffffu, have)) break;
            bool hit = false;
            if (have) {
                float r2, hj;
                if (sphere) {
                    const float4 lj = v.lf[j];
                    r2 = list_r2(li, lj);
                    hj = lj.w;
                } else {
                    const float4 pj = v.pf[j];
                    float dx = (pi.x - pj.x) + dxc;
                    float dy = (pi.y - pj.y) + dyc;
                    float dz = (pi.z - pj.z) + dzc;
                    if (I.per[0]) dx -= I.Lf[0] * rintf(dx / I.Lf[0]);
                    if (I.per[1]) dy -= I.Lf[1] * rintf(dy / I.Lf[1]);
                    if (I.per[2]) dz -= I.Lf[2] * rintf(dz / I.Lf[2]);
                    r2 = dx * dx + dy * dy + dz * dz;
                    hj = pj.w;
                }
                hit = r2 < ri2;
                if (hit) {
                    const float rj = 2.0f * hj * sl + m;
                    const float rb = (pi.w + hj) * sl + m;
                    if (!(r2 < rj * rj) && r2 < rb * rb) {
                        const int slot = atomicAdd(&v.xcnt[j], 1);
                        if (slot < kExtraCap) v.xnbr[(int64_t)slot * v.ls + j] = (int32_t)k;
                    }
                }
            }
            const unsigned bm = __ballot_sync(0xffffffffu, hit);
            if (hit) {
                const int pos = cnt + __popc(bm & below);
                if (pos < cap) out[nbr_slot(pos, v.ls)] = j;
            }
            cnt += __popc(bm);
            if (have) j++;
        }
    }
    if (lane == 0) {
        v.nbr_cnt[k] = cnt;
        v.hlist[k] = pi.w;
        if (cnt > cap) atomicMax(&v.flags[0], cnt);
    }
}

// Sort each particle's extra list (filled by atomics) into ascending order
// (refresh != 0: only in impacts whose lists are being rebuilt).
template <class R>
static __global__ void k_sort_extra(View<R> v, int refresh) {
    int64_t k = gtid();
    if (k >= v.n) return;
    if (refresh && !v.imps[v.imp[k]].slack_flag) return;
    const int c = min(v.xcnt[k], kExtraCap);
    if (c < 2) return;
    int32_t* a = v.xnbr + k;  // entry t at a[t * ls]
    const int64_t ls = v.ls;
    for (int i = 1; i < c; i++) {
        int32_t x = a[i * ls];
        int j = i - 1;
        while (j >= 0 && a[j * ls] > x) {
            a[(j + 1) * ls] = a[j * ls];
            j--;
        }
        a[(j + 1) * ls] = x;
    }
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
    // the part of the exact sum the rounded value misses (value() + low())
    __device__ __forceinline__ R low() const { return -c; }
};
template <class R>
struct Plain {
    R s;
    __device__ __forceinline__ void init() { s = R(0); }
    __device__ __forceinline__ void add(R x) { s += x; }
    __device__ __forceinline__ R value() const { return s; }
    __device__ __forceinline__ R low() const { return R(0); }
};
template <class R>
using AccT = typename std::conditional<sizeof(R) == 4, Kahan<R>, Plain<R>>::type;

// Packed FP32 arithmetic: one sm_100-class instruction works on two lanes of a
// float2, each rounded exactly as the scalar operation (x - y is formed as the
// fused y * -1 + x, which rounds once, like the subtraction).
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

// Two compensated sums side by side (the Kahan steps above, lane by lane).
struct Kahan2 {
    float2 s, c;
    __device__ __forceinline__ void init() { s = c = make_float2(0.0f, 0.0f); }
    __device__ __forceinline__ void add(float2 x) {
        const float2 y = sub2(x, c);
        const float2 t = add2(s, y);
        c = sub2(sub2(t, s), y);
        s = t;
    }
};

// Does particle k's superset list still cover it (count within capacity and h
// within the slack, with an allowance for the FP32 distance)?
template <class R>
__device__ __forceinline__ bool list_covers(const View<R>& v, const ImpactD& I, int64_t k, float h_now) {
    return v.nbr_cnt[k] <= v.cap && h_now <= v.hlist[k] * (1.0f + I.slack) * 0.99999f;
}

// Density sum and h update (sph.hpp:189-201), `iters` iterations in one
// launch.  Criterion r < 2 h_i (self included) within the reference stencil;
// compensated sum in the mixed form.  An iteration reads only the particle's
// own h and the neighbours' positions and masses, so running the iterations
// back to back per particle gives the same result as one launch per iteration.
template <class R, bool LV = false, bool PER = true>
static __global__ void __launch_bounds__(256, sizeof(R) == 4 ? 4 : 2) k_density(View<R> v, int iters) {
    int64_t k = gtid();
    if (k >= v.n) return;
    ImpactD& I = v.imps[v.imp[k]];
    if (!(I.mask && I.active)) return;
    R hi = v.hh[k];
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    const unsigned long long bi = v.refbin[k];
    const float m = sizeof(R) == 8 ? I.margin : 0.0f;
    const R mass_k = v.mass[k];
    const R h0 = I.use_h0 ? v.h0[k] : (R)I.h_init;
    R rho = R(1e-30), rho_lo = R(0);
    for (int it = 0; it < iters; it++) {
        const R ihi = R(1) / hi;
        const bool need_member = 2.0f * (float)hi + 2.0f * m >= I.cwmin * 0.999f;
        AccT<R> sum;
        sum.init();
        const float th2 = (2.0f * (float)hi + m) * (2.0f * (float)hi + m);
        // mixed form: one entry's m_j W(r, h_i) from its offset record and (mass, cell)
        auto w_mixed = [&](int32_t j, float4 pj, float2 mk) -> float {
            float dx, dy, dz;
            sep_f32<PER>(I, pi, ci, pj, __float_as_uint(mk.y), dx, dy, dz);
            const float r2 = dx * dx + dy * dy + dz * dz;
            // the kernel vanishes at q >= 2; only the stencil restriction needs a test
            const float r = r2 > 0.0f ? r2 * rsqrtf(r2) : 0.0f;  // hardware 1/sqrt (2 ulp)
            float w = mk.x * kernel_W_bf<float>(r, (float)ihi);
            if (need_member && !ref_member(bi, v.refbin[j], I)) w = 0.0f;
            return w;
        };
        auto body = [&](int32_t j) {
            if constexpr (sizeof(R) == 8) {
                float fx, fy, fz;  // FP32 pre-filter: skip entries that clearly fail
                sep_f32<PER>(I, pi, ci, v.pf[j], v.cpk[j], fx, fy, fz);
                if (!(fx * fx + fy * fy + fz * fz < th2)) return;
                double dx, dy, dz;
                double rr = sep_exact<PER>(v, I, k, j, dx, dy, dz);
                if (!(rr < 2.0 * (double)hi)) return;
                if (need_member && !ref_member(bi, v.refbin[j], I)) return;
                sum.add(v.mass[j] * kernel_W_ih<R>((R)rr, ihi));
            } else {
                sum.add((R)w_mixed(j, v.pf[j], v.pk[j]));
            }
        };
        if (list_covers(v, I, k, (float)hi)) {
            const int cnt = v.nbr_cnt[k];
            if constexpr (sizeof(R) == 4) {
                // two entries per trip: both loads in flight, summed in list order
                walk_list_pairs(v.nbr, v.ls, k, cnt, body, [&](int32_t j0, int32_t j1) {
                    const float4 p0 = v.pf[j0], p1 = v.pf[j1];
                    const float2 m0 = v.pk[j0], m1 = v.pk[j1];
                    const float w0 = w_mixed(j0, p0, m0), w1 = w_mixed(j1, p1, m1);
                    sum.add((R)w0);
                    sum.add((R)w1);
                });
            } else {
                walk_list(v.nbr, v.ls, k, cnt, body);
            }
        } else {
            const float hf = (float)hi;
            traverse<R, LV>(v, I, pi, ci, 2.0f * hf * 1.0001f + 2.0f * I.margin + 1e-6f * hf,
                     [&](int32_t j, float, float, float) { body(j); });
        }
        rho = rmax(sum.value(), R(1e-30));
        rho_lo = rho > R(1e-30) ? sum.low() : R(0);
        hi = rmin(R(2) * h0, rmax(R(0.5) * h0, (R)I.eta * rcbrt(mass_k / rho)));
    }
    v.rho[k] = rho;
    v.rho_lo[k] = rho_lo;
    v.hh[k] = hi;
    v.pf[k].w = (float)hi;
    v.lf[k].w = (float)hi;
    impact_atomic_max(&I.hm_bits, (double)hi);  // the round's new max h
    if (!((float)hi <= v.hlist[k] * (1.0f + I.slack) * 0.99999f)) {
        atomicOr(&I.slack_flag, 1);
        atomicOr(&v.flags[2], 1);
    }
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
    // all loads before the stores (the columns may alias as far as the compiler knows)
    const R rho = v.rho[k];
    const R u = (R)v.u[k];
    const R rho_lo = v.rho_lo[k];
    const R mass = v.mass[k];
    R S[6];
#pragma unroll
    for (int c = 0; c < 6; c++) S[c] = v.S[c][k];
    const R D = I.damage_on ? v.D[k] : R(0);
    double vx = 0.0, vy = 0.0, vz = 0.0;
    float4 pfk = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t cpk = 0;
    if (sizeof(R) == 4) {
        vx = v.vx[k]; vy = v.vy[k]; vz = v.vz[k];
        pfk = v.pf[k];
        cpk = v.cpk[k];
    }
    R P, cs;
    eos_P_cs(m, rho, u, P, cs, rho_lo);
    const R csig = rsqrt_(cs * cs + (R(4) / R(3)) * m.G / rmax(rho, R(1e-30)));
    R pf = P, dsc = R(1);
    R sigmax = R(0);
    if (I.damage_on) {
        sigmax = -P + eig_max(S[0], S[1], S[2], S[3], S[4], S[5]);
        dsc = R(1) - D;
        if (P < R(0)) pf = dsc * P;
    }
    const R irho2 = R(1) / (rho * rho);
    const R Rart = (I.eps_as > 0 && pf < R(0)) ? (R)I.eps_as * (-pf) * irho2 : R(0);
    const R pfr2 = pf * irho2, dsr2 = irho2 * dsc, vol = mass / rho;
    v.P[k] = P;
    v.cs[k] = cs;
    v.csig[k] = csig;
    if (I.damage_on) v.sigmax[k] = sigmax;
    v.Pf[k] = pf;
    v.dscale[k] = dsc;
    v.Rart[k] = Rart;
    v.pfr2[k] = pfr2;
    v.dsr2[k] = dsr2;
    v.vol[k] = vol;
    if (sizeof(R) == 4) {
        float4* o = v.fr + 6 * k;
        const float hx = (float)vx, hy = (float)vy, hz = (float)vz;
        o[0] = pfk;
        // .w lanes carry the mass and packed cell of the particle
        o[1] = make_float4(hx, hy, hz, (float)mass);
        o[2] = make_float4((float)(vx - (double)hx), (float)(vy - (double)hy), (float)(vz - (double)hz),
                           __uint_as_float(cpk));
        o[3] = make_float4((float)vol, (float)rho, (float)csig, (float)pfr2);
        o[4] = make_float4((float)dsr2, (float)Rart, (float)S[4], (float)S[5]);
        o[5] = make_float4((float)S[0], (float)S[1], (float)S[2], (float)S[3]);
    }
}

// Velocity gradient -> Jaumann dS/dt and deviatoric power (sph.hpp:212-258)
// fused with the momentum / energy pair loop (sph.hpp:277-317).  Writes acc,
// the new dudt and dSdt, eps_work.
// Shared-memory staging of the neighbour records of the mixed force pass: every
// lane owns a ring of SS stages of SE entries; a stage is filled by one
// 96-byte bulk copy (cp.async.bulk, the TMA engine) per entry straight from the
// record array, completing on the warp's mbarrier of that stage, while the lane
// evaluates the pairs of the other stages from shared memory.  A lane's slot is
// SE x 96 bytes plus 16 of padding, so the 32 lanes' 16-byte reads of the same
// field fall in distinct bank groups.
template <int SE, int SS>
struct ForceStaging {
    static constexpr int kLaneBytes = SE * 96 + 16;
    static constexpr int kStageBytes = 32 * kLaneBytes;
    static constexpr int kWarpBytes = 16 * SS + SS * kStageBytes;
    static constexpr int kBlock = 128;
    static constexpr int kSmemBytes = (kBlock / 32) * kWarpBytes;
};
constexpr long long kWaitNs = 500000000ll;   // a bounded wait gives up after 0.5 s
constexpr int kWaitPolls = 1 << 26;          // ... or after this many polls

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// mbar_wait bounded in time as well as in polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    if (mbar_test(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (int i = 0; i < kWaitPolls; i += 64) {
        if (mbar_wait(bar, parity, 64)) return true;
        if ((long long)(global_ns() - t0) > kWaitNs) return false;
    }
    return false;
}

// ASYNC selects the copy engine of the staging: false = one bulk copy per
// entry (cp.async.bulk, TMA), true = six 16-byte cp.async per entry (the load
// path through L1, completion tracked by cp.async.mbarrier.arrive).
template <class R, int SE = 0, int SS = 0, bool ASYNC = false, bool LV = false, bool PER = true>
static __global__ void __launch_bounds__(128, sizeof(R) == 4 ? 4 : 1) k_force(View<R> v, int32_t* wait_err) {
    using Acc = AccT<R>;
    constexpr bool kStaged = SS > 0 && sizeof(R) == 4;
    int64_t k = gtid();
    bool live = k < v.n;
    if constexpr (!kStaged) {
        if (!live) return;
    }
    if (!live) k = v.n - 1;  // staged: every lane of the warp takes part in the barrier phases
    const ImpactD& I = v.imps[v.imp[k]];
    if constexpr (!kStaged) {
        if (!I.mask) return;
    }
    live = live && I.mask;
    const R G = v.mats[v.mat[k]].G;
    const bool strength = G > R(0);
    const R alpha = (R)I.alpha, beta = (R)I.beta, eps = (R)I.eps, eps_as = (R)I.eps_as;
    const R alpha_u = (R)I.alpha_u;
    const R inv_poly = sizeof(R) == 4 ? (R)I.inv_poly_eta_f : (R)I.inv_poly_eta;
    const R hi = v.hh[k], rhoi = v.rho[k], csi = v.csig[k], Pi_over = v.pfr2[k];
    const R dsri = v.dsr2[k], Rai = v.Rart[k];
    const double vxi = v.vx[k], vyi = v.vy[k], vzi = v.vz[k];
    float4 vhi = make_float4(0, 0, 0, 0), vli = vhi;
    if (sizeof(R) == 4) { vhi = v.fr[6 * k + 1]; vli = v.fr[6 * k + 2]; }
    const R sxx = v.S[0][k], syy = v.S[1][k], szz = v.S[2][k];
    const R sxy = v.S[3][k], sxz = v.S[4][k], syz = v.S[5][k];
    R L00 = 0, L01 = 0, L02 = 0, L10 = 0, L11 = 0, L12 = 0, L20 = 0, L21 = 0, L22 = 0;
    Acc ax, ay, az, du;
    ax.init(); ay.init(); az.init(); du.init();
    // mixed form: the same sums in packed pairs -- (L00, L01), (L10, L11),
    // (L20, L21), (L02, L12), and compensated (ax, ay), (az, du)
    float2 Lp0 = f2(0.0f), Lp1 = f2(0.0f), Lp2 = f2(0.0f), Lpz = f2(0.0f);
    float Lp22 = 0.0f;
    Kahan2 kxy, kzu;
    kxy.init(); kzu.init();
    const float4 pi = v.pf[k];
    const uint32_t ci = v.cpk[k];
    const float m = sizeof(R) == 8 ? I.margin : 0.0f;
    const bool need_member = (float)hi + I.hmax_f + 2.0f * m >= I.cwmin * 0.999f;
    // one pair's contributions: strain-rate tensor, momentum, energy
    auto pair_math = [&](R rx, R ry, R rz, R r, R hbar, R ihb, R dW, R gx, R gy, R gz, R vx, R vy, R vz,
                         R Vj, R rhoj, R csj, R pfj, R dsj, R Raj, R mj, R tjxx, R tjyy, R tjzz, R tjxy,
                         R tjxz, R tjyz, int32_t j) {
        if (strength) {
            const R ex = -vx * Vj, ey = -vy * Vj, ez = -vz * Vj;  // Vj (v_j - v_i)
            L00 += ex * gx; L01 += ex * gy; L02 += ex * gz;
            L10 += ey * gx; L11 += ey * gy; L12 += ey * gz;
            L20 += ez * gx; L21 += ez * gy; L22 += ez * gz;
        }
        const R dvr = vx * rx + vy * ry + vz * rz;
        R Pij = R(0);
        if (dvr < R(0)) {
            const R mu = pair_div(hbar * dvr, r * r + eps * hbar * hbar);
            const R cbar = R(0.5) * (csi + csj);
            Pij = pair_div(-alpha * cbar * mu + beta * mu * mu, R(0.5) * (rhoi + rhoj));
        }
        const R term = Pi_over + pfj + Pij;
        du.add(R(0.5) * mj * term * (vx * gx + vy * gy + vz * gz));
        R mterm = term;
        if (eps_as > R(0)) {
            const R q = r * ihb;
            const R t = rmax(R(2) - q, R(0)), a = rmax(R(1) - q, R(0));
            const R fr = (R(0.25) * t * t * t - a * a * a) * inv_poly;
            R fn = fr * fr;
            fn *= fn;
            mterm += (Rai + Raj) * fn;
        }
        const R mm = mj * mterm;
        const R stx = (sxx * gx + sxy * gy + sxz * gz) * dsri + (tjxx * gx + tjxy * gy + tjxz * gz) * dsj;
        const R sty = (sxy * gx + syy * gy + syz * gz) * dsri + (tjxy * gx + tjyy * gy + tjyz * gz) * dsj;
        const R stz = (sxz * gx + syz * gy + szz * gz) * dsri + (tjxz * gx + tjyz * gy + tjzz * gz) * dsj;
        ax.add(stx * mj - gx * mm);
        ay.add(sty * mj - gy * mm);
        az.add(stz * mj - gz * mm);
        if (alpha_u > R(0)) {
            const R rbar = R(0.5) * (rhoi + rhoj);
            // own P and u read here: the conductivity term is off in most runs,
            // and keeping them live through the pair loop costs registers
            const R vsig = rsqrt_(pair_div(rabs(v.P[k] - v.P[j]), rbar));
            du.add(pair_div(alpha_u * mj * vsig * ((R)v.u[k] - (R)v.u[j]) * dW, rbar));
        }
    };
    // mixed form: one list entry's contributions from its six record float4s
    // (global memory or a shared-memory stage); exact zeros for a failing pair
    auto rec_body = [&](int32_t j, const float4 pj, const float4 vhj, const float4 vlj, const float4 fa,
                        const float4 fb, const float4 fc) {
        const float mj = vhj.w;  // (mass, packed cell) ride in the .w lanes
        float dx, dy, dz;
        sep_f32<PER>(I, pi, ci, pj, __float_as_uint(vlj.w), dx, dy, dz);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float hif = (float)hi;
        const float hs = hif + pj.w;
        bool ok = r2 < hs * hs && r2 != 0.0f;
        if (need_member) ok = ok && ref_member(v.refbin[k], v.refbin[j], I);  // own bins re-read: rarely needed
        const float irs = ok ? rsqrtf(r2) : 1.0f;  // hardware 1/sqrt (2 ulp)
        const float r = ok ? r2 * irs : 1.0f;
        const float hbar = 0.5f * (hif + pj.w);
        const float ihb = pair_div(1.0f, hbar);
        const float dW = ok ? kernel_dW_bf<float>(r, ihb) : 0.0f;
        const float wg = dW * irs;
        const float2 gxy = mul2(f2(dx, dy), f2(wg));
        const float gz = dz * wg;
        // hi parts nearly cancel exactly; lo parts restore the FP64 difference
        const float2 vxy = add2(sub2(f2(vhi.x, vhi.y), f2(vhj.x, vhj.y)), sub2(f2(vli.x, vli.y), f2(vlj.x, vlj.y)));
        const float vz = (vhi.z - vhj.z) + (vli.z - vlj.z);
        const float Vj = fa.x, rhoj = fa.y, csj = fa.z, pfj = fa.w, dsj = fb.x, Raj = fb.y;
        if (strength) {  // Vj (v_j - v_i) (x) grad W
            const float2 exy = mul2(vxy, f2(-Vj));
            const float ez = -vz * Vj;
            Lp0 = fma2(f2(exy.x), gxy, Lp0);
            Lp1 = fma2(f2(exy.y), gxy, Lp1);
            Lp2 = fma2(f2(ez), gxy, Lp2);
            Lpz = fma2(exy, f2(gz), Lpz);
            Lp22 = fmaf(ez, gz, Lp22);
        }
        const float dvr = vxy.x * dx + vxy.y * dy + vz * dz;
        float Pij = 0.0f;
        if (dvr < 0.0f) {
            const float mu = pair_div(hbar * dvr, r * r + (float)eps * hbar * hbar);
            const float cbar = 0.5f * ((float)csi + csj);
            Pij = pair_div(-(float)alpha * cbar * mu + (float)beta * mu * mu, 0.5f * ((float)rhoi + rhoj));
        }
        const float term = (float)Pi_over + pfj + Pij;
        float dut = 0.5f * mj * term * (vxy.x * gxy.x + vxy.y * gxy.y + vz * gz);
        float mterm = term;
        if (eps_as > R(0)) {
            const float q = r * ihb;
            const float t = fmaxf(2.0f - q, 0.0f), a = fmaxf(1.0f - q, 0.0f);
            const float fr = (0.25f * t * t * t - a * a * a) * (float)inv_poly;
            float fn = fr * fr;
            fn *= fn;
            mterm += ((float)Rai + Raj) * fn;
        }
        const float mm = mj * mterm;
        // (S_i dscale_i / rho_i^2 + S_j dscale_j / rho_j^2) . grad W, x and y rows packed
        const float2 own = fma2(f2((float)sxz, (float)syz), f2(gz),
                                fma2(f2((float)sxy, (float)syy), f2(gxy.y), mul2(f2((float)sxx, (float)sxy), f2(gxy.x))));
        const float2 oth = fma2(f2(fb.z, fb.w), f2(gz), fma2(f2(fc.w, fc.y), f2(gxy.y), mul2(f2(fc.x, fc.w), f2(gxy.x))));
        const float2 stxy = fma2(oth, f2(dsj), mul2(own, f2((float)dsri)));
        const float stz = ((float)sxz * gxy.x + (float)syz * gxy.y + (float)szz * gz) * (float)dsri +
                          (fb.z * gxy.x + fb.w * gxy.y + fc.z * gz) * dsj;
        kxy.add(fma2(gxy, f2(-mm), mul2(stxy, f2(mj))));
        if (alpha_u > R(0)) {
            const float rbar = 0.5f * ((float)rhoi + rhoj);
            const float vsig = rsqrt_(pair_div(fabsf((float)v.P[k] - (float)v.P[j]), rbar));
            dut += pair_div((float)alpha_u * mj * vsig * ((float)v.u[k] - (float)v.u[j]) * dW, rbar);
        }
        kzu.add(f2(stz * mj - gz * mm, dut));
    };
    const float hs_pad = 2.0f * m;
    auto body = [&](int32_t j) {
        if constexpr (sizeof(R) == 8) {
            if (j == (int32_t)k) return;
            const float4 pjf = v.pf[j];
            float fx, fy, fz;  // FP32 pre-filter: skip entries that clearly fail
            sep_f32<PER>(I, pi, ci, pjf, v.cpk[j], fx, fy, fz);
            const float lim = pi.w + pjf.w + hs_pad;
            if (!(fx * fx + fy * fy + fz * fz < lim * lim)) return;
            const R hj = v.hh[j];
            double dx, dy, dz;
            double rr = sep_exact<PER>(v, I, k, j, dx, dy, dz);
            double hsum = __dadd_rn((double)hi, (double)hj);
            if (rr >= hsum || rr == 0.0) return;
            if (need_member && !ref_member(v.refbin[k], v.refbin[j], I)) return;
            const R rx = (R)dx, ry = (R)dy, rz = (R)dz, r = (R)rr;
            const R hbar = R(0.5) * (hi + hj);
            const R ihb = R(1) / hbar;
            const R dW = kernel_dW_bf<R>(r, ihb);
            const R wg = dW / r;
            const R gx = rx * wg, gy = ry * wg, gz = rz * wg;
            const R vx = (R)(vxi - v.vx[j]), vy = (R)(vyi - v.vy[j]), vz = (R)(vzi - v.vz[j]);
            const R Vj = v.vol[j], rhoj = v.rho[j], csj = v.csig[j], pfj = v.pfr2[j];
            const R dsj = v.dsr2[j], Raj = v.Rart[j], mj = v.mass[j];
            const R tj0 = v.S[0][j], tj1 = v.S[1][j], tj2 = v.S[2][j];
            const R tj3 = v.S[3][j], tj4 = v.S[4][j], tj5 = v.S[5][j];
            pair_math(rx, ry, rz, r, hbar, ihb, dW, gx, gy, gz, vx, vy, vz, Vj, rhoj, csj, pfj, dsj, Raj, mj,
                      tj0, tj1, tj2, tj3, tj4, tj5, j);
        } else {
            // Branch-free: every record of the entry is loaded up front (most
            // entries interact), and a pair that fails the criterion -- or the
            // particle itself (r = 0) -- contributes exact zeros through dW = 0.
            float4 pj, vhj, vlj, fa, fb, fc;
            const float4* rec = v.fr + 6 * (int64_t)j;
            ld_f32x8_ro(rec, pj, vhj);
            ld_f32x8_ro(rec + 2, vlj, fa);
            ld_f32x8_ro(rec + 4, fb, fc);
            rec_body(j, pj, vhj, vlj, fa, fb, fc);
        }
    };
    if constexpr (kStaged) {
        using FS = ForceStaging<SE, SS>;
        extern __shared__ __align__(128) unsigned char force_smem[];
        const unsigned full = 0xffffffffu;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        unsigned char* wb = force_smem + warp * FS::kWarpBytes;
        uint64_t* bars = reinterpret_cast<uint64_t*>(wb);  // stage s's barrier at bars[2 s]
        unsigned char* mine = wb + 16 * SS + lane * FS::kLaneBytes;  // stage s at + s * kStageBytes
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < SS; q++) mbar_init(&bars[2 * q], 32);
            mbar_init_fence();
        }
        __syncwarp();
        const bool use_list = live && !I.slack_flag && v.nbr_cnt[k] <= v.cap && v.xcnt[k] <= kExtraCap;
        const int cnt = use_list ? v.nbr_cnt[k] : 0;
        const int cmax = __reduce_max_sync(full, cnt);
        int32_t jb[SS][SE];
        uint32_t parity = 0;  // bit q: parity of stage q's pending phase
        // fill stage q with entries t0 .. t0 + SE - 1 of this lane's list (0 bytes past its end)
        auto issue = [&](const int q, const int t0) {
            const int32_t* blk = v.nbr + 4 * k + nbr_slot(t0, v.ls);
            if constexpr (SE == 4) {
                const int4 b4 = t0 < cnt ? *reinterpret_cast<const int4*>(blk) : make_int4(0, 0, 0, 0);
                jb[q][0] = b4.x; jb[q][SE > 1 ? 1 : 0] = b4.y; jb[q][SE > 2 ? 2 : 0] = b4.z; jb[q][SE - 1] = b4.w;
            } else {
                const int2 b2 = t0 < cnt ? *reinterpret_cast<const int2*>(blk) : make_int2(0, 0);
                jb[q][0] = b2.x; jb[q][SE - 1] = b2.y;
            }
            const int nv = max(0, min(SE, cnt - t0));
            if constexpr (ASYNC) {
#pragma unroll
                for (int e = 0; e < SE; e++)
                    if (e < nv) {
                        const float4* src = v.fr + 6 * (int64_t)jb[q][e];
                        float4* dst = reinterpret_cast<float4*>(mine + q * FS::kStageBytes + e * 96);
#pragma unroll
                        for (int c = 0; c < 6; c++) async16_g2s(dst + c, src + c);
                    }
                async_arrive(&bars[2 * q]);
            } else {
                mbar_arrive_tx(&bars[2 * q], 96u * (uint32_t)nv);
#pragma unroll
                for (int e = 0; e < SE; e++)
                    if (e < nv)
                        bulk_g2s(mine + q * FS::kStageBytes + e * 96, v.fr + 6 * (int64_t)jb[q][e], 96u,
                                 &bars[2 * q]);
            }
        };
#pragma unroll
        for (int q = 0; q < SS; q++) issue(q, q * SE);
        bool failed = false;
        for (int base = 0; base < cmax && !failed; base += SS * SE) {
#pragma unroll
            for (int q = 0; q < SS; q++) {
                const int t0 = base + q * SE;
                const bool ok = mbar_wait_bounded(&bars[2 * q], (parity >> q) & 1u);
                if (__any_sync(full, !ok)) {
                    failed = true;
                    break;
                }
                parity ^= 1u << q;
                const float4* rb = reinterpret_cast<const float4*>(mine + q * FS::kStageBytes);
#pragma unroll
                for (int e = 0; e < SE; e++)
                    if (t0 + e < cnt)
                        rec_body(jb[q][e], rb[6 * e], rb[6 * e + 1], rb[6 * e + 2], rb[6 * e + 3], rb[6 * e + 4],
                                 rb[6 * e + 5]);
                issue(q, t0 + SS * SE);
            }
        }
        if (failed) {
            // a stage's copies did not land in time: report it, let every copy
            // still in flight into this warp's slots complete (bounded), leave
            // this warp's outputs unwritten
            if (lane == 0) atomicOr(wait_err, 1);
#pragma unroll
            for (int q = 0; q < SS; q++) mbar_wait_bounded(&bars[2 * q], (parity >> q) & 1u);
            return;
        }
        if (!live) return;
        if (use_list) {
            const int xc = v.xcnt[k];
            const int32_t* xl = v.xnbr + k;
            for (int t = 0; t < xc; t++, xl += v.ls) body(*xl);
        } else {
            traverse<R, LV>(v, I, pi, ci, pi.w + I.hmax_f + 2.0f * I.margin + 1e-6f * pi.w,
                     [&](int32_t j, float, float, float) { body(j); });
        }
    } else if (!I.slack_flag && v.nbr_cnt[k] <= v.cap && v.xcnt[k] <= kExtraCap) {
        const int cnt = v.nbr_cnt[k];
        walk_list(v.nbr, v.ls, k, cnt, body);
        const int xc = v.xcnt[k];
        const int32_t* xl = v.xnbr + k;
        for (int t = 0; t < xc; t++, xl += v.ls) body(*xl);
    } else {
        traverse<R, LV>(v, I, pi, ci, pi.w + I.hmax_f + 2.0f * I.margin + 1e-6f * pi.w,
                 [&](int32_t j, float, float, float) { body(j); });
    }
    if constexpr (sizeof(R) == 4) {
        L00 = Lp0.x; L01 = Lp0.y; L10 = Lp1.x; L11 = Lp1.y; L20 = Lp2.x; L21 = Lp2.y;
        L02 = Lpz.x; L12 = Lpz.y; L22 = Lp22;
        ax.s = kxy.s.x; ay.s = kxy.s.y; az.s = kzu.s.x; du.s = kzu.s.y;
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
    v.dudt_new[k] = du.value() + epsw * v.dscale[k];
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
        int64_t b = v.flaw_beg[g], e = v.flaw_end[g];
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
        // all loads before the stores (the columns may alias as far as the compiler knows)
        const double vx = v.vx[k] + (double)v.ax[k] * (0.5 * dt);
        const double vy = v.vy[k] + (double)v.ay[k] * (0.5 * dt);
        const double vz = v.vz[k] + (double)v.az[k] * (0.5 * dt);
        double u = v.u[k] + (0.5 * dt) * ((double)v.dudt[k] + (double)dn);
        R s[6];
#pragma unroll
        for (int c = 0; c < 6; c++) s[c] = v.S[c][k] + hd * (v.dS[c][k] + dsn[c]);
        const R Pk = v.P[k], Dk = v.D[k];
        const MatT<R>& m = v.mats[v.mat[k]];
        v.vx[k] = vx;
        v.vy[k] = vy;
        v.vz[k] = vz;
        if (u < 1e-12) u = 1e-12;
        v.u[k] = u;
        const R Y = yield_stress(m, Pk, Dk);
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
// The FP64 quotient is formed only where it can be the minimum: an FP32
// estimate (within 3e-7 of it) is reduced over the warp first, and only lanes
// within 1e-5 of the warp's smallest estimate -- which include the lane of the
// exact minimum -- divide in FP64 (warps that straddle two impacts: all lanes).
template <class R>
static __global__ void k_dt(View<R> v) {
    const unsigned full = 0xffffffffu;
    const int64_t k0 = gtid();
    const bool inb = k0 < v.n;
    const int64_t k = inb ? k0 : v.n - 1;
    const int ib = v.imp[k];
    ImpactD& I = v.imps[ib];
    const bool live = inb && I.mask;
    const float qf = live ? (float)v.hh[k] / ((float)v.csig[k] * (1.0f + (float)I.alpha) + 1e-30f) : INFINITY;
    const bool uniform = __all_sync(full, ib == __shfl_sync(full, ib, 0));
    const float qmin = __uint_as_float(__reduce_min_sync(full, __float_as_uint(qf)));  // qf >= 0
    const bool cand = live && (!uniform || !(qf > qmin * (1.0f + 1.0e-5f)));
    double d = 0.0;
    if (cand) d = I.cfl * (double)v.hh[k] / ((double)v.csig[k] * (1.0 + I.alpha) + 1e-30);
    block_atomic_ext<false>(&I.dt_bits, dbits(d), cand);
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
        if (I.max_steps > 0 && I.nsteps >= I.max_steps) { I.mask = 0; return; }
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

// Total entries of the current neighbour lists (own list + reverse extras,
// each clipped to its capacity): the list bytes every list consumer reads.
static __global__ void k_sum_list_entries(const int32_t* cnt, const int32_t* xcnt, int64_t n, int32_t cap,
                                   unsigned long long* out) {
    unsigned long long s = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (unsigned long long)min(cnt[i], cap) + (unsigned long long)min(xcnt[i], kExtraCap);
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

}  // namespace dsph
