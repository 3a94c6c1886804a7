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

namespace dsph {
void set_error_message(const std::string& m);
}

namespace deu {

using dsph::SphError;

// ---------------------------------------------------------------- materials

struct Mat {
    int32_t ideal;
    double gamma, rho0, a, b, A, B, alpha, beta, u0, uiv, ucv, G, Y, Emod, wm, wk;
};

// Settings + material + grid geometry, passed by value to every kernel.
struct P {
    Mat m;
    double gz, tdec, eta_af, c_act, p_coh, p_act, rho_cfl, damp, rho_vac;
    double y_i0, mu_i, mu_d, y_d0, y_m, y_bingham, c_reg, af_sat;
    int32_t axisym, rock, af_reg, af_prel, af_seeddp;
    int32_t nx, ny, nz;
    int64_t n;
    double dx, invdx;
    double eps_act;  // weakest-flaw activation strain, formed on the host as in hydro_cpu.cpp:254
};

__device__ __forceinline__ double dmax2(double a, double b) { return a < b ? b : a; }  // std::max
__device__ __forceinline__ double dmin2(double a, double b) { return b < a ? b : a; }  // std::min

// Tillotson pressure, eos.hpp:52-63.
__device__ double till(const Mat& m, double rho, double u) {
    if (rho <= 0) return 0.0;
    double eta = rho / m.rho0, mu = eta - 1.0;
    double w0 = u / (m.u0 * eta * eta) + 1.0;
    double Pc = (m.a + m.b / w0) * rho * u + m.A * mu + m.B * mu * mu;
    if (rho >= m.rho0 || u <= m.uiv) return Pc;
    double z = m.rho0 / rho - 1.0;
    double Pe = m.a * rho * u + (m.b * rho * u / w0 + m.A * mu * exp(-m.beta * z)) * exp(-m.alpha * z * z);
    if (u >= m.ucv) return Pe;
    return ((u - m.uiv) * Pe + (m.ucv - u) * Pc) / (m.ucv - m.uiv);
}

__device__ __forceinline__ double pressure(const Mat& m, double rho, double u) {  // eos.hpp:65-68
    if (m.ideal) return (m.gamma - 1.0) * rho * u;
    return till(m, rho, u);
}

// Condensed-branch value and analytic derivatives, eos.hpp:72-79.
__device__ void cond_d(const Mat& m, double rho, double u, double& P, double& dPdr, double& dPdu) {
    double eta = rho / m.rho0, mu = eta - 1.0;
    double w = 1.0 + u / (m.u0 * eta * eta), aob = m.a + m.b / w;
    P = aob * rho * u + m.A * mu + m.B * mu * mu;
    dPdu = aob * rho - m.b * rho * u / (w * w * m.u0 * eta * eta);
    double dwdr = -2.0 * u / (m.u0 * eta * eta * eta * m.rho0);
    dPdr = aob * u + rho * u * (-m.b / (w * w)) * dwdr + m.A / m.rho0 + 2.0 * m.B * mu / m.rho0;
}

// Expanded-branch value and analytic derivatives, eos.hpp:80-94.
__device__ void expd_d(const Mat& m, double rho, double u, double& P, double& dPdr, double& dPdu) {
    double eta = rho / m.rho0, mu = eta - 1.0;
    double w = 1.0 + u / (m.u0 * eta * eta);
    double z = m.rho0 / rho - 1.0, dzdr = -m.rho0 / (rho * rho);
    double E1 = exp(-m.alpha * z * z), E2 = exp(-m.beta * z);
    double G = m.b * rho * u / w + m.A * mu * E2;
    P = m.a * rho * u + G * E1;
    double dwdr = -2.0 * u / (m.u0 * eta * eta * eta * m.rho0);
    double dGu = m.b * rho / w - m.b * rho * u / (w * w * m.u0 * eta * eta);
    dPdu = m.a * rho + dGu * E1;
    double dbruw_dr = m.b * u / w + m.b * rho * u * (-1.0 / (w * w)) * dwdr;
    double dGr = dbruw_dr + m.A * E2 / m.rho0 + m.A * mu * (E2 * (-m.beta) * dzdr);
    double dE1dr = E1 * (-m.alpha * 2.0 * z) * dzdr;
    dPdr = m.a * u + dGr * E1 + G * dE1dr;
}

// Analytic sound speed, eos.hpp:95-113.
__device__ double sound_speed(const Mat& m, double rho, double u) {
    if (m.ideal) {
        double Pi = (m.gamma - 1.0) * rho * u;
        return sqrt(dmax2(m.gamma * Pi / dmax2(rho, 1e-30), 1e-12));
    }
    if (rho <= 0) return 1e-3;
    double Pp, dPdr, dPdu;
    if (rho >= m.rho0 || u <= m.uiv) {
        cond_d(m, rho, u, Pp, dPdr, dPdu);
    } else if (u >= m.ucv) {
        expd_d(m, rho, u, Pp, dPdr, dPdu);
    } else {
        double Pc, dPcr, dPcu, Pe, dPer, dPeu;
        cond_d(m, rho, u, Pc, dPcr, dPcu);
        expd_d(m, rho, u, Pe, dPer, dPeu);
        double inv = 1.0 / (m.ucv - m.uiv);
        Pp = ((u - m.uiv) * Pe + (m.ucv - u) * Pc) * inv;
        dPdu = ((Pe + (u - m.uiv) * dPeu) + (-Pc + (m.ucv - u) * dPcu)) * inv;
        dPdr = ((u - m.uiv) * dPer + (m.ucv - u) * dPcr) * inv;
    }
    return sqrt(dmax2(dPdr + Pp / (rho * rho) * dPdu, 1e-6));
}

// hydro_cpu.cpp:38: pressure clamped at 0 and the sound speed.
__device__ __forceinline__ void eos_pc(const Mat& m, double rho, double e, double& p, double& cs) {
    p = pressure(m, rho, e);
    if (p < 0) p = 0;
    cs = sound_speed(m, rho, e);
}

// ---------------------------------------------------------------- face flux

struct F5 {
    double r, mn, mt1, mt2, E;
};

__device__ __forceinline__ F5 flux_of(double r, double vn, double t1, double t2, double p, double E) {
    return F5{r * vn, r * vn * vn + p, r * vn * t1, r * vn * t2, (E + p) * vn};
}

// Exact rarefaction into vacuum sampled at the face, hydro_cpu.cpp:43-53.
__device__ F5 vac_flux(const Mat& m, double rM, double vnM, double t1M, double t2M, double eM, int side) {
    double pM, cM;
    eos_pc(m, rM, eM, pM, cM);
    double g = rM * cM * cM / dmax2(pM, 1e-30);
    if (g < 1.01) g = 1.01;
    if (g > 1e5) g = 1e5;
    double s = (double)side, vn = s * vnM;
    if (vn - cM >= 0) {
        double E = rM * eM + 0.5 * rM * (vnM * vnM + t1M * t1M + t2M * t2M);
        return F5{rM * vnM, rM * vnM * vnM + pM, rM * vnM * t1M, rM * vnM * t2M, (E + pM) * vnM};
    }
    if (vn + 2 * cM / (g - 1) <= 0) return F5{0, 0, 0, 0, 0};
    double u0 = 2.0 / (g + 1) * (cM + 0.5 * (g - 1) * vn), c0 = u0;
    double r0 = rM * pow(c0 / cM, 2.0 / (g - 1)), p0 = pM * pow(r0 / rM, g), e0 = p0 / ((g - 1) * r0), un0 = s * u0;
    double E0 = r0 * e0 + 0.5 * r0 * (un0 * un0 + t1M * t1M + t2M * t2M);
    return F5{r0 * un0, r0 * un0 * un0 + p0, r0 * un0 * t1M, r0 * un0 * t2M, (E0 + p0) * un0};
}

__device__ __forceinline__ F5 hllc_star(double r, double vn, double t1, double t2, double p, double E, double S,
                                        double Ss, F5 Fk) {
    double f = r * (S - vn) / (S - Ss);
    F5 Us{f, f * Ss, f * t1, f * t2, f * (E / r + (Ss - vn) * (Ss + p / (r * (S - vn))))};
    F5 U{r, r * vn, r * t1, r * t2, E};
    return F5{Fk.r + S * (Us.r - U.r), Fk.mn + S * (Us.mn - U.mn), Fk.mt1 + S * (Us.mt1 - U.mt1),
              Fk.mt2 + S * (Us.mt2 - U.mt2), Fk.E + S * (Us.E - U.E)};
}

// HLLC, hydro_cpu.cpp:54-74.
__device__ F5 hllc(const P& p, double rL, double vnL, double t1L, double t2L, double eL, double rR, double vnR,
                   double t1R, double t2R, double eR) {
    if (p.rho_vac > 0) {
        bool vL = rL < p.rho_vac, vR = rR < p.rho_vac;
        if (vL && vR) return F5{0, 0, 0, 0, 0};
        if (vR) return vac_flux(p.m, rL, vnL, t1L, t2L, eL, +1);
        if (vL) return vac_flux(p.m, rR, vnR, t1R, t2R, eR, -1);
    }
    double pL, cL, pR, cR;
    eos_pc(p.m, rL, eL, pL, cL);
    eos_pc(p.m, rR, eR, pR, cR);
    double SL = dmin2(vnL - cL, vnR - cR), SR = dmax2(vnL + cL, vnR + cR);
    double Ss = (pR - pL + rL * vnL * (SL - vnL) - rR * vnR * (SR - vnR)) / (rL * (SL - vnL) - rR * (SR - vnR));
    double EL = rL * eL + 0.5 * rL * (vnL * vnL + t1L * t1L + t2L * t2L),
           ER = rR * eR + 0.5 * rR * (vnR * vnR + t1R * t1R + t2R * t2R);
    if (SL >= 0) return flux_of(rL, vnL, t1L, t2L, pL, EL);
    if (SR <= 0) return flux_of(rR, vnR, t1R, t2R, pR, ER);
    if (Ss >= 0) return hllc_star(rL, vnL, t1L, t2L, pL, EL, SL, Ss, flux_of(rL, vnL, t1L, t2L, pL, EL));
    return hllc_star(rR, vnR, t1R, t2R, pR, ER, SR, Ss, flux_of(rR, vnR, t1R, t2R, pR, ER));
}

__device__ __forceinline__ double mm(double a, double b) {  // minmod, hydro_cpu.cpp:89
    return (a * b <= 0) ? 0.0 : (fabs(a) < fabs(b) ? a : b);
}

// ---------------------------------------------------------------- state

enum { F_R, F_MU, F_MV, F_MW, F_E, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ, F_D, F_AF, F_RC, F_VIB, F_PMAX, NF };
// Runge-Kutta fields (hydro_cpu.cpp:413-417) and the right-hand side, same order.
enum { D_R, D_MU, D_MV, D_MW, D_E, D_SXX, D_SYY, D_SZZ, D_SXY, D_SXZ, D_SYZ, D_D, D_RC, D_VIB, ND };
__host__ __device__ constexpr int rk_field(int q) {  // r .. Syz, D keep their index; rc, vib follow af
    return q <= D_D ? q : (q == D_RC ? F_RC : F_VIB);
}
static const char* kFieldNames[NF] = {"r", "mu", "mv", "mw", "E", "Sxx", "Syy", "Szz",
                                      "Sxy", "Sxz", "Syz", "D", "af", "rc", "vib", "Pmax"};
static const char* kRhsNames[ND] = {"r", "mu", "mv", "mw", "E", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz", "D", "rc", "vib"};

// One state of the grid: the 16 fields (a predictor state aliases af and Pmax
// of the state it was formed from).
struct Fields {
    double* q[NF];
};
struct Rhs {
    double* q[ND];
};
struct Prim {  // rho, vx, vy, vz, e, rc/rho
    double* w[6];
};
struct Faces {  // per direction: mass, normal / tangential momentum, energy, tracer fluxes
    double* q[3][6];
};

// Device-resident step control (the drivers' loop of hydro_cpu.cpp:452).
struct Ctl {
    double dt, t, t_end, cfl;
    int64_t steps, max_steps;
    int32_t active, pad;
    unsigned long long smax_bits;  // CFL speed of this step (positive doubles order as their bits)
};

__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }

// hydro_cpu.cpp:94-95
__device__ __forceinline__ double eint_of(double r, double mu, double mv, double mw, double E) {
    double ke = 0.5 * (mu * mu + mv * mv + mw * mw) / r;
    return (E - ke) / r;
}
__device__ __forceinline__ double pcell(const P& p, const Fields& s, int64_t c) {
    double pr, cs;
    const double r = s.q[F_R][c];
    eos_pc(p.m, r, eint_of(r, s.q[F_MU][c], s.q[F_MV][c], s.q[F_MW][c], s.q[F_E][c]), pr, cs);
    return pr;
}

// Acoustic fluidization of one cell, hydro_cpu.cpp:390-410.
__device__ void update_af_cell(const P& p, const Fields& g, int64_t c, double dt) {
    const double dec = exp(-dt / p.tdec);
    double* r = g.q[F_R];
    double* vib = g.q[F_VIB];
    double* Pmax = g.q[F_PMAX];
    const double e = eint_of(r[c], g.q[F_MU][c], g.q[F_MV][c], g.q[F_MW][c], g.q[F_E][c]);
    double Pc, cs;  // Pcell and MAT.sound_speed of the cell
    eos_pc(p.m, r[c], e, Pc, cs);
    if (Pc > Pmax[c]) {
        double dP = Pc - Pmax[c];
        Pmax[c] = Pc;
        if (dP > p.p_act) {
            double sp = p.af_seeddp ? dP / (dmax2(r[c], 1e-30) * dmax2(cs, 1e-30))
                                    : sqrt(g.q[F_MU][c] * g.q[F_MU][c] + g.q[F_MV][c] * g.q[F_MV][c] +
                                           g.q[F_MW][c] * g.q[F_MW][c]) / dmax2(r[c], 1e-30);
            vib[c] = dmax2(vib[c], p.c_act * sp);
        }
    }
    double v0 = vib[c];
    vib[c] *= dec;
    double pov = dmax2(Pc, p.p_coh);
    if (p.af_reg) {
        if (r[c] > dmax2(p.rho_cfl, 1e-12)) g.q[F_E][c] += 0.5 * r[c] * (v0 * v0 - vib[c] * vib[c]);
        double vcap = p.af_sat * pov / (dmax2(r[c], 1e-30) * dmax2(cs, 1e-30));
        if (vib[c] > vcap) vib[c] = vcap;
    }
    double pvib = r[c] * cs * vib[c];
    g.q[F_AF][c] = pvib / (pvib + pov);
}

// Radial return of one cell, hydro_cpu.cpp:229-252 (s: the stress / energy /
// vibration state; af from the state the step started from).
__device__ void vonmises_cell(const P& p, const Fields& s, const double* af, int64_t c, bool reg) {
    if (p.m.Y <= 0 && !p.rock) return;
    double Y;
    const double r = s.q[F_R][c];
    if (p.rock) {
        double Pp = dmax2(pcell(p, s, c), 0.0);
        double Peff = Pp;
        if (p.af_prel && s.q[F_VIB][c] > 0) {
            double p2, cs2;
            eos_pc(p.m, r, eint_of(r, s.q[F_MU][c], s.q[F_MV][c], s.q[F_MW][c], s.q[F_E][c]), p2, cs2);
            Peff = dmax2(Pp - r * cs2 * s.q[F_VIB][c], 0.0);
        }
        double Yi = p.y_i0 + p.mu_i * Peff / (1.0 + p.mu_i * Peff / dmax2(p.y_m - p.y_i0, 1.0));
        double Yd = dmin2(p.y_d0 + p.mu_d * Peff, p.y_m);
        const double D = s.q[F_D][c];
        double Yb = (1.0 - D) * Yi + D * Yd;
        Y = p.af_prel ? Yb : Yb * (1.0 - af[c]);
        if (p.y_bingham > 0 && af[c] > 1e-3) {
            double Yf = dmin2(p.y_bingham, Yb);
            if (Y < Yf) Y = Yf;
        }
    } else {
        Y = (1.0 - s.q[F_D][c]) * (1.0 - af[c]) * p.m.Y;
    }
    double sxx = s.q[F_SXX][c], syy = s.q[F_SYY][c], szz = s.q[F_SZZ][c], sxy = s.q[F_SXY][c], sxz = s.q[F_SXZ][c],
           syz = s.q[F_SYZ][c];
    double J2 = 0.5 * (sxx * sxx + syy * syy + szz * szz) + sxy * sxy + sxz * sxz + syz * syz;
    double vm = sqrt(3.0 * J2);
    if (vm > Y) {
        double f = (vm > 0 ? Y / vm : 0.0);
        s.q[F_SXX][c] = sxx * f; s.q[F_SYY][c] = syy * f; s.q[F_SZZ][c] = szz * f;
        s.q[F_SXY][c] = sxy * f; s.q[F_SXZ][c] = sxz * f; s.q[F_SYZ][c] = syz * f;
        if (p.af_reg && reg && p.m.G > 0 && (p.rho_cfl <= 0 || r > p.rho_cfl)) {
            double dW = (vm * vm - Y * Y) / (6.0 * p.m.G);
            s.q[F_VIB][c] = sqrt(s.q[F_VIB][c] * s.q[F_VIB][c] + 2.0 * p.c_reg * dW / r);
            s.q[F_E][c] -= p.c_reg * dW;
        }
    }
}

// Tensile damage growth of one cell, hydro_cpu.cpp:253-258.
__device__ void grow_damage_cell(const P& p, const Fields& g, int64_t c, double dt) {
    if (p.m.Emod <= 0 || p.m.wk <= 0) return;
    double* D = g.q[F_D];
    if (D[c] >= 1.0) return;
    double Pp = pcell(p, g, c);
    double sigmax = dmax2(-Pp + g.q[F_SXX][c], dmax2(-Pp + g.q[F_SYY][c], -Pp + g.q[F_SZZ][c]));
    if (sigmax > 0.0 && sigmax / p.m.Emod > p.eps_act) {
        double cg = 0.4 * sqrt(p.m.Emod / dmax2(g.q[F_R][c], 1e-30)), Rs = 0.5 * p.dx;
        double d13 = pow(D[c], 1.0 / 3.0) + (cg / Rs) * dt;
        D[c] = dmin2(1.0, d13 * d13 * d13);
    }
}

// ---------------------------------------------------------------- kernels

// Step start (drivers' loop): is there a step to take, and reset the speed.
static __global__ void k_begin(Ctl* ctl) {
    ctl->active = (ctl->t < ctl->t_end && (ctl->max_steps < 0 || ctl->steps < ctl->max_steps)) ? 1 : 0;
    ctl->smax_bits = (unsigned long long)__double_as_longlong(1e-30);
}

// maxspeed (hydro_cpu.cpp:378-380): per-cell signal speed, block maximum, one
// atomic per block on the ordered bits.
static __global__ void __launch_bounds__(256) k_maxspeed(P p, Fields g, Ctl* ctl) {
    __shared__ double red[8];
    const int64_t c = gtid();
    double s = 1e-30;
    if (ctl->active && c < p.n) {
        const double r = g.q[F_R][c];
        if (!(r < p.rho_cfl)) {
            const double mu = g.q[F_MU][c], mv = g.q[F_MV][c], mw = g.q[F_MW][c];
            double pr, cs;
            eos_pc(p.m, r, eint_of(r, mu, mv, mw, g.q[F_E][c]), pr, cs);
            double cel = sqrt(cs * cs + (p.m.G > 0 ? (4.0 / 3.0) * p.m.G / r : 0.0));
            double v = sqrt(mu * mu + mv * mv + mw * mw) / r;
            s = dmax2(s, v + cel);
        }
    }
    for (int o = 16; o > 0; o >>= 1) s = dmax2(s, __shfl_xor_sync(0xffffffffu, s, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 1e-30;
        for (int o = 16; o > 0; o >>= 1) s = dmax2(s, __shfl_xor_sync(0xffffffffu, s, o));
        if (threadIdx.x == 0) atomicMax(&ctl->smax_bits, (unsigned long long)__double_as_longlong(s));
    }
}

// dt = CFL dx / maxspeed, clipped at t_end (hydro_cpu.cpp:452).
static __global__ void k_dt(P p, Ctl* ctl) {
    if (!ctl->active) return;
    double dt = ctl->cfl * p.dx / __longlong_as_double((long long)ctl->smax_bits);
    if (ctl->t + dt > ctl->t_end) dt = ctl->t_end - ctl->t;
    ctl->dt = dt;
}

static __global__ void k_end(Ctl* ctl) {
    if (!ctl->active) return;
    ctl->t += ctl->dt;
    ctl->steps++;
}

// update_af before the stage (hydro_cpu.cpp:412).
static __global__ void k_update_af(P p, Fields g, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    update_af_cell(p, g, c, ctl->dt);
}

// Primitives of one state (hydro_cpu.cpp:101) and the tracer ratio rc/rho.
static __global__ void k_prim(P p, Fields s, Prim W, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const double r = s.q[F_R][c], mu = s.q[F_MU][c], mv = s.q[F_MV][c], mw = s.q[F_MW][c];
    const double E = s.q[F_E][c], rc = s.q[F_RC][c];
    W.w[0][c] = r;
    W.w[1][c] = mu / r;
    W.w[2][c] = mv / r;
    W.w[3][c] = mw / r;
    W.w[4][c] = eint_of(r, mu, mv, mw, E);
    W.w[5][c] = rc / r;
}

// Face geometry of direction DIR: number of faces and, for face id, the face
// position f along DIR and the cell of position p along DIR on its line.
template <int DIR>
struct FaceLine {
    int64_t base, stride;  // cell(p) = base + p * stride
    int f, nL;
    __device__ __forceinline__ FaceLine(const P& p, int64_t id) {
        if (DIR == 0) {
            const int64_t plane = (int64_t)p.ny * p.nz;
            f = (int)(id / plane);
            base = id - (int64_t)f * plane;
            stride = plane;
            nL = p.nx;
        } else if (DIR == 1) {
            const int64_t row = (int64_t)(p.ny + 1) * p.nz;
            const int64_t i = id / row, rem = id - i * row;
            f = (int)(rem / p.nz);
            base = i * (int64_t)p.ny * p.nz + (rem - (int64_t)f * p.nz);
            stride = p.nz;
            nL = p.ny;
        } else {
            const int64_t line = id / (p.nz + 1);
            f = (int)(id - line * (p.nz + 1));
            base = line * p.nz;
            stride = 1;
            nL = p.nz;
        }
    }
    __device__ __forceinline__ int64_t cell(int q) const { return base + (int64_t)q * stride; }
};

template <int DIR>
__host__ __device__ __forceinline__ int64_t face_count(int nx, int ny, int nz) {
    return DIR == 0 ? (int64_t)(nx + 1) * ny * nz : (DIR == 1 ? (int64_t)nx * (ny + 1) * nz : (int64_t)nx * ny * (nz + 1));
}

// Face fluxes of direction DIR (hydro_cpu.cpp:109-121): MUSCL-minmod
// reconstruction of the primitives, floors, HLLC / vacuum flux, tracer flux
// upwinded by the mass flux.
template <int DIR>
static __global__ void __launch_bounds__(256) k_face(P p, Prim W, Faces F, const Ctl* ctl) {
    const int64_t id = gtid();
    if (id >= face_count<DIR>(p.nx, p.ny, p.nz) || !ctl->active) return;
    const FaceLine<DIR> ln(p, id);
    const int f = ln.f, nL = ln.nL;
    const int iL = max(0, f - 1), iR = min(nL - 1, f), iLL = max(0, f - 2), iRR = min(nL - 1, f + 1);
    const int64_t cL = ln.cell(iL), cR = ln.cell(iR), cLL = ln.cell(iLL), cRR = ln.cell(iRR);
    double L[5], R[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
        const double* w = W.w[q];
        const double A = w[cL], B = w[cR], AA = w[cLL], BB = w[cRR];
        L[q] = A + 0.5 * mm(A - AA, B - A);
        R[q] = B - 0.5 * mm(B - A, BB - B);
        if (q == 0) {
            if (L[0] < 1e-9) L[0] = A;
            if (R[0] < 1e-9) R[0] = B;
        }
        if (q == 4) {
            if (L[4] < 0) L[4] = A;
            if (R[4] < 0) R[4] = B;
        }
    }
    constexpr int in = DIR == 0 ? 1 : (DIR == 1 ? 2 : 3), it1 = DIR == 0 ? 2 : 1, it2 = DIR == 2 ? 2 : 3;
    const F5 fl = hllc(p, L[0], L[in], L[it1], L[it2], L[4], R[0], R[in], R[it1], R[it2], R[4]);
    F.q[DIR][0][id] = fl.r;
    F.q[DIR][1][id] = fl.mn;
    F.q[DIR][2][id] = fl.mt1;
    F.q[DIR][3][id] = fl.mt2;
    F.q[DIR][4][id] = fl.E;
    F.q[DIR][5][id] = fl.r * (fl.r >= 0.0 ? W.w[5][cL] : W.w[5][cR]);
}

// Right-hand side of one cell (hydro_cpu.cpp:98-214): the three directions'
// flux differences in the reference's order, gravity, strength sources.
// s: the state Lop reads; W: its primitives (k_prim), whose velocities mu/rho
// are the very quotients the reference forms for every neighbour it reads;
// af: the fluidization ratio.
static __global__ void __launch_bounds__(128, 3) k_rhs(P p, Fields s, Prim W, const double* af, Faces F, Rhs d,
                                                   const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const int64_t plane = (int64_t)p.ny * p.nz;
    const int i = (int)(c / plane);
    const int64_t rem = c - (int64_t)i * plane;
    const int j = (int)(rem / p.nz), k = (int)(rem - (int64_t)j * p.nz);
    const double* r = s.q[F_R];
    const double* mu = s.q[F_MU];
    const double* mv = s.q[F_MV];
    const double* mw = s.q[F_MW];
    double dr = 0.0, dE = 0.0, drc = 0.0, dmu = 0.0, dmv = 0.0, dmw = 0.0;
    // ---- hydro sweeps (hydro_cpu.cpp:122-133), x then y then z
    {
        const int64_t lo[3] = {c, ((int64_t)i * (p.ny + 1) + j) * p.nz + k, ((int64_t)i * p.ny + j) * (p.nz + 1) + k};
        const int64_t up[3] = {(int64_t)p.ny * p.nz, p.nz, 1};
#pragma unroll
        for (int dir = 0; dir < 3; dir++) {
            const int64_t a = lo[dir], b = lo[dir] + up[dir];
            const double* const* Fq = F.q[dir];
            double vr, vE, vrc, dmn, dt1, dt2;
            if (dir == 0 && p.axisym) {
                const double w0 = i * p.dx, w1 = (i + 1) * p.dx, inv = 1.0 / (((i + 0.5) * p.dx) * p.dx);
                vr = -(w1 * Fq[0][b] - w0 * Fq[0][a]) * inv;
                vE = -(w1 * Fq[4][b] - w0 * Fq[4][a]) * inv;
                vrc = -(w1 * Fq[5][b] - w0 * Fq[5][a]) * inv;
                dmn = -(w1 * Fq[1][b] - w0 * Fq[1][a]) * inv;
                dt1 = -(w1 * Fq[2][b] - w0 * Fq[2][a]) * inv;
                dt2 = -(w1 * Fq[3][b] - w0 * Fq[3][a]) * inv;
                double pr, cs;
                eos_pc(p.m, r[c], W.w[4][c], pr, cs);  // Pcell: EOS at the cell's internal energy
                dmn += pr / ((i + 0.5) * p.dx);
            } else {  // face weights 1 (exact products)
                const double inv = p.invdx;
                vr = -(Fq[0][b] - Fq[0][a]) * inv;
                vE = -(Fq[4][b] - Fq[4][a]) * inv;
                vrc = -(Fq[5][b] - Fq[5][a]) * inv;
                dmn = -(Fq[1][b] - Fq[1][a]) * inv;
                dt1 = -(Fq[2][b] - Fq[2][a]) * inv;
                dt2 = -(Fq[3][b] - Fq[3][a]) * inv;
            }
            dr += vr;
            dE += vE;
            drc += vrc;
            if (dir == 0) {
                dmu += dmn; dmv += dt1; dmw += dt2;
            } else if (dir == 1) {
                dmv += dmn; dmu += dt1; dmw += dt2;
            } else {
                dmw += dmn; dmu += dt1; dmv += dt2;
            }
        }
    }
    if (p.gz != 0.0) {  // plain gravity body force, hydro_cpu.cpp:137-138
        dmw += -p.gz * r[c];
        dE += -p.gz * mw[c];
    }
    double dS[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, dD = 0.0, dvib = 0.0;
    if (p.m.G > 0 && !(p.rho_cfl > 0 && r[c] < p.rho_cfl)) {  // strength sources, hydro_cpu.cpp:145-213
        const double G = p.m.G, dx = p.dx;
        const int64_t xm = c - (i > 0 ? plane : 0), xp = c + (i < p.nx - 1 ? plane : 0);
        const int64_t ym = c - (j > 0 ? p.nz : 0), yp = c + (j < p.ny - 1 ? p.nz : 0);
        const int64_t zm = c - (k > 0 ? 1 : 0), zp = c + (k < p.nz - 1 ? 1 : 0);
        const double hx = ((i > 0 && i < p.nx - 1) ? 2.0 : 1.0) * dx, hy = ((j > 0 && j < p.ny - 1) ? 2.0 : 1.0) * dx,
                     hz = ((k > 0 && k < p.nz - 1) ? 2.0 : 1.0) * dx;
        const double* Vx = W.w[1];  // mu / rho of every cell
        const double* Vy = W.w[2];
        const double* Vz = W.w[3];
        const double vxc = Vx[c], vyc = Vy[c], vzc = Vz[c];
        const bool vd = p.rho_cfl > 0;
        auto vxw = [&](int64_t q) { return (vd && r[q] < p.rho_cfl) ? vxc : Vx[q]; };
        auto vyw = [&](int64_t q) { return (vd && r[q] < p.rho_cfl) ? vyc : Vy[q]; };
        auto vzw = [&](int64_t q) { return (vd && r[q] < p.rho_cfl) ? vzc : Vz[q]; };
        const double Lxx = (vxw(xp) - vxw(xm)) / hx, Lxy = (vxw(yp) - vxw(ym)) / hy, Lxz = (vxw(zp) - vxw(zm)) / hz;
        const double Lyx = (vyw(xp) - vyw(xm)) / hx, Lyy = (vyw(yp) - vyw(ym)) / hy, Lyz = (vyw(zp) - vyw(zm)) / hz;
        const double Lzx = (vzw(xp) - vzw(xm)) / hx, Lzy = (vzw(yp) - vzw(ym)) / hy, Lzz = (vzw(zp) - vzw(zm)) / hz;
        const double rcyl = (i + 0.5) * dx;
        const double eyy = p.axisym ? (vxc / rcyl) : Lyy;
        const double exx = Lxx, ezz = Lzz, exy = 0.5 * (Lxy + Lyx), exz = 0.5 * (Lxz + Lzx), eyz = 0.5 * (Lyz + Lzy),
                     tr = (exx + eyy + ezz) / 3.0;
        const double Wxy = 0.5 * (Lxy - Lyx), Wxz = 0.5 * (Lxz - Lzx), Wyz = 0.5 * (Lyz - Lzy);
        const double* Sxx = s.q[F_SXX];
        const double* Syy = s.q[F_SYY];
        const double* Szz = s.q[F_SZZ];
        const double* Sxy = s.q[F_SXY];
        const double* Sxz = s.q[F_SXZ];
        const double* Syz = s.q[F_SYZ];
        const double sxx = Sxx[c], syy = Syy[c], szz = Szz[c], sxy = Sxy[c], sxz = Sxz[c], syz = Syz[c];
        const double Sm[3][3] = {{sxx, sxy, sxz}, {sxy, syy, syz}, {sxz, syz, szz}};
        const double Wm[3][3] = {{0, Wxy, Wxz}, {-Wxy, 0, Wyz}, {-Wxz, -Wyz, 0}};
        double Jm[3][3];
#pragma unroll
        for (int aa = 0; aa < 3; aa++)
#pragma unroll
            for (int bb = 0; bb < 3; bb++) {  // (S.W - W.S), hydro_cpu.cpp:172-173
                double t = 0;
#pragma unroll
                for (int cc = 0; cc < 3; cc++) t += Sm[aa][cc] * Wm[cc][bb] - Wm[aa][cc] * Sm[cc][bb];
                Jm[aa][bb] = t;
            }
        const double u = vxc, v = vyc, w = vzc;
        const double ix_ = i > 0 ? dx : 1e30, ixp = i < p.nx - 1 ? dx : 1e30;
        const double iy_ = j > 0 ? dx : 1e30, iyp = j < p.ny - 1 ? dx : 1e30;
        const double iz_ = k > 0 ? dx : 1e30, izp = k < p.nz - 1 ? dx : 1e30;
        auto adv = [&](const double* S) {  // upwind v . grad S, hydro_cpu.cpp:175-178
            double ax = u > 0 ? (S[c] - S[xm]) / ix_ : (S[xp] - S[c]) / ixp;
            double ay = v > 0 ? (S[c] - S[ym]) / iy_ : (S[yp] - S[c]) / iyp;
            double az = w > 0 ? (S[c] - S[zm]) / iz_ : (S[zp] - S[c]) / izp;
            return u * ax + v * ay + w * az;
        };
        dS[0] = 0.0 + (2 * G * (exx - tr) + Jm[0][0] - adv(Sxx));
        dS[1] = 0.0 + (2 * G * (eyy - tr) + Jm[1][1] - adv(Syy));
        dS[2] = 0.0 + (2 * G * (ezz - tr) + Jm[2][2] - adv(Szz));
        dS[3] = 0.0 + (2 * G * exy + Jm[0][1] - adv(Sxy));
        dS[4] = 0.0 + (2 * G * exz + Jm[0][2] - adv(Sxz));
        dS[5] = 0.0 + (2 * G * eyz + Jm[1][2] - adv(Syz));
        dD = 0.0 + (-adv(s.q[F_D]));
        dvib = 0.0 + (-adv(s.q[F_VIB]));
        // div S into momentum (central differences), hydro_cpu.cpp:183-186
        const double dSxx_x = (Sxx[xp] - Sxx[xm]) / hx, dSxy_y = (Sxy[yp] - Sxy[ym]) / hy, dSxz_z = (Sxz[zp] - Sxz[zm]) / hz;
        const double dSxy_x = (Sxy[xp] - Sxy[xm]) / hx, dSyy_y = (Syy[yp] - Syy[ym]) / hy, dSyz_z = (Syz[zp] - Syz[zm]) / hz;
        const double dSxz_x = (Sxz[xp] - Sxz[xm]) / hx, dSyz_y = (Syz[yp] - Syz[ym]) / hy, dSzz_z = (Szz[zp] - Szz[zm]) / hz;
        dmu += dSxx_x + dSxy_y + dSxz_z;
        dmv += dSxy_x + dSyy_y + dSyz_z;
        dmw += dSxz_x + dSyz_y + dSzz_z;
        if (p.axisym) {
            dmu += (sxx - syy) / rcyl;
            dmw += sxz / rcyl;
        }
        if (af[c] > 0 && p.eta_af > 0) {  // explicit fluidization viscosity, hydro_cpu.cpp:190-197
            const double eta = af[c] * p.eta_af, id2 = 1.0 / (dx * dx);
            auto vx = [&](int64_t q) { return Vx[q]; };
            auto vy = [&](int64_t q) { return Vy[q]; };
            auto vz = [&](int64_t q) { return Vz[q]; };
            dmu += eta * (vx(xp) + vx(xm) + vx(yp) + vx(ym) + vx(zp) + vx(zm) - 6 * vx(c)) * id2;
            dmv += eta * (vy(xp) + vy(xm) + vy(yp) + vy(ym) + vy(zp) + vy(zm) - 6 * vy(c)) * id2;
            dmw += eta * (vz(xp) + vz(xm) + vz(yp) + vz(ym) + vz(zp) + vz(zm) - 6 * vz(c)) * id2;
            if (p.axisym) {
                dmu += eta * (Lxx / rcyl - vxc / (rcyl * rcyl));
                dmw += eta * (Lzx / rcyl);
            }
        }
        // div(S.v) into energy, hydro_cpu.cpp:198-203
        auto svx = [&](int64_t q) { return Sxx[q] * Vx[q] + Sxy[q] * Vy[q] + Sxz[q] * Vz[q]; };
        auto svy = [&](int64_t q) { return Sxy[q] * Vx[q] + Syy[q] * Vy[q] + Syz[q] * Vz[q]; };
        auto svz = [&](int64_t q) { return Sxz[q] * Vx[q] + Syz[q] * Vy[q] + Szz[q] * Vz[q]; };
        dE += (svx(xp) - svx(xm)) / hx + (svy(yp) - svy(ym)) / hy + (svz(zp) - svz(zm)) / hz;
        if (p.axisym) dE += svx(c) / rcyl;
    }
    d.q[D_R][c] = dr;
    d.q[D_MU][c] = dmu;
    d.q[D_MV][c] = dmv;
    d.q[D_MW][c] = dmw;
    d.q[D_E][c] = dE;
#pragma unroll
    for (int q = 0; q < 6; q++) d.q[D_SXX + q][c] = dS[q];
    d.q[D_D][c] = dD;
    d.q[D_RC][c] = drc;
    d.q[D_VIB][c] = dvib;
}

// Predictor (hydro_cpu.cpp:413-418): g1 = g + dt d, void-cell reset, radial
// return without regeneration.
static __global__ void k_predict(P p, Fields g, Fields g1, Rhs d, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const double dt = ctl->dt;
#pragma unroll
    for (int q = 0; q < ND; q++) g1.q[rk_field(q)][c] = g.q[rk_field(q)][c] + dt * d.q[q][c];
    if (p.rho_cfl > 0 && g1.q[F_R][c] < p.rho_cfl) g1.q[F_MU][c] = g1.q[F_MV][c] = g1.q[F_MW][c] = 0;
    vonmises_cell(p, g1, g.q[F_AF], c, false);
}

// Corrector and the end of the step (hydro_cpu.cpp:419-424): trapezoidal
// average, damage growth, radial return, damping, void-cell reset.
static __global__ void k_correct(P p, Fields g, Fields g1, Rhs d, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const double dt = ctl->dt;
#pragma unroll
    for (int q = 0; q < ND; q++) {
        double* x = g.q[rk_field(q)];
        x[c] = 0.5 * (x[c] + g1.q[rk_field(q)][c] + dt * d.q[q][c]);
    }
    grow_damage_cell(p, g, c, dt);
    vonmises_cell(p, g, g.q[F_AF], c, true);
    if (p.damp < 1.0) {
        g.q[F_MU][c] *= p.damp;
        g.q[F_MV][c] *= p.damp;
        g.q[F_MW][c] *= p.damp;
    }
    if (p.rho_cfl > 0 && g.q[F_R][c] < p.rho_cfl) g.q[F_MU][c] = g.q[F_MV][c] = g.q[F_MW][c] = 0;
}

// Single operators for the C ABI's unit calls.
static __global__ void k_vonmises(P p, Fields g, int reg) {
    const int64_t c = gtid();
    if (c < p.n) vonmises_cell(p, g, g.q[F_AF], c, reg != 0);
}
static __global__ void k_grow_damage(P p, Fields g, double dt) {
    const int64_t c = gtid();
    if (c < p.n) grow_damage_cell(p, g, c, dt);
}
static __global__ void k_pressure(P p, Fields g, double* out) {
    const int64_t c = gtid();
    if (c < p.n) out[c] = pcell(p, g, c);
}

static __global__ void k_set_step(Ctl* ctl, double dt) {  // a step at a host dt
    ctl->dt = dt;
    ctl->active = 1;
}
static __global__ void k_set_run(Ctl* ctl, double cfl, double t_end, int64_t max_steps) {
    ctl->cfl = cfl;
    ctl->t_end = t_end;
    ctl->max_steps = max_steps < 0 ? -1 : ctl->steps + max_steps;
}
static __global__ void k_set_time(Ctl* ctl, double t) { ctl->t = t; }
static __global__ void k_maxspeed_begin(Ctl* ctl) {
    ctl->active = 1;
    ctl->smax_bits = (unsigned long long)__double_as_longlong(1e-30);
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
    Prim W{};
    Faces F{};
    Ctl* ctl = nullptr;
    double* scratch = nullptr;  // pressure read-out
    std::vector<void*> allocs;
    int64_t bytes = 0;
    int64_t launches = 0;
    cudaEvent_t ev[8] = {};
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;

    double* alloc(int64_t count) {
        void* ptr = nullptr;
        const size_t b = sizeof(double) * (size_t)std::max<int64_t>(count, 1);
        cudaError_t e = cudaMalloc(&ptr, b);
        if (e != cudaSuccess) throw SphError(SPH_ERR_NOMEM, std::string("device allocation failed: ") + cudaGetErrorString(e));
        allocs.push_back(ptr);
        bytes += (int64_t)b;
        EU_CUDA(cudaMemsetAsync(ptr, 0, b, st));
        return (double*)ptr;
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
        const int64_t n = p.n;
        k_prim<<<grid_of(n), 256, 0, st>>>(p, s, W, ctl);
        k_face<0><<<grid_of(face_count<0>(p.nx, p.ny, p.nz)), 256, 0, st>>>(p, W, F, ctl);
        k_face<1><<<grid_of(face_count<1>(p.nx, p.ny, p.nz)), 256, 0, st>>>(p, W, F, ctl);
        k_face<2><<<grid_of(face_count<2>(p.nx, p.ny, p.nz)), 256, 0, st>>>(p, W, F, ctl);
        k_rhs<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(p, s, W, g.q[F_AF], F, d, ctl);
        launches += 5;
    }

    // One step_rk2 (hydro_cpu.cpp:411-425); with_dt: the drivers' dt and stop
    // test on the device first.
    void enqueue_step(bool with_dt) {
        const int64_t n = p.n;
        if (with_dt) {
            k_begin<<<1, 1, 0, st>>>(ctl);
            k_maxspeed<<<grid_of(n), 256, 0, st>>>(p, g, ctl);
            k_dt<<<1, 1, 0, st>>>(p, ctl);
            launches += 3;
        }
        if (p.c_act > 0 && p.tdec > 0) {
            k_update_af<<<grid_of(n), 256, 0, st>>>(p, g, ctl);
            launches++;
        }
        enqueue_lop(g);
        k_predict<<<grid_of(n), 256, 0, st>>>(p, g, g1, d, ctl);
        enqueue_lop(g1);
        k_correct<<<grid_of(n), 256, 0, st>>>(p, g, g1, d, ctl);
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
    return guard([&] {
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
            for (int q = 0; q < 6; q++) g->W.w[q] = g->alloc(n);
            const int64_t nfc[3] = {deu::face_count<0>(nx, ny, nz), deu::face_count<1>(nx, ny, nz),
                                    deu::face_count<2>(nx, ny, nz)};
            for (int dir = 0; dir < 3; dir++)
                for (int q = 0; q < 6; q++) g->F.q[dir][q] = g->alloc(nfc[dir]);
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
        to_params(g->p, *e);
        g->graph_valid = false;
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
        deu::k_maxspeed<<<g->grid_of(g->p.n), 256, 0, g->st>>>(g->p, g->g, g->ctl);
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
        const int64_t per_step = 16 + ((g->p.c_act > 0 && g->p.tdec > 0) ? 1 : 0);
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
