// euler_kernels.cuh -- device code of the Eulerian grid hydrocode (the
// reference's hydrocodes/euler/hydro_cpu.cpp), shared by the two precision
// forms:
//   plain (FP64, euler.cu, compiled without fused multiply-adds): every
//     expression in the reference's operation order;
//   mixed (euler_mixed.cu): primitives, face fluxes, the right-hand side's
//     sources, the yield surface, damage growth and the CFL speed in FP32 (the
//     arithmetic of the reference's own GPU solver); the state and its
//     Runge-Kutta updates, the fluidization update and dt in FP64.
// The compute type R is the template parameter; state and right-hand side
// are always FP64.  Literals are written as R(...) so that an
// FP32 instantiation never promotes to FP64.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace deu {

// ---------------------------------------------------------------- materials

template <class R>
struct MatT {
    int32_t ideal;
    R gamma, rho0, a, b, A, B, alpha, beta, u0, uiv, ucv, G, Y, Emod, wm, wk;
};
using Mat = MatT<double>;

template <class R>
__host__ __device__ __forceinline__ MatT<R> mat_as(const Mat& m) {
    return MatT<R>{m.ideal, R(m.gamma), R(m.rho0), R(m.a), R(m.b), R(m.A), R(m.B), R(m.alpha), R(m.beta),
                   R(m.u0), R(m.uiv), R(m.ucv), R(m.G), R(m.Y), R(m.Emod), R(m.wm), R(m.wk)};
}

// Settings + material + grid geometry, passed by value to every kernel.
struct P {
    Mat m;
    MatT<float> mf;  // the material rounded to FP32 once on the host (for the FP32 form)
    // settings the FP32 form reads, rounded to FP32 once on the host (ymi: y_m - y_i0)
    struct {
        float y_i0, mu_i, ymi, y_d0, mu_d, y_m, y_bingham, c_reg, eps_act, dx, invdx, rho_vac;
    } cf;
    double gz, tdec, eta_af, c_act, p_coh, p_act, rho_cfl, damp, rho_vac;
    double y_i0, mu_i, mu_d, y_d0, y_m, y_bingham, c_reg, af_sat;
    int32_t axisym, rock, af_reg, af_prel, af_seeddp;
    int32_t nx, ny, nz;
    int64_t n;
    double dx, invdx;
    double eps_act;  // weakest-flaw activation strain, formed on the host as in hydro_cpu.cpp:254
    // hydrostatic reference of set_ref (hydro_cpu.cpp:259-261), null when off:
    // the well-balanced z-sweep and gravity source and the void-cell reset
    const double* ref_r0;
    const double* ref_p0;
    const double* ref_dp;  // per cell p0(top face) - p0(bottom face) of the well-balanced gravity source
    double void_amb;  // VOID_AMB: void cells reset to this density instead of the reference's
    int32_t void_cons;  // VOID_CONS: the reset moves the excess mass to a neighbour first
    int32_t visc_imp;   // VISC_IMP: fluidization viscosity by the implicit solve, not in the Lop
};

// The material in the compute type R: FP64 as given, FP32 as rounded once on
// the host (the same values a per-thread conversion gives, without the
// per-thread conversions, which run on the FP64 pipe).
template <class R>
__device__ __forceinline__ MatT<R> mat_of(const P& p) {
    if constexpr (sizeof(R) == 4) return p.mf;
    else return p.m;
}

// A setting in the compute type R: FP64 as given, FP32 as rounded on the host.
#define EU_SETTING(R, name) (sizeof(R) == 4 ? R(p.cf.name) : R(p.name))

// x in the compute type R (FP64: x itself) and back to FP64.  (Conversions by
// integer operations instead of the hardware's were tried: bit-identical, but
// the 256^3 mixed step went from 14.9 to 16.2 ms -- the conversions are not
// what keeps the FP64 pipe busy; the FP64 state arithmetic is.)
template <class R>
__device__ __forceinline__ R narrow(double x) {
    return R(x);
}
__device__ __forceinline__ double widen(float y) { return (double)y; }
__device__ __forceinline__ double widen(double y) { return y; }

template <class R> __device__ __forceinline__ R dmax2(R a, R b) { return a < b ? b : a; }  // std::max
template <class R> __device__ __forceinline__ R dmin2(R a, R b) { return b < a ? b : a; }  // std::min

// Tillotson pressure, eos.hpp:52-63.
template <class R>
__device__ R till(const MatT<R>& m, R rho, R u) {
    if (rho <= R(0)) return R(0);
    R eta = rho / m.rho0, mu = eta - R(1);
    R w0 = u / (m.u0 * eta * eta) + R(1);
    R Pc = (m.a + m.b / w0) * rho * u + m.A * mu + m.B * mu * mu;
    if (rho >= m.rho0 || u <= m.uiv) return Pc;
    R z = m.rho0 / rho - R(1);
    R Pe = m.a * rho * u + (m.b * rho * u / w0 + m.A * mu * exp(-m.beta * z)) * exp(-m.alpha * z * z);
    if (u >= m.ucv) return Pe;
    return ((u - m.uiv) * Pe + (m.ucv - u) * Pc) / (m.ucv - m.uiv);
}

template <class R>
__device__ __forceinline__ R pressure(const MatT<R>& m, R rho, R u) {  // eos.hpp:65-68
    if (m.ideal) return (m.gamma - R(1)) * rho * u;
    return till(m, rho, u);
}

// Condensed-branch value and analytic derivatives, eos.hpp:72-79.
template <class R>
__device__ void cond_d(const MatT<R>& m, R rho, R u, R& P, R& dPdr, R& dPdu) {
    R eta = rho / m.rho0, mu = eta - R(1);
    R w = R(1) + u / (m.u0 * eta * eta), aob = m.a + m.b / w;
    P = aob * rho * u + m.A * mu + m.B * mu * mu;
    dPdu = aob * rho - m.b * rho * u / (w * w * m.u0 * eta * eta);
    R dwdr = R(-2) * u / (m.u0 * eta * eta * eta * m.rho0);
    dPdr = aob * u + rho * u * (-m.b / (w * w)) * dwdr + m.A / m.rho0 + R(2) * m.B * mu / m.rho0;
}

// Expanded-branch value and analytic derivatives, eos.hpp:80-94.
template <class R>
__device__ void expd_d(const MatT<R>& m, R rho, R u, R& P, R& dPdr, R& dPdu) {
    R eta = rho / m.rho0, mu = eta - R(1);
    R w = R(1) + u / (m.u0 * eta * eta);
    R z = m.rho0 / rho - R(1), dzdr = -m.rho0 / (rho * rho);
    R E1 = exp(-m.alpha * z * z), E2 = exp(-m.beta * z);
    R G = m.b * rho * u / w + m.A * mu * E2;
    P = m.a * rho * u + G * E1;
    R dwdr = R(-2) * u / (m.u0 * eta * eta * eta * m.rho0);
    R dGu = m.b * rho / w - m.b * rho * u / (w * w * m.u0 * eta * eta);
    dPdu = m.a * rho + dGu * E1;
    R dbruw_dr = m.b * u / w + m.b * rho * u * (R(-1) / (w * w)) * dwdr;
    R dGr = dbruw_dr + m.A * E2 / m.rho0 + m.A * mu * (E2 * (-m.beta) * dzdr);
    R dE1dr = E1 * (-m.alpha * R(2) * z) * dzdr;
    dPdr = m.a * u + dGr * E1 + G * dE1dr;
}

// Analytic sound speed, eos.hpp:95-113.
template <class R>
__device__ R sound_speed(const MatT<R>& m, R rho, R u) {
    if (m.ideal) {
        R Pi = (m.gamma - R(1)) * rho * u;
        return sqrt(dmax2(m.gamma * Pi / dmax2(rho, R(1e-30)), R(1e-12)));
    }
    if (rho <= R(0)) return R(1e-3);
    R Pp, dPdr, dPdu;
    if (rho >= m.rho0 || u <= m.uiv) {
        cond_d(m, rho, u, Pp, dPdr, dPdu);
    } else if (u >= m.ucv) {
        expd_d(m, rho, u, Pp, dPdr, dPdu);
    } else {
        R Pc, dPcr, dPcu, Pe, dPer, dPeu;
        cond_d(m, rho, u, Pc, dPcr, dPcu);
        expd_d(m, rho, u, Pe, dPer, dPeu);
        R inv = R(1) / (m.ucv - m.uiv);
        Pp = ((u - m.uiv) * Pe + (m.ucv - u) * Pc) * inv;
        dPdu = ((Pe + (u - m.uiv) * dPeu) + (-Pc + (m.ucv - u) * dPcu)) * inv;
        dPdr = ((u - m.uiv) * dPer + (m.ucv - u) * dPcr) * inv;
    }
    return sqrt(dmax2(dPdr + Pp / (rho * rho) * dPdu, R(1e-6)));
}

// hydro_cpu.cpp:38: pressure clamped at 0 and the sound speed.
template <class R>
__device__ __forceinline__ void eos_pc(const MatT<R>& m, R rho, R e, R& p, R& cs) {
    p = pressure(m, rho, e);
    if (p < R(0)) p = R(0);
    cs = sound_speed(m, rho, e);
}

// ---------------------------------------------------------------- face flux

template <class R>
struct F5 {
    R r, mn, mt1, mt2, E;
};

template <class R>
__device__ __forceinline__ F5<R> flux_of(R r, R vn, R t1, R t2, R p, R E) {
    return F5<R>{r * vn, r * vn * vn + p, r * vn * t1, r * vn * t2, (E + p) * vn};
}

// Exact rarefaction into vacuum sampled at the face, hydro_cpu.cpp:43-53.
template <class R>
__device__ F5<R> vac_flux(const MatT<R>& m, R rM, R vnM, R t1M, R t2M, R eM, int side) {
    R pM, cM;
    eos_pc(m, rM, eM, pM, cM);
    R g = rM * cM * cM / dmax2(pM, R(1e-30));
    if (g < R(1.01)) g = R(1.01);
    if (g > R(1e5)) g = R(1e5);
    R s = (R)side, vn = s * vnM;
    if (vn - cM >= R(0)) {
        R E = rM * eM + R(0.5) * rM * (vnM * vnM + t1M * t1M + t2M * t2M);
        return F5<R>{rM * vnM, rM * vnM * vnM + pM, rM * vnM * t1M, rM * vnM * t2M, (E + pM) * vnM};
    }
    if (vn + R(2) * cM / (g - R(1)) <= R(0)) return F5<R>{R(0), R(0), R(0), R(0), R(0)};
    R u0 = R(2) / (g + R(1)) * (cM + R(0.5) * (g - R(1)) * vn), c0 = u0;
    R r0 = rM * pow(c0 / cM, R(2) / (g - R(1))), p0 = pM * pow(r0 / rM, g), e0 = p0 / ((g - R(1)) * r0),
      un0 = s * u0;
    R E0 = r0 * e0 + R(0.5) * r0 * (un0 * un0 + t1M * t1M + t2M * t2M);
    return F5<R>{r0 * un0, r0 * un0 * un0 + p0, r0 * un0 * t1M, r0 * un0 * t2M, (E0 + p0) * un0};
}

template <class R>
__device__ __forceinline__ F5<R> hllc_star(R r, R vn, R t1, R t2, R p, R E, R S, R Ss, F5<R> Fk) {
    R f = r * (S - vn) / (S - Ss);
    F5<R> Us{f, f * Ss, f * t1, f * t2, f * (E / r + (Ss - vn) * (Ss + p / (r * (S - vn))))};
    F5<R> U{r, r * vn, r * t1, r * t2, E};
    return F5<R>{Fk.r + S * (Us.r - U.r), Fk.mn + S * (Us.mn - U.mn), Fk.mt1 + S * (Us.mt1 - U.mt1),
                 Fk.mt2 + S * (Us.mt2 - U.mt2), Fk.E + S * (Us.E - U.E)};
}

// HLLC, hydro_cpu.cpp:54-74.
template <class R>
__device__ F5<R> hllc(const MatT<R>& m, R rho_vac, R rL, R vnL, R t1L, R t2L, R eL, R rR, R vnR, R t1R, R t2R,
                      R eR) {
    if (rho_vac > R(0)) {
        bool vL = rL < rho_vac, vR = rR < rho_vac;
        if (vL && vR) return F5<R>{R(0), R(0), R(0), R(0), R(0)};
        if (vR) return vac_flux(m, rL, vnL, t1L, t2L, eL, +1);
        if (vL) return vac_flux(m, rR, vnR, t1R, t2R, eR, -1);
    }
    R pL, cL, pR, cR;
    eos_pc(m, rL, eL, pL, cL);
    eos_pc(m, rR, eR, pR, cR);
    R SL = dmin2(vnL - cL, vnR - cR), SR = dmax2(vnL + cL, vnR + cR);
    R Ss = (pR - pL + rL * vnL * (SL - vnL) - rR * vnR * (SR - vnR)) / (rL * (SL - vnL) - rR * (SR - vnR));
    R EL = rL * eL + R(0.5) * rL * (vnL * vnL + t1L * t1L + t2L * t2L),
      ER = rR * eR + R(0.5) * rR * (vnR * vnR + t1R * t1R + t2R * t2R);
    if (SL >= R(0)) return flux_of(rL, vnL, t1L, t2L, pL, EL);
    if (SR <= R(0)) return flux_of(rR, vnR, t1R, t2R, pR, ER);
    if (Ss >= R(0)) return hllc_star(rL, vnL, t1L, t2L, pL, EL, SL, Ss, flux_of(rL, vnL, t1L, t2L, pL, EL));
    return hllc_star(rR, vnR, t1R, t2R, pR, ER, SR, Ss, flux_of(rR, vnR, t1R, t2R, pR, ER));
}

// HLLC with the face pressures given (the well-balanced z-sweep), hydro_cpu.cpp:75-88.
template <class R>
__device__ F5<R> hllc_p(const MatT<R>& m, R rL, R vnL, R t1L, R t2L, R eL, R pL, R rR, R vnR, R t1R, R t2R, R eR,
                        R pR) {
    R cL = sound_speed(m, rL, eL), cR = sound_speed(m, rR, eR);
    if (pL < R(0)) pL = R(0);
    if (pR < R(0)) pR = R(0);
    R SL = dmin2(vnL - cL, vnR - cR), SR = dmax2(vnL + cL, vnR + cR);
    R Ss = (pR - pL + rL * vnL * (SL - vnL) - rR * vnR * (SR - vnR)) / (rL * (SL - vnL) - rR * (SR - vnR));
    R EL = rL * eL + R(0.5) * rL * (vnL * vnL + t1L * t1L + t2L * t2L),
      ER = rR * eR + R(0.5) * rR * (vnR * vnR + t1R * t1R + t2R * t2R);
    if (SL >= R(0)) return flux_of(rL, vnL, t1L, t2L, pL, EL);
    if (SR <= R(0)) return flux_of(rR, vnR, t1R, t2R, pR, ER);
    if (Ss >= R(0)) return hllc_star(rL, vnL, t1L, t2L, pL, EL, SL, Ss, flux_of(rL, vnL, t1L, t2L, pL, EL));
    return hllc_star(rR, vnR, t1R, t2R, pR, ER, SR, Ss, flux_of(rR, vnR, t1R, t2R, pR, ER));
}

template <class R>
__device__ __forceinline__ R mm(R a, R b) {  // minmod, hydro_cpu.cpp:89
    return (a * b <= R(0)) ? R(0) : (fabs(a) < fabs(b) ? a : b);
}

// ---------------------------------------------------------------- state

enum { F_R, F_MU, F_MV, F_MW, F_E, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ, F_D, F_AF, F_RC, F_VIB, F_PMAX, NF };
// Runge-Kutta fields (hydro_cpu.cpp:413-417) and the right-hand side, same order.
enum { D_R, D_MU, D_MV, D_MW, D_E, D_SXX, D_SYY, D_SZZ, D_SXY, D_SXZ, D_SYZ, D_D, D_RC, D_VIB, ND };
__host__ __device__ constexpr int rk_field(int q) {  // r .. Syz, D keep their index; rc, vib follow af
    return q <= D_D ? q : (q == D_RC ? F_RC : F_VIB);
}
inline const char* const kFieldNames[NF] = {"r", "mu", "mv", "mw", "E", "Sxx", "Syy", "Szz",
                                      "Sxy", "Sxz", "Syz", "D", "af", "rc", "vib", "Pmax"};
inline const char* const kRhsNames[ND] = {"r", "mu", "mv", "mw", "E", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz", "D", "rc", "vib"};

// One state of the grid: the 16 fields (a predictor state aliases af and Pmax
// of the state it was formed from).
struct Fields {
    double* q[NF];
};
struct Rhs {
    double* q[ND];
};
template <class R>
struct PrimT {  // rho, vx, vy, vz, e, rc/rho in the Lop's compute type, and (with a
    R* w[7];    // reference state) the pressure deviation Pcell - REF_P0 formed in FP64
    // Sxx Syy Szz Sxy Sxz Syz D vib as the right-hand side reads them: in FP64
    // the state's own arrays; in FP32 copies converted once per Lop by k_prim
    // (the same values the conversion at every stencil read gave)
    R* sq[8];
    uint8_t* vd;  // FP32 form: near-void flag per cell (rho < RHO_CFL), formed in FP64
};
template <class R>
struct FacesT {  // per direction: mass, normal / tangential momentum, energy, tracer fluxes
    R* q[3][6];
};

// Device-resident step control (the drivers' loop of hydro_cpu.cpp:452).
struct Ctl {
    double dt, t, t_end, cfl;
    int64_t steps, max_steps;
    int32_t active, pad;
    unsigned long long smax_bits;  // CFL speed of this step (positive doubles order as their bits)
    // implicit viscosity: grid barrier of its persistent launch, a wait that
    // ran out (error), conjugate-gradient iterations so far
    unsigned int bar_count;
    int32_t visc_err;  // bar_count and visc_err are cleared together before each launch
    unsigned int bar_gen;
    int32_t pad2;
    long long visc_iters;
};

static __device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }

// hydro_cpu.cpp:94-95
static __device__ __forceinline__ double eint_of(double r, double mu, double mv, double mw, double E) {
    double ke = 0.5 * (mu * mu + mv * mv + mw * mw) / r;
    return (E - ke) / r;
}
static __device__ __forceinline__ double pcell(const P& p, const Fields& s, int64_t c) {
    double pr, cs;
    const double r = s.q[F_R][c];
    eos_pc(p.m, r, eint_of(r, s.q[F_MU][c], s.q[F_MV][c], s.q[F_MW][c], s.q[F_E][c]), pr, cs);
    return pr;
}

// Acoustic fluidization of one cell, hydro_cpu.cpp:390-410.
static __device__ void update_af_cell(const P& p, const Fields& g, int64_t c, double dt) {
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

// Specific internal energy for an EOS evaluated in R: FP64, the reference's
// two quotients (eint_of); FP32, one FP64 reciprocal of rho (E - ke cancels in
// kinetic-dominated cells, so the difference stays FP64), the result rounded
// to FP32 by the caller.
template <class R>
static __device__ __forceinline__ double eint_r(double r, double mu, double mv, double mw, double E) {
    if constexpr (sizeof(R) == 8) {
        return eint_of(r, mu, mv, mw, E);
    } else {
        const double inv = 1.0 / r;
        return (E - 0.5 * (mu * mu + mv * mv + mw * mw) * inv) * inv;
    }
}

// Pcell (hydro_cpu.cpp:95) with the EOS evaluated in R: the clamped pressure.
template <class R>
static __device__ __forceinline__ double pcell_r(const P& p, const Fields& s, int64_t c) {
    const double r = s.q[F_R][c];
    R pr = pressure(mat_of<R>(p), narrow<R>(r),
                    narrow<R>(eint_r<R>(r, s.q[F_MU][c], s.q[F_MV][c], s.q[F_MW][c], s.q[F_E][c])));
    if (pr < R(0)) pr = R(0);
    return widen(pr);
}

// A cell's Pcell formed at most once per state and shared by the damage
// growth and the radial return that follow each other in a stage (damage
// growth changes only D, so both see the same pressure).
template <class R>
struct PcellOnce {
    bool have = false;
    double v = 0.0;
    __device__ __forceinline__ double get(const P& p, const Fields& s, int64_t c) {
        if (!have) {
            v = pcell_r<R>(p, s, c);
            have = true;
        }
        return v;
    }
};

// Radial return of one cell, hydro_cpu.cpp:229-252 (s: the stress / energy /
// vibration state; af from the state the step started from).  The yield
// surface and the return factor are formed in R; the state stays FP64.
template <class R>
static __device__ void vonmises_cell(const P& p, const Fields& s, const double* af, int64_t c, bool reg,
                                     PcellOnce<R>& pc) {
    if (p.m.Y <= 0 && !p.rock) return;
    R Y;
    const double r = s.q[F_R][c];
    const R afc = narrow<R>(af[c]);
    if (p.rock) {
        R Pp = R(dmax2(pc.get(p, s, c), 0.0));
        R Peff = Pp;
        if (p.af_prel && s.q[F_VIB][c] > 0) {
            R p2, cs2;
            eos_pc(mat_of<R>(p), narrow<R>(r),
                   narrow<R>(eint_r<R>(r, s.q[F_MU][c], s.q[F_MV][c], s.q[F_MW][c], s.q[F_E][c])), p2, cs2);
            Peff = dmax2(Pp - narrow<R>(r) * cs2 * narrow<R>(s.q[F_VIB][c]), R(0));
        }
        const R mu_i = EU_SETTING(R, mu_i);
        const R ymi = sizeof(R) == 4 ? R(p.cf.ymi) : R(p.y_m - p.y_i0);
        R Yi = EU_SETTING(R, y_i0) + mu_i * Peff / (R(1) + mu_i * Peff / dmax2(ymi, R(1)));
        R Yd = dmin2(EU_SETTING(R, y_d0) + EU_SETTING(R, mu_d) * Peff, EU_SETTING(R, y_m));
        const R D = narrow<R>(s.q[F_D][c]);
        R Yb = (R(1) - D) * Yi + D * Yd;
        Y = p.af_prel ? Yb : Yb * (R(1) - afc);
        if (p.y_bingham > 0 && afc > R(1e-3)) {
            R Yf = dmin2(EU_SETTING(R, y_bingham), Yb);
            if (Y < Yf) Y = Yf;
        }
    } else {
        Y = (R(1) - narrow<R>(s.q[F_D][c])) * (R(1) - afc) * mat_of<R>(p).Y;
    }
    const double sxx = s.q[F_SXX][c], syy = s.q[F_SYY][c], szz = s.q[F_SZZ][c], sxy = s.q[F_SXY][c],
                 sxz = s.q[F_SXZ][c], syz = s.q[F_SYZ][c];
    const R xx = narrow<R>(sxx), yy = narrow<R>(syy), zz = narrow<R>(szz), xy = narrow<R>(sxy),
            xz = narrow<R>(sxz), yz = narrow<R>(syz);
    R J2 = R(0.5) * (xx * xx + yy * yy + zz * zz) + xy * xy + xz * xz + yz * yz;
    R vm = sqrt(R(3) * J2);
    if (vm > Y) {
        const double f = widen(vm > R(0) ? Y / vm : R(0));
        s.q[F_SXX][c] = sxx * f; s.q[F_SYY][c] = syy * f; s.q[F_SZZ][c] = szz * f;
        s.q[F_SXY][c] = sxy * f; s.q[F_SXZ][c] = sxz * f; s.q[F_SYZ][c] = syz * f;
        if (p.af_reg && reg && p.m.G > 0 && (p.rho_cfl <= 0 || r > p.rho_cfl)) {
            R dW = (vm * vm - Y * Y) / (R(6) * mat_of<R>(p).G);
            const R vb = narrow<R>(s.q[F_VIB][c]);
            s.q[F_VIB][c] = widen(sqrt(vb * vb + R(2) * EU_SETTING(R, c_reg) * dW / narrow<R>(r)));
            s.q[F_E][c] -= widen(EU_SETTING(R, c_reg) * dW);
        }
    }
}

// Tensile damage growth of one cell, hydro_cpu.cpp:253-258 (threshold and
// growth formed in R).
template <class R>
static __device__ void grow_damage_cell(const P& p, const Fields& g, int64_t c, double dt, PcellOnce<R>& pc) {
    if (p.m.Emod <= 0 || p.m.wk <= 0) return;
    double* D = g.q[F_D];
    if (D[c] >= 1.0) return;
    const R Pp = R(pc.get(p, g, c));
    const R sigmax = dmax2(-Pp + narrow<R>(g.q[F_SXX][c]),
                           dmax2(-Pp + narrow<R>(g.q[F_SYY][c]), -Pp + narrow<R>(g.q[F_SZZ][c])));
    if (sigmax > R(0) && sigmax / mat_of<R>(p).Emod > EU_SETTING(R, eps_act)) {
        R cg = R(0.4) * sqrt(mat_of<R>(p).Emod / dmax2(narrow<R>(g.q[F_R][c]), R(1e-30))),
          Rs = R(0.5) * EU_SETTING(R, dx);
        R d13 = pow(narrow<R>(D[c]), R(1) / R(3)) + (cg / Rs) * R(dt);
        D[c] = widen(dmin2(R(1), d13 * d13 * d13));
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
template <class R>
static __global__ void __launch_bounds__(256) k_maxspeed(P p, Fields g, Ctl* ctl) {
    __shared__ double red[8];
    const int64_t c = gtid();
    double s = 1e-30;
    if (ctl->active && c < p.n) {
        const double r = g.q[F_R][c];
        if (!(r < p.rho_cfl)) {
            const double mu = g.q[F_MU][c], mv = g.q[F_MV][c], mw = g.q[F_MW][c];
            const R rr = narrow<R>(r);
            R pr, cs;
            eos_pc(mat_of<R>(p), rr, narrow<R>(eint_r<R>(r, mu, mv, mw, g.q[F_E][c])), pr, cs);
            R cel = sqrt(cs * cs + (p.m.G > 0 ? R(4.0 / 3.0) * mat_of<R>(p).G / rr : R(0)));
            const R fu = narrow<R>(mu), fv = narrow<R>(mv), fw = narrow<R>(mw);
            R v = sqrt(fu * fu + fv * fv + fw * fw) / rr;
            s = dmax2(s, widen(v + cel));
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

// Primitives of one state (hydro_cpu.cpp:101) and the tracer ratio rc/rho,
// formed in FP64 and stored in the Lop's compute type R.  FP64: the
// reference's quotients, one division each.  FP32: one FP64 reciprocal of
// rho, the velocities, kinetic energy and internal energy from it in FP64
// (E - ke cancels in kinetic-dominated cells), rounded to FP32; also the
// strength fields in FP32 and the near-void flags for the right-hand side.
template <class R>
static __global__ void k_prim(P p, Fields s, PrimT<R> W, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const double r = s.q[F_R][c], mu = s.q[F_MU][c], mv = s.q[F_MV][c], mw = s.q[F_MW][c];
    const double E = s.q[F_E][c], rc = s.q[F_RC][c];
    if constexpr (sizeof(R) == 4) {
        const double inv = 1.0 / r, vx = mu * inv, vy = mv * inv, vz = mw * inv;
        const double e = (E - 0.5 * (mu * vx + mv * vy + mw * vz)) * inv;
        W.w[0][c] = narrow<R>(r);
        W.w[1][c] = narrow<R>(vx);
        W.w[2][c] = narrow<R>(vy);
        W.w[3][c] = narrow<R>(vz);
        W.w[4][c] = narrow<R>(e);
        W.w[5][c] = narrow<R>(rc * inv);
        if (p.ref_p0) {
            double pr = pressure(p.m, r, e);
            if (pr < 0) pr = 0;
            W.w[6][c] = narrow<R>(pr - p.ref_p0[c]);
        }
#pragma unroll
        for (int q = 0; q < 6; q++) W.sq[q][c] = narrow<R>(s.q[F_SXX + q][c]);
        W.sq[6][c] = narrow<R>(s.q[F_D][c]);
        W.sq[7][c] = narrow<R>(s.q[F_VIB][c]);
        W.vd[c] = (p.rho_cfl > 0 && r < p.rho_cfl) ? 1 : 0;
        return;
    }
    W.w[0][c] = R(r);
    W.w[1][c] = R(mu / r);
    W.w[2][c] = R(mv / r);
    W.w[3][c] = R(mw / r);
    const double e = eint_of(r, mu, mv, mw, E);
    W.w[4][c] = R(e);
    W.w[5][c] = R(rc / r);
    if (p.ref_p0) {  // Pcell - REF_P0 (hydro_cpu.cpp:116)
        double pr = pressure(p.m, r, e);
        if (pr < 0) pr = 0;
        W.w[6][c] = R(pr - p.ref_p0[c]);
    }
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
template <int DIR, class R>
static __global__ void __launch_bounds__(256) k_face(P p, PrimT<R> W, FacesT<R> F, const Ctl* ctl) {
    const int64_t id = gtid();
    if (id >= face_count<DIR>(p.nx, p.ny, p.nz) || !ctl->active) return;
    const FaceLine<DIR> ln(p, id);
    const int f = ln.f, nL = ln.nL;
    const int iL = max(0, f - 1), iR = min(nL - 1, f), iLL = max(0, f - 2), iRR = min(nL - 1, f + 1);
    const int64_t cL = ln.cell(iL), cR = ln.cell(iR), cLL = ln.cell(iLL), cRR = ln.cell(iRR);
    R L[5], Rr[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
        const R* w = W.w[q];
        const R A = w[cL], B = w[cR], AA = w[cLL], BB = w[cRR];
        L[q] = A + R(0.5) * mm(A - AA, B - A);
        Rr[q] = B - R(0.5) * mm(B - A, BB - B);
        if (q == 0) {
            if (L[0] < R(1e-9)) L[0] = A;
            if (Rr[0] < R(1e-9)) Rr[0] = B;
        }
        if (q == 4) {
            if (L[4] < R(0)) L[4] = A;
            if (Rr[4] < R(0)) Rr[4] = B;
        }
    }
    constexpr int in = DIR == 0 ? 1 : (DIR == 1 ? 2 : 3), it1 = DIR == 0 ? 2 : 1, it2 = DIR == 2 ? 2 : 3;
    const MatT<R> m = mat_of<R>(p);
    F5<R> fl;
    if (DIR == 2 && p.ref_p0) {  // well-balanced: reconstruct the deviation from the reference (hydro_cpu.cpp:114-119)
        const R* dv = W.w[6];
        const R dLL = dv[cLL], dL = dv[cL], dR = dv[cR], dRR = dv[cRR];
        const R dLf = dL + R(0.5) * mm(dL - dLL, dR - dL), dRf = dR - R(0.5) * mm(dR - dL, dRR - dR);
        double p0f = pressure(p.m, 0.5 * (p.ref_r0[cL] + p.ref_r0[cR]), 0.0);
        if (p0f < 0) p0f = 0;
        fl = hllc_p(m, L[0], L[in], L[it1], L[it2], L[4], R(p0f) + dLf, Rr[0], Rr[in], Rr[it1], Rr[it2], Rr[4],
                    R(p0f) + dRf);
    } else {
        fl = hllc(m, EU_SETTING(R, rho_vac), L[0], L[in], L[it1], L[it2], L[4], Rr[0], Rr[in], Rr[it1], Rr[it2], Rr[4]);
    }
    F.q[DIR][0][id] = fl.r;
    F.q[DIR][1][id] = fl.mn;
    F.q[DIR][2][id] = fl.mt1;
    F.q[DIR][3][id] = fl.mt2;
    F.q[DIR][4][id] = fl.E;
    F.q[DIR][5][id] = fl.r * (fl.r >= R(0) ? W.w[5][cL] : W.w[5][cR]);
}

// Right-hand side of one cell (hydro_cpu.cpp:98-214): the three directions'
// flux differences in the reference's order, gravity, strength sources.
// s: the state Lop reads; W: its primitives (k_prim), whose velocities mu/rho
// are the very quotients the reference forms for every neighbour it reads;
// af: the fluidization ratio.  Flux differences and strength sources are
// formed in R and added to the FP64 right-hand side (with R = double: every
// operation of the reference, in its order).
// Resident blocks per SM asked of the right-hand side (launch bounds) in the
// FP32 form; the FP64 form keeps 3.  The FP32 form waits on neighbour loads at
// low occupancy: 256^3 impact, mixed step 16.2 / 15.3 / 15.0 ms at 5 / 7 / 8
// blocks (80 / 72 / 64 registers, with spills to L1).
#ifndef DEU_RHS_MINB_F32
#define DEU_RHS_MINB_F32 8
#endif
template <class R>
static __global__ void __launch_bounds__(128, sizeof(R) == 4 ? DEU_RHS_MINB_F32 : 3)
    k_rhs(P p, Fields s, PrimT<R> W, const double* af, FacesT<R> F, Rhs d, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const int64_t plane = (int64_t)p.ny * p.nz;
    const int i = (int)(c / plane);
    const int64_t rem = c - (int64_t)i * plane;
    const int j = (int)(rem / p.nz), k = (int)(rem - (int64_t)j * p.nz);
    const double* r = s.q[F_R];
    const double* mw = s.q[F_MW];
    // Sums of the right-hand side: FP64 in the FP64 form (the reference's
    // additions); in the FP32 form the terms are FP32 already and are summed
    // in FP32 (in the same order) and widened once at the store.
    using A = R;
    A dr = A(0), dE = A(0), drc = A(0), dmu = A(0), dmv = A(0), dmw = A(0);
    // ---- hydro sweeps (hydro_cpu.cpp:122-133), x then y then z
    {
        const int64_t lo[3] = {c, ((int64_t)i * (p.ny + 1) + j) * p.nz + k, ((int64_t)i * p.ny + j) * (p.nz + 1) + k};
        const int64_t up[3] = {(int64_t)p.ny * p.nz, p.nz, 1};
#pragma unroll
        for (int dir = 0; dir < 3; dir++) {
            const int64_t a = lo[dir], b = lo[dir] + up[dir];
            const R* const* Fq = F.q[dir];
            R vr, vE, vrc, dmn, dt1, dt2;
            if (dir == 0 && p.axisym) {
                const R w0 = R(i * p.dx), w1 = R((i + 1) * p.dx), inv = R(1.0 / (((i + 0.5) * p.dx) * p.dx));
                vr = -(w1 * Fq[0][b] - w0 * Fq[0][a]) * inv;
                vE = -(w1 * Fq[4][b] - w0 * Fq[4][a]) * inv;
                vrc = -(w1 * Fq[5][b] - w0 * Fq[5][a]) * inv;
                dmn = -(w1 * Fq[1][b] - w0 * Fq[1][a]) * inv;
                dt1 = -(w1 * Fq[2][b] - w0 * Fq[2][a]) * inv;
                dt2 = -(w1 * Fq[3][b] - w0 * Fq[3][a]) * inv;
                R pr, cs;
                eos_pc(mat_of<R>(p), W.w[0][c], W.w[4][c], pr, cs);  // Pcell: EOS at the cell's internal energy
                dmn += pr / R((i + 0.5) * p.dx);
            } else {  // face weights 1 (exact products)
                const R inv = EU_SETTING(R, invdx);
                vr = -(Fq[0][b] - Fq[0][a]) * inv;
                vE = -(Fq[4][b] - Fq[4][a]) * inv;
                vrc = -(Fq[5][b] - Fq[5][a]) * inv;
                dmn = -(Fq[1][b] - Fq[1][a]) * inv;
                dt1 = -(Fq[2][b] - Fq[2][a]) * inv;
                dt2 = -(Fq[3][b] - Fq[3][a]) * inv;
            }
            dr += A(vr);
            dE += A(vE);
            drc += A(vrc);
            if (dir == 0) {
                dmu += A(dmn); dmv += A(dt1); dmw += A(dt2);
            } else if (dir == 1) {
                dmv += A(dmn); dmu += A(dt1); dmw += A(dt2);
            } else {
                dmw += A(dmn); dmu += A(dt1); dmv += A(dt2);
            }
        }
    }
    if (p.gz != 0.0) {
        if (!p.ref_r0) {  // plain gravity body force, hydro_cpu.cpp:137-138
            dmw += narrow<A>(-p.gz * r[c]);
            dE += narrow<A>(-p.gz * mw[c]);
        } else {  // well-balanced source against the reference, hydro_cpu.cpp:139-143
            const double* R0 = p.ref_r0;
            dmw += narrow<A>(-p.gz * (r[c] - R0[c]) + p.ref_dp[c] * p.invdx);  // ref_dp: k_ref_dp
            dE += narrow<A>(-p.gz * mw[c]);
        }
    }
    A dS[6] = {A(0), A(0), A(0), A(0), A(0), A(0)}, dD = A(0), dvib = A(0);
    // near-void cell (rho < RHO_CFL): the FP32 form reads k_prim's flags
    auto is_void = [&](int64_t q) -> bool {
        if constexpr (sizeof(R) == 4) return W.vd[q] != 0;
        else return p.rho_cfl > 0 && r[q] < p.rho_cfl;
    };
    if (p.m.G > 0 && !is_void(c)) {  // strength sources, hydro_cpu.cpp:145-213
        const R G = mat_of<R>(p).G, dx = EU_SETTING(R, dx);
        const int64_t xm = c - (i > 0 ? plane : 0), xp = c + (i < p.nx - 1 ? plane : 0);
        const int64_t ym = c - (j > 0 ? p.nz : 0), yp = c + (j < p.ny - 1 ? p.nz : 0);
        const int64_t zm = c - (k > 0 ? 1 : 0), zp = c + (k < p.nz - 1 ? 1 : 0);
        const R hx = ((i > 0 && i < p.nx - 1) ? R(2) : R(1)) * dx, hy = ((j > 0 && j < p.ny - 1) ? R(2) : R(1)) * dx,
                hz = ((k > 0 && k < p.nz - 1) ? R(2) : R(1)) * dx;
        const R* Vx = W.w[1];  // mu / rho of every cell
        const R* Vy = W.w[2];
        const R* Vz = W.w[3];
        const R vxc = Vx[c], vyc = Vy[c], vzc = Vz[c];
        auto vxw = [&](int64_t q) { return is_void(q) ? vxc : Vx[q]; };
        auto vyw = [&](int64_t q) { return is_void(q) ? vyc : Vy[q]; };
        auto vzw = [&](int64_t q) { return is_void(q) ? vzc : Vz[q]; };
        const R Lxx = (vxw(xp) - vxw(xm)) / hx, Lxy = (vxw(yp) - vxw(ym)) / hy, Lxz = (vxw(zp) - vxw(zm)) / hz;
        const R Lyx = (vyw(xp) - vyw(xm)) / hx, Lyy = (vyw(yp) - vyw(ym)) / hy, Lyz = (vyw(zp) - vyw(zm)) / hz;
        const R Lzx = (vzw(xp) - vzw(xm)) / hx, Lzy = (vzw(yp) - vzw(ym)) / hy, Lzz = (vzw(zp) - vzw(zm)) / hz;
        const R rcyl = R((i + 0.5) * p.dx);
        const R eyy = p.axisym ? (vxc / rcyl) : Lyy;
        const R exx = Lxx, ezz = Lzz, exy = R(0.5) * (Lxy + Lyx), exz = R(0.5) * (Lxz + Lzx),
                eyz = R(0.5) * (Lyz + Lzy), tr = (exx + eyy + ezz) / R(3);
        const R Wxy = R(0.5) * (Lxy - Lyx), Wxz = R(0.5) * (Lxz - Lzx), Wyz = R(0.5) * (Lyz - Lzy);
        const R* Sxx = W.sq[0];
        const R* Syy = W.sq[1];
        const R* Szz = W.sq[2];
        const R* Sxy = W.sq[3];
        const R* Sxz = W.sq[4];
        const R* Syz = W.sq[5];
        const R sxx = R(Sxx[c]), syy = R(Syy[c]), szz = R(Szz[c]), sxy = R(Sxy[c]), sxz = R(Sxz[c]), syz = R(Syz[c]);
        const R Sm[3][3] = {{sxx, sxy, sxz}, {sxy, syy, syz}, {sxz, syz, szz}};
        const R Wm[3][3] = {{R(0), Wxy, Wxz}, {-Wxy, R(0), Wyz}, {-Wxz, -Wyz, R(0)}};
        R Jm[3][3];
#pragma unroll
        for (int aa = 0; aa < 3; aa++)
#pragma unroll
            for (int bb = 0; bb < 3; bb++) {  // (S.W - W.S), hydro_cpu.cpp:172-173
                R t = R(0);
#pragma unroll
                for (int cc = 0; cc < 3; cc++) t += Sm[aa][cc] * Wm[cc][bb] - Wm[aa][cc] * Sm[cc][bb];
                Jm[aa][bb] = t;
            }
        const R u = vxc, v = vyc, w = vzc;
        const R ix_ = i > 0 ? dx : R(1e30), ixp = i < p.nx - 1 ? dx : R(1e30);
        const R iy_ = j > 0 ? dx : R(1e30), iyp = j < p.ny - 1 ? dx : R(1e30);
        const R iz_ = k > 0 ? dx : R(1e30), izp = k < p.nz - 1 ? dx : R(1e30);
        auto adv = [&](const R* S) {  // upwind v . grad S, hydro_cpu.cpp:175-178
            const R sc = R(S[c]);
            R ax = u > R(0) ? (sc - R(S[xm])) / ix_ : (R(S[xp]) - sc) / ixp;
            R ay = v > R(0) ? (sc - R(S[ym])) / iy_ : (R(S[yp]) - sc) / iyp;
            R az = w > R(0) ? (sc - R(S[zm])) / iz_ : (R(S[zp]) - sc) / izp;
            return u * ax + v * ay + w * az;
        };
        dS[0] = A(0) + A(R(2) * G * (exx - tr) + Jm[0][0] - adv(Sxx));
        dS[1] = A(0) + A(R(2) * G * (eyy - tr) + Jm[1][1] - adv(Syy));
        dS[2] = A(0) + A(R(2) * G * (ezz - tr) + Jm[2][2] - adv(Szz));
        dS[3] = A(0) + A(R(2) * G * exy + Jm[0][1] - adv(Sxy));
        dS[4] = A(0) + A(R(2) * G * exz + Jm[0][2] - adv(Sxz));
        dS[5] = A(0) + A(R(2) * G * eyz + Jm[1][2] - adv(Syz));
        dD = A(0) + A(-adv(W.sq[6]));
        dvib = A(0) + A(-adv(W.sq[7]));
        // div S into momentum (central differences), hydro_cpu.cpp:183-186
        auto cd = [&](const R* S, int64_t q1, int64_t q0, R h) { return (R(S[q1]) - R(S[q0])) / h; };
        const R dSxx_x = cd(Sxx, xp, xm, hx), dSxy_y = cd(Sxy, yp, ym, hy), dSxz_z = cd(Sxz, zp, zm, hz);
        const R dSxy_x = cd(Sxy, xp, xm, hx), dSyy_y = cd(Syy, yp, ym, hy), dSyz_z = cd(Syz, zp, zm, hz);
        const R dSxz_x = cd(Sxz, xp, xm, hx), dSyz_y = cd(Syz, yp, ym, hy), dSzz_z = cd(Szz, zp, zm, hz);
        dmu += A(dSxx_x + dSxy_y + dSxz_z);
        dmv += A(dSxy_x + dSyy_y + dSyz_z);
        dmw += A(dSxz_x + dSyz_y + dSzz_z);
        if (p.axisym) {
            dmu += A((sxx - syy) / rcyl);
            dmw += A(sxz / rcyl);
        }
        if (af[c] > 0 && p.eta_af > 0 && !p.visc_imp) {  // explicit fluidization viscosity, hydro_cpu.cpp:190-197
            const R eta = R(af[c] * p.eta_af), id2 = R(1.0 / (p.dx * p.dx));
            auto vx = [&](int64_t q) { return Vx[q]; };
            auto vy = [&](int64_t q) { return Vy[q]; };
            auto vz = [&](int64_t q) { return Vz[q]; };
            dmu += A(eta * (vx(xp) + vx(xm) + vx(yp) + vx(ym) + vx(zp) + vx(zm) - R(6) * vx(c)) * id2);
            dmv += A(eta * (vy(xp) + vy(xm) + vy(yp) + vy(ym) + vy(zp) + vy(zm) - R(6) * vy(c)) * id2);
            dmw += A(eta * (vz(xp) + vz(xm) + vz(yp) + vz(ym) + vz(zp) + vz(zm) - R(6) * vz(c)) * id2);
            if (p.axisym) {
                dmu += A(eta * (Lxx / rcyl - vxc / (rcyl * rcyl)));
                dmw += A(eta * (Lzx / rcyl));
            }
        }
        // div(S.v) into energy, hydro_cpu.cpp:198-203
        auto svx = [&](int64_t q) { return R(Sxx[q]) * Vx[q] + R(Sxy[q]) * Vy[q] + R(Sxz[q]) * Vz[q]; };
        auto svy = [&](int64_t q) { return R(Sxy[q]) * Vx[q] + R(Syy[q]) * Vy[q] + R(Syz[q]) * Vz[q]; };
        auto svz = [&](int64_t q) { return R(Sxz[q]) * Vx[q] + R(Syz[q]) * Vy[q] + R(Szz[q]) * Vz[q]; };
        dE += A((svx(xp) - svx(xm)) / hx + (svy(yp) - svy(ym)) / hy + (svz(zp) - svz(zm)) / hz);
        if (p.axisym) dE += A(svx(c) / rcyl);
    }
    d.q[D_R][c] = widen(dr);
    d.q[D_MU][c] = widen(dmu);
    d.q[D_MV][c] = widen(dmv);
    d.q[D_MW][c] = widen(dmw);
    d.q[D_E][c] = widen(dE);
#pragma unroll
    for (int q = 0; q < 6; q++) d.q[D_SXX + q][c] = widen(dS[q]);
    d.q[D_D][c] = widen(dD);
    d.q[D_RC][c] = widen(drc);
    d.q[D_VIB][c] = widen(dvib);
}

// Near-void cell: momentum zeroed; with a reference state also reset to the
// reference (or ambient) density with no energy, stress or tracer,
// hydro_cpu.cpp:272-290 (not the conservative transfer).
static __device__ __forceinline__ void void_cell(const P& p, const Fields& g, int64_t c) {
    if (!(p.rho_cfl > 0 && g.q[F_R][c] < p.rho_cfl)) return;
    if (p.void_cons && p.ref_r0) return;  // the serial conservative pass (k_void_cons) does it
    g.q[F_MU][c] = g.q[F_MV][c] = g.q[F_MW][c] = 0;
    if (p.ref_r0) {
        g.q[F_R][c] = (p.void_amb > 0 ? p.void_amb : p.ref_r0[c]);
        g.q[F_E][c] = 0;
        g.q[F_SXX][c] = g.q[F_SYY][c] = g.q[F_SZZ][c] = g.q[F_SXY][c] = g.q[F_SXZ][c] = g.q[F_SYZ][c] = 0;
        g.q[F_RC][c] = 0;
    }
}

// The conservative void reset (VOID_CONS, hydro_cpu.cpp:272-290): every
// near-void cell, in index order, zeroes its momentum, moves its excess over
// the ambient density to the densest face neighbour above RHO_CFL (candidates
// x-, x+, z-, z+, then y-, y+ when ny > 1; first of equals; volume-weighted in
// cylindrical geometry) and is reset.  The choice of neighbour depends on the
// transfers of the cells before it, so one thread walks the cells in order;
// the block loads each 1024-cell chunk's densities in parallel first.  A cell
// below RHO_CFL is never a transfer target (targets exceed RHO_CFL and only
// grow), so whether a cell is void and its own density are unchanged from the
// chunk's load until its turn.
static __global__ void __launch_bounds__(1024) k_void_cons(P p, Fields g, const Ctl* ctl) {
    if (!ctl->active) return;
    __shared__ double rs[1024];
    double* r = g.q[F_R];
    const int64_t plane = (int64_t)p.ny * p.nz;
    for (int64_t base = 0; base < p.n; base += 1024) {
        const int64_t c0 = base + threadIdx.x;
        rs[threadIdx.x] = c0 < p.n ? r[c0] : 1e300;
        __syncthreads();
        if (threadIdx.x == 0) {
            const int m = (int)(p.n - base < 1024 ? p.n - base : 1024);
            for (int t = 0; t < m; t++) {
                if (!(rs[t] < p.rho_cfl)) continue;
                const int64_t c = base + t;
                g.q[F_MU][c] = g.q[F_MV][c] = g.q[F_MW][c] = 0;
                const double amb = (p.void_amb > 0 ? p.void_amb : 0.27), exc = rs[t] - amb;
                if (exc > 0) {
                    const int i = (int)(c / plane), j = (int)((c / p.nz) % p.ny), k = (int)(c % p.nz);
                    int64_t nb = -1;
                    double rbest = p.rho_cfl;
                    const int cand[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j, k - 1},
                                            {i, j, k + 1}, {i, j - 1, k}, {i, j + 1, k}};
                    const int nc = p.ny > 1 ? 6 : 4;
                    for (int q = 0; q < nc; q++) {
                        const int ii = cand[q][0], jj = cand[q][1], kk = cand[q][2];
                        if (ii < 0 || ii >= p.nx || jj < 0 || jj >= p.ny || kk < 0 || kk >= p.nz) continue;
                        const int64_t cc = ((int64_t)ii * p.ny + jj) * p.nz + kk;
                        if (r[cc] > rbest) {
                            rbest = r[cc];
                            nb = cc;
                        }
                    }
                    if (nb >= 0) {
                        double w = 1.0;
                        if (p.axisym) {
                            const int inb = (int)(nb / plane);
                            w = (i + 0.5) / (inb + 0.5);
                        }
                        r[nb] += exc * w;
                    }
                }
                r[c] = (p.void_amb > 0 ? p.void_amb : p.ref_r0[c]);
                g.q[F_E][c] = 0;
                g.q[F_SXX][c] = g.q[F_SYY][c] = g.q[F_SZZ][c] = g.q[F_SXY][c] = g.q[F_SXZ][c] = g.q[F_SYZ][c] = 0;
                g.q[F_RC][c] = 0;
            }
        }
        __syncthreads();
    }
}

// The predictor's radial return when the conservative void pass runs between
// the update and the return.
template <class R>
static __global__ void k_yield_stage(P p, Fields g1, const double* af, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    PcellOnce<R> pc;
    vonmises_cell<R>(p, g1, af, c, false, pc);
}

// The reference state's face-pressure difference of the well-balanced gravity
// source (hydro_cpu.cpp:139-143): p0 at the averaged reference densities of the
// cell's top and bottom faces (zero internal energy, clamped at 0), in the
// reference's operation order.  It depends only on the frozen reference and the
// material, so it is formed once per reference (and material) instead of in
// every right-hand side.
static __global__ void k_ref_dp(P p, const double* R0, double* dp) {
    const int64_t c = gtid();
    if (c >= p.n) return;
    const int k = (int)(c % p.nz);
    const int64_t ct = c + (k < p.nz - 1 ? 1 : 0), cb = c - (k > 0 ? 1 : 0);
    double r0t = 0.5 * (R0[c] + R0[ct]), r0b = 0.5 * (R0[cb] + R0[c]);
    double p0t = pressure(p.m, r0t, 0.0);
    if (p0t < 0) p0t = 0;
    double p0b = pressure(p.m, r0b, 0.0);
    if (p0b < 0) p0b = 0;
    dp[c] = p0t - p0b;
}

// set_ref (hydro_cpu.cpp:259-261): density and pressure frozen as the reference.
static __global__ void k_set_ref(P p, Fields g, double* r0, double* p0) {
    const int64_t c = gtid();
    if (c >= p.n) return;
    r0[c] = g.q[F_R][c];
    p0[c] = pcell(p, g, c);
}

// Predictor (hydro_cpu.cpp:413-418): g1 = g + dt d, void-cell reset, radial
// return without regeneration.
template <class R>
static __global__ void k_predict(P p, Fields g, Fields g1, Rhs d, const Ctl* ctl) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const double dt = ctl->dt;
#pragma unroll
    for (int q = 0; q < ND; q++) g1.q[rk_field(q)][c] = g.q[rk_field(q)][c] + dt * d.q[q][c];
    void_cell(p, g1, c);
    if (!(p.void_cons && p.ref_r0)) {  // else after k_void_cons
        PcellOnce<R> pc;
        vonmises_cell<R>(p, g1, g.q[F_AF], c, false, pc);
    }
}

// Corrector and the end of the step (hydro_cpu.cpp:419-424): trapezoidal
// average, damage growth, radial return, damping, void-cell reset.  With the
// implicit viscosity, which runs between the average and the rest, stage 1 is
// the average alone and stage 2 the rest; stage 0 is all of it.
template <class R>
static __global__ void k_correct(P p, Fields g, Fields g1, Rhs d, const Ctl* ctl, int stage) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const double dt = ctl->dt;
    if (stage != 2) {
#pragma unroll
        for (int q = 0; q < ND; q++) {
            double* x = g.q[rk_field(q)];
            x[c] = 0.5 * (x[c] + g1.q[rk_field(q)][c] + dt * d.q[q][c]);
        }
        if (stage == 1) return;
    }
    PcellOnce<R> pc;
    grow_damage_cell<R>(p, g, c, dt, pc);
    vonmises_cell<R>(p, g, g.q[F_AF], c, true, pc);
    if (p.damp < 1.0) {
        g.q[F_MU][c] *= p.damp;
        g.q[F_MV][c] *= p.damp;
        g.q[F_MW][c] *= p.damp;
    }
    void_cell(p, g, c);
}

// Driver adjustments after each step (eu_set_driver), in this order:
//   pin:   the lowest `pin` z-layers return to the reference density at rest
//          with no energy (DRV_PIN_STRESS: and no deviatoric stress);
//   isp:   columns i >= isp relax toward the reference with weight
//          ((i - isp) / max(1, nx - 1 - isp))^2 (isp < 0: none);
//   DRV_VOID_AMBIENT: near-void cells (rho < RHO_CFL) become ambient gas
//          (0.27 kg/m^3) at rest with no energy and no stress;
//   DRV_TRACK_PMAX: Pmax = max(Pmax, Pcell) per cell.
// The crater mode's floor pin and radial sponge (hydro_cpu.cpp:634-637), the
// collapse demo's held floor (893-894), the Prater run's void cleanup
// (823-824) and the Pierazzo run's peak-pressure record (769).
enum { DRV_PIN_STRESS = 1, DRV_VOID_AMBIENT = 2, DRV_TRACK_PMAX = 4 };

static __global__ void k_driver(P p, Fields g, const Ctl* ctl, int pin, int isp, int flags) {
    const int64_t c = gtid();
    if (c >= p.n || !ctl->active) return;
    const int i = (int)(c / ((int64_t)p.ny * p.nz)), k = (int)(c % p.nz);
    if (k < pin) {
        g.q[F_R][c] = p.ref_r0[c];
        g.q[F_MU][c] = g.q[F_MV][c] = g.q[F_MW][c] = 0;
        g.q[F_E][c] = 0;
        if (flags & DRV_PIN_STRESS)
            g.q[F_SXX][c] = g.q[F_SYY][c] = g.q[F_SZZ][c] = g.q[F_SXY][c] = g.q[F_SXZ][c] = g.q[F_SYZ][c] = 0;
    }
    if (isp >= 0 && i >= isp) {
        const int span = p.nx - 1 - isp;
        const double xi = (double)(i - isp) / (span > 1 ? span : 1), sp = xi * xi;
        g.q[F_R][c] = (1 - sp) * g.q[F_R][c] + sp * p.ref_r0[c];
        g.q[F_MU][c] *= (1 - sp);
        g.q[F_MV][c] *= (1 - sp);
        g.q[F_MW][c] *= (1 - sp);
        g.q[F_E][c] *= (1 - sp);
    }
    if ((flags & DRV_VOID_AMBIENT) && g.q[F_R][c] < p.rho_cfl) {
        g.q[F_R][c] = 0.27;
        g.q[F_MU][c] = g.q[F_MV][c] = g.q[F_MW][c] = 0;
        g.q[F_E][c] = 0;
        g.q[F_SXX][c] = g.q[F_SYY][c] = g.q[F_SZZ][c] = g.q[F_SXY][c] = g.q[F_SXZ][c] = g.q[F_SYZ][c] = 0;
    }
    if (flags & DRV_TRACK_PMAX) {
        const double P = pcell(p, g, c);
        if (P > g.q[F_PMAX][c]) g.q[F_PMAX][c] = P;
    }
}

// Single operators for the C ABI's unit calls.
static __global__ void k_vonmises(P p, Fields g, int reg) {
    const int64_t c = gtid();
    PcellOnce<double> pc;
    if (c < p.n) vonmises_cell<double>(p, g, g.q[F_AF], c, reg != 0, pc);
}
static __global__ void k_grow_damage(P p, Fields g, double dt) {
    const int64_t c = gtid();
    PcellOnce<double> pc;
    if (c < p.n) grow_damage_cell<double>(p, g, c, dt, pc);
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


// ---------------------------------------------------------------- Lop launcher

// Side streams and events that let the face passes of one Lop run side by side.
struct FaceFork {
    cudaStream_t side[2];
    cudaEvent_t fork, join[2];
};

// One Lop (hydro_cpu.cpp:98-214) of state s in compute type R: primitives,
// the three directions' face fluxes, the right-hand side.
template <class R>
// Returns the first error of the fork's event calls (kernel launch errors
// are the caller's cudaGetLastError).
inline cudaError_t enqueue_lop_t(const P& p, const Fields& s, PrimT<R> W, const double* af, FacesT<R> F, Rhs d,
                                 const Ctl* ctl, cudaStream_t st, const FaceFork* fork) {
    cudaError_t err = cudaSuccess;
    auto fork_check = [&](cudaError_t e) {
        if (err == cudaSuccess) err = e;
    };
    auto blocks = [](int64_t count, int b) { return (unsigned)((count + b - 1) / b); };
    if constexpr (sizeof(R) == 8) {  // FP64: the right-hand side reads the state's own strength fields
#pragma unroll
        for (int q = 0; q < 6; q++) W.sq[q] = s.q[F_SXX + q];
        W.sq[6] = s.q[F_D];
        W.sq[7] = s.q[F_VIB];
        W.vd = nullptr;
    }
    k_prim<R><<<blocks(p.n, 256), 256, 0, st>>>(p, s, W, ctl);
    // the three directions' face passes are independent: with a fork, y and z
    // run on side streams beside x (a small grid's passes then share the SMs;
    // inside a captured graph they become parallel branches)
    cudaStream_t sy = st, sz = st;
    if (fork) {
        fork_check(cudaEventRecord(fork->fork, st));
        fork_check(cudaStreamWaitEvent(fork->side[0], fork->fork, 0));
        fork_check(cudaStreamWaitEvent(fork->side[1], fork->fork, 0));
        sy = fork->side[0];
        sz = fork->side[1];
    }
    k_face<0, R><<<blocks(face_count<0>(p.nx, p.ny, p.nz), 256), 256, 0, st>>>(p, W, F, ctl);
    k_face<1, R><<<blocks(face_count<1>(p.nx, p.ny, p.nz), 256), 256, 0, sy>>>(p, W, F, ctl);
    k_face<2, R><<<blocks(face_count<2>(p.nx, p.ny, p.nz), 256), 256, 0, sz>>>(p, W, F, ctl);
    if (fork) {
        fork_check(cudaEventRecord(fork->join[0], sy));
        fork_check(cudaEventRecord(fork->join[1], sz));
        fork_check(cudaStreamWaitEvent(st, fork->join[0], 0));
        fork_check(cudaStreamWaitEvent(st, fork->join[1], 0));
    }
    k_rhs<R><<<blocks(p.n, 128), 128, 0, st>>>(p, s, W, af, F, d, ctl);
    return err;
}

// The CFL speed reduction, the predictor and the corrector in compute type R.
template <class R>
inline void enqueue_maxspeed_t(const P& p, const Fields& g, Ctl* ctl, cudaStream_t st) {
    k_maxspeed<R><<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p, g, ctl);
}
template <class R>
inline void enqueue_predict_t(const P& p, const Fields& g, const Fields& g1, Rhs d, const Ctl* ctl, cudaStream_t st) {
    k_predict<R><<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p, g, g1, d, ctl);
    if (p.void_cons && p.ref_r0 && p.rho_cfl > 0) {  // void_cells(g1) in order, then vonmises(g1, false)
        k_void_cons<<<1, 1024, 0, st>>>(p, g1, ctl);
        k_yield_stage<R><<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p, g1, g.q[F_AF], ctl);
    }
}
template <class R>
inline void enqueue_correct_t(const P& p, const Fields& g, const Fields& g1, Rhs d, const Ctl* ctl, cudaStream_t st,
                              int stage) {
    k_correct<R><<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(p, g, g1, d, ctl, stage);
    if (stage != 1 && p.void_cons && p.ref_r0 && p.rho_cfl > 0)
        k_void_cons<<<1, 1024, 0, st>>>(p, g, ctl);  // void_cells(g) last
}

// The FP32 instantiations live in euler_mixed.cu (compiled with fused
// multiply-adds); the FP64 ones in euler.cu (compiled without).
cudaError_t enqueue_lop_f32(const P& p, const Fields& s, PrimT<float> W, const double* af, FacesT<float> F, Rhs d,
                            const Ctl* ctl, cudaStream_t st, const FaceFork* fork);
void enqueue_maxspeed_f32(const P& p, const Fields& g, Ctl* ctl, cudaStream_t st);
void enqueue_predict_f32(const P& p, const Fields& g, const Fields& g1, Rhs d, const Ctl* ctl, cudaStream_t st);
void enqueue_correct_f32(const P& p, const Fields& g, const Fields& g1, Rhs d, const Ctl* ctl, cudaStream_t st,
                         int stage);

}  // namespace deu
