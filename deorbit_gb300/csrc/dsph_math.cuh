// dsph_math.cuh -- per-particle and per-pair physics of the SPH step, templated
// on the arithmetic type R (double for the plain form, float for the mixed form).
//
// Semantics follow the reference solver: cubic-spline kernel and derivative
// (hydrocodes/sph/sph.hpp:17-28), Smith's largest eigenvalue (sph.hpp:41-54),
// Tillotson pressure and analytic sound speed (hydrocodes/common/eos.hpp:52-113).
// The device code is free to fuse multiply-adds and to share subexpressions;
// parity with the FP64 oracle is checked to a stated tolerance.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace dsph {

constexpr int kMaxMaterials = 32;

template <class R>
struct MatT {
    int32_t type;         // 0 ideal, 1 Tillotson
    int32_t yield_model;  // 0 von Mises, 1 Collins
    R gamma, rho0, a, b, A, B, alpha, beta, u0, uiv, ucv;
    R G, Y, Emod, wm, wk;
    R Y0, mu_i, Ylim, Yd0, mu_d;
};

template <class R> __device__ __forceinline__ R rmax(R a, R b) { return (a < b) ? b : a; }
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return (b < a) ? b : a; }

__device__ __forceinline__ double rsqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float rsqrt_(float x) { return sqrtf(x); }

// Divisions inside pair loops: the hardware approximation (__fdividef, 2 ulp)
// in FP32 -- far inside the mixed form's error budget -- and the IEEE division
// in FP64, whose results stay bit-comparable with the oracle's.
__device__ __forceinline__ float pair_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double pair_div(double a, double b) { return a / b; }
__device__ __forceinline__ double rexp(double x) { return exp(x); }
__device__ __forceinline__ float rexp(float x) { return expf(x); }
__device__ __forceinline__ double rcbrt(double x) { return cbrt(x); }
__device__ __forceinline__ float rcbrt(float x) { return cbrtf(x); }
__device__ __forceinline__ double racos(double x) { return acos(x); }
__device__ __forceinline__ float racos(float x) { return acosf(x); }
__device__ __forceinline__ double rcos(double x) { return cos(x); }
__device__ __forceinline__ float rcos(float x) { return cosf(x); }
__device__ __forceinline__ double rabs(double x) { return fabs(x); }
__device__ __forceinline__ float rabs(float x) { return fabsf(x); }

template <class R> struct K;
template <> struct K<double> { static constexpr double inv_pi = 0.31830988618379067154; };
template <> struct K<float> { static constexpr float inv_pi = 0.31830988618379067154f; };

// Cubic spline W(r, h) with support 2h (sph.hpp:17-22).
template <class R>
__device__ __forceinline__ R kernel_W(R r, R h) {
    R ih = R(1) / h;
    R q = r * ih, s = K<R>::inv_pi * ih * ih * ih;
    if (q < R(1)) return s * (R(1) - R(1.5) * q * q + R(0.75) * q * q * q);
    if (q < R(2)) {
        R t = R(2) - q;
        return s * R(0.25) * t * t * t;
    }
    return R(0);
}

// dW/dr (sph.hpp:23-28), given 1/h.
template <class R>
__device__ __forceinline__ R kernel_dW(R r, R ih) {
    R q = r * ih, s = K<R>::inv_pi * ih * ih * ih * ih;
    if (q < R(1)) return s * (R(-3) * q + R(2.25) * q * q);
    if (q < R(2)) {
        R t = R(2) - q;
        return s * (R(-0.75) * t * t);
    }
    return R(0);
}

// W(r,h) given 1/h (same value as kernel_W up to rounding).
template <class R>
__device__ __forceinline__ R kernel_W_ih(R r, R ih) {
    R q = r * ih, s = K<R>::inv_pi * ih * ih * ih;
    if (q < R(1)) return s * (R(1) - R(1.5) * q * q + R(0.75) * q * q * q);
    if (q < R(2)) {
        R t = R(2) - q;
        return s * R(0.25) * t * t * t;
    }
    return R(0);
}

// Branch-free forms of the same spline: with t = max(2 - q, 0) and
// a = max(1 - q, 0), W = s (t^3 / 4 - a^3) and dW/dr = s / h (3 a^2 - 3 t^2 / 4)
// reproduce both pieces and the zero tail (no divergence inside warps).
template <class R>
__device__ __forceinline__ R kernel_W_bf(R r, R ih) {
    R q = r * ih;
    R t = rmax(R(2) - q, R(0)), a = rmax(R(1) - q, R(0));
    return K<R>::inv_pi * ih * ih * ih * (R(0.25) * t * t * t - a * a * a);
}
template <class R>
__device__ __forceinline__ R kernel_dW_bf(R r, R ih) {
    R q = r * ih;
    R t = rmax(R(2) - q, R(0)), a = rmax(R(1) - q, R(0));
    return K<R>::inv_pi * ih * ih * ih * ih * (R(3) * a * a - R(0.75) * t * t);
}

// Largest eigenvalue of the symmetric tensor {xx,yy,zz,xy,xz,yz} by Smith's
// trigonometric method (sph.hpp:41-54).
template <class R>
__device__ __forceinline__ R eig_max(R xx, R yy, R zz, R xy, R xz, R yz) {
    R p1 = xy * xy + xz * xz + yz * yz;
    R q = (xx + yy + zz) / R(3);
    if (p1 < R(1e-30)) return rmax(rmax(xx, yy), zz);
    R p2 = (xx - q) * (xx - q) + (yy - q) * (yy - q) + (zz - q) * (zz - q) + R(2) * p1;
    R p = rsqrt_(p2 / R(6));
    R ip = R(1) / p;
    R a = (xx - q) * ip, b = (yy - q) * ip, c = (zz - q) * ip;
    R d = xy * ip, e = xz * ip, f = yz * ip;
    R r = (a * (b * c - f * f) - d * (d * c - f * e) + e * (d * f - b * e)) * R(0.5);
    r = rmax(R(-1), rmin(R(1), r));
    R phi = racos(r) / R(3);
    return q + R(2) * p * rcos(phi);
}

// Compression mu = rho / rho0 - 1 (eos.hpp:71) and the expansion
// z = rho0 / rho - 1 (eos.hpp:83).  In FP32 the rounding of rho (and of the
// quotient) is amplified 1/mu-fold in weakly compressed material, so the
// mixed form forms rho - rho0 exactly (Sterbenz: rho within a factor two of
// rho0) and adds rho_lo, the low part of the compensated density sum.  FP64
// keeps the reference's operations.
__device__ __forceinline__ void till_mu_z(double rho0, double rho, double /*rho_lo*/, double& mu, double& z) {
    mu = rho / rho0 - 1.0;
    z = rho0 / rho - 1.0;
}
__device__ __forceinline__ void till_mu_z(float rho0, float rho, float rho_lo, float& mu, float& z) {
    const float d = (rho - rho0) + rho_lo;
    mu = d / rho0;
    z = -d / (rho + rho_lo);
}

// Tillotson condensed branch: value and analytic derivatives (eos.hpp:72-79).
template <class R>
__device__ __forceinline__ void till_cond(const MatT<R>& m, R rho, R u, R mu, R& P, R& dPdr, R& dPdu) {
    R eta = rho / m.rho0;
    R ue2 = m.u0 * eta * eta;
    R w = R(1) + u / ue2, iw = R(1) / w, aob = m.a + m.b * iw;
    P = aob * rho * u + m.A * mu + m.B * mu * mu;
    dPdu = aob * rho - m.b * rho * u * iw * iw / ue2;
    R dwdr = R(-2) * u / (ue2 * eta * m.rho0);
    dPdr = aob * u + rho * u * (-m.b * iw * iw) * dwdr + m.A / m.rho0 + R(2) * m.B * mu / m.rho0;
}

// Tillotson expanded branch: value and analytic derivatives (eos.hpp:80-94).
template <class R>
__device__ __forceinline__ void till_expd(const MatT<R>& m, R rho, R u, R mu, R z, R& P, R& dPdr, R& dPdu) {
    R eta = rho / m.rho0;
    R ue2 = m.u0 * eta * eta;
    R w = R(1) + u / ue2, iw = R(1) / w;
    R irho = R(1) / rho;
    R dzdr = -m.rho0 * irho * irho;
    R E1 = rexp(-m.alpha * z * z), E2 = rexp(-m.beta * z);
    R Gt = m.b * rho * u * iw + m.A * mu * E2;
    P = m.a * rho * u + Gt * E1;
    R dwdr = R(-2) * u / (ue2 * eta * m.rho0);
    R dGu = m.b * rho * iw - m.b * rho * u * iw * iw / ue2;
    dPdu = m.a * rho + dGu * E1;
    R dbruw_dr = m.b * u * iw + m.b * rho * u * (-iw * iw) * dwdr;
    R dGr = dbruw_dr + m.A * E2 / m.rho0 + m.A * mu * (E2 * (-m.beta) * dzdr);
    R dE1dr = E1 * (-m.alpha * R(2) * z) * dzdr;
    dPdr = m.a * u + dGr * E1 + Gt * dE1dr;
}

// Pressure (eos.hpp:52-68) and sound speed (eos.hpp:95-113) in one pass.
template <class R>
__device__ __forceinline__ void eos_P_cs(const MatT<R>& m, R rho, R u, R& P, R& cs, R rho_lo = R(0)) {
    if (m.type == 0) {  // ideal gas
        P = (m.gamma - R(1)) * rho * u;
        cs = rsqrt_(rmax(m.gamma * P / rmax(rho, R(1e-30)), R(1e-12)));
        return;
    }
    if (rho <= R(0)) {
        P = R(0);
        cs = R(1e-3);
        return;
    }
    R Pp, dPdr, dPdu, mu, z;
    till_mu_z(m.rho0, rho, rho_lo, mu, z);
    // rho >= rho0 (eos.hpp:77); FP64 compares as the reference does
    const bool compressed = sizeof(R) == 8 ? (rho >= m.rho0) : (mu >= R(0));
    if (compressed || u <= m.uiv) {
        till_cond(m, rho, u, mu, Pp, dPdr, dPdu);
        P = Pp;
    } else if (u >= m.ucv) {
        till_expd(m, rho, u, mu, z, Pp, dPdr, dPdu);
        P = Pp;
    } else {  // intermediate: energy-weighted blend of the two branches
        R Pc, dPcr, dPcu, Pe, dPer, dPeu;
        till_cond(m, rho, u, mu, Pc, dPcr, dPcu);
        till_expd(m, rho, u, mu, z, Pe, dPer, dPeu);
        R inv = R(1) / (m.ucv - m.uiv);
        P = ((u - m.uiv) * Pe + (m.ucv - u) * Pc) * inv;
        Pp = P;
        dPdu = ((Pe + (u - m.uiv) * dPeu) + (-Pc + (m.ucv - u) * dPcu)) * inv;
        dPdr = ((u - m.uiv) * dPer + (m.ucv - u) * dPcr) * inv;
    }
    cs = rsqrt_(rmax(dPdr + Pp / (rho * rho) * dPdu, R(1e-6)));
}

// Flow stress of a material: von Mises Y (sph.hpp:321) or, for the Collins
// model, the Lundborg intact / friction damaged blend of
// hydrocodes/euler/hydro_cpu.cpp:231-236 with P clamped at zero.
template <class R>
__device__ __forceinline__ R yield_stress(const MatT<R>& m, R P, R D) {
    if (m.yield_model != 1) return m.Y;
    R Pc = rmax(P, R(0));
    R Yi = m.Y0 + m.mu_i * Pc / (R(1) + m.mu_i * Pc / rmax(m.Ylim - m.Y0, R(1)));
    R Yd = rmin(m.Yd0 + m.mu_d * Pc, m.Ylim);
    return (R(1) - D) * Yi + D * Yd;
}

}  // namespace dsph
