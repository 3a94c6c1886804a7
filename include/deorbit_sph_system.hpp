// deorbit_sph_system.hpp -- header-only C++ facade with the member names and
// call order of the reference solver's `struct System`
// (hydrocodes/sph/sph.hpp:72-380), `struct Material` (hydrocodes/common/eos.hpp:15-50)
// and `Vec3` / `Sym3` (hydrocodes/sph/vec3.hpp, sph.hpp:31-33), running on the GPU
// through the C ABI of libdeorbit_sph.so (deorbit_sph.h).
//
// A driver written against sph.hpp (run_ic.cpp, cpu_bench.cpp, cpu_dump.cpp)
// rebuilds against this header by replacing `#include "sph.hpp"` with
// `#include "deorbit_sph_system.hpp"` and linking -ldeorbit_sph.
//
// State model.  The public vectors (pos, vel, rho, S, ...) are a host mirror of
// the device state.  With `sync` true (the default) every device call pushes
// the mirror's carried fields to the device first and pulls every field back
// afterwards, so a driver may read or modify any vector between calls exactly
// as with the CPU solver (run_ic.cpp:36-38 writes D, eps_act and S after add());
// step(dt) does the push, the step and the pull in one sph_step_fields call,
// whose host copies overlap the step's kernels.
// A driver that only reads occasionally sets `sync = false` and calls pull()
// when it needs the fields (and push() after changing them); run(nsteps) is the
// batched device loop with each step's CFL dt taken on the device.
//
// Differences a caller sees: errors throw std::runtime_error with the library's
// message (the reference has no error reporting); particles are added before
// init(); `precision` selects the plain FP64 solver (default) or the mixed form.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "deorbit_sph.h"

namespace deorbit_sph {

struct Vec3 {
    double x = 0, y = 0, z = 0;
    Vec3() {}
    Vec3(double a, double b, double c) : x(a), y(b), z(c) {}
    Vec3 operator+(const Vec3& o) const { return {x + o.x, y + o.y, z + o.z}; }
    Vec3 operator-(const Vec3& o) const { return {x - o.x, y - o.y, z - o.z}; }
    Vec3 operator*(double s) const { return {x * s, y * s, z * s}; }
    Vec3& operator+=(const Vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    Vec3& operator-=(const Vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
};
inline double dot(const Vec3& a, const Vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm2(const Vec3& a) { return dot(a, a); }
inline double norm(const Vec3& a) { return std::sqrt(dot(a, a)); }

struct Sym3 {
    double xx = 0, yy = 0, zz = 0, xy = 0, xz = 0, yz = 0;
};

// Material with the reference's field names; the factories take their values
// from the library (sph_material_tillotson / sph_material_standard).  The
// Collins fields are the library's pressure-dependent yield extension.
struct Material {
    enum Type { IDEAL, TILLOTSON };
    Type type = IDEAL;
    double gamma = 1.4;
    double rho0 = 0, a = 0, b = 0, A = 0, B = 0, alpha = 0, beta = 0;
    double u0 = 0, uiv = 0, ucv = 0;
    double G = 0, Y = 0;
    double Emod = 0, wm = 0, wk = 0;
    int yield_model = SPH_YIELD_VON_MISES;
    double Y0 = 0, mu_i = 0, Ylim = 0, Yd0 = 0, mu_d = 0;

    static Material from_c(const sph_material& c) {
        Material m;
        m.type = c.type == SPH_EOS_TILLOTSON ? TILLOTSON : IDEAL;
        m.gamma = c.gamma;
        m.rho0 = c.rho0; m.a = c.a; m.b = c.b; m.A = c.A; m.B = c.B;
        m.alpha = c.alpha; m.beta = c.beta; m.u0 = c.u0; m.uiv = c.uiv; m.ucv = c.ucv;
        m.G = c.G; m.Y = c.Y; m.Emod = c.Emod; m.wm = c.wm; m.wk = c.wk;
        m.yield_model = c.yield_model;
        m.Y0 = c.Y0; m.mu_i = c.mu_i; m.Ylim = c.Ylim; m.Yd0 = c.Yd0; m.mu_d = c.mu_d;
        return m;
    }
    sph_material to_c() const {
        sph_material c{};
        c.type = type == TILLOTSON ? SPH_EOS_TILLOTSON : SPH_EOS_IDEAL;
        c.yield_model = yield_model;
        c.gamma = gamma;
        c.rho0 = rho0; c.a = a; c.b = b; c.A = A; c.B = B;
        c.alpha = alpha; c.beta = beta; c.u0 = u0; c.uiv = uiv; c.ucv = ucv;
        c.G = G; c.Y = Y; c.Emod = Emod; c.wm = wm; c.wk = wk;
        c.Y0 = Y0; c.mu_i = mu_i; c.Ylim = Ylim; c.Yd0 = Yd0; c.mu_d = mu_d;
        return c;
    }
    static Material ideal(double g) {
        sph_material c;
        sph_material_ideal(&c, g);
        return from_c(c);
    }
    static Material tillotson(double rho0_, double A_, double B_, double a_, double b_, double al,
                              double be, double u0_, double uiv_, double ucv_, double G_ = 0,
                              double Y_ = 0, double wm_ = 0, double wk_ = 0) {
        sph_material c;
        sph_material_tillotson(&c, rho0_, A_, B_, a_, b_, al, be, u0_, uiv_, ucv_, G_, Y_, wm_, wk_);
        return from_c(c);
    }
    static Material standard(int which) {
        sph_material c;
        if (sph_material_standard(which, &c) != SPH_OK) throw std::runtime_error(sph_last_error());
        return from_c(c);
    }
    static Material iron() { return standard(0); }
    static Material basalt() { return standard(1); }
    static Material water() { return standard(2); }
    static Material aluminum() { return standard(3); }
};

struct System {
    // ---- particle state (host mirror), sph.hpp:73-81
    std::vector<Vec3> pos, vel, acc;
    std::vector<double> mass, rho, u, dudt, P, cs, csig, hh, eps_work;
    std::vector<double> D, eps_act, sigmax, Pf, Rart, dscale;
    std::vector<Sym3> S, dSdt;
    std::vector<int> mat;
    std::vector<char> fixed;
    std::vector<Material> materials;
    int cur_mat = 0;
    int n = 0;

    // ---- parameters, sph.hpp:84-92
    double eta = 1.3;
    double h_init = 0.01, h_max = 0.01;
    double alpha = 1.0, beta = 2.0, eps = 0.01, alpha_u = 0.0;
    double cfl = 0.2;
    double eps_as = 0.0;
    int as_n = 4;
    bool damage_on = false;
    double dlo[3] = {0, 0, 0}, dhi[3] = {0, 0, 0};
    bool per[3] = {false, false, false};
    int nc[3] = {1, 1, 1};  // reference cell grid of the last cell build

    // ---- facade controls
    int precision = SPH_FP64;
    int device = 0;
    bool sync = true;
    double t = 0.0;  // simulated time advanced by step() / run()

    System() {}
    explicit System(int precision_, int device_ = 0) : precision(precision_), device(device_) {}
    ~System() {
        if (ctx_) sph_destroy(ctx_);
    }
    System(const System&) = delete;
    System& operator=(const System&) = delete;

    void set_domain(double xl, double xh, bool px, double yl, double yh, bool py, double zl, double zh,
                    bool pz) {
        dlo[0] = xl; dhi[0] = xh; per[0] = px;
        dlo[1] = yl; dhi[1] = yh; per[1] = py;
        dlo[2] = zl; dhi[2] = zh; per[2] = pz;
    }

    void add(Vec3 p, Vec3 v, double m, double uu, bool fix = false) {
        if (ctx_) throw std::runtime_error("System::add after init() is not supported");
        pos.push_back(p); vel.push_back(v); acc.push_back({});
        mass.push_back(m); rho.push_back(0); u.push_back(uu); dudt.push_back(0);
        P.push_back(0); cs.push_back(0); csig.push_back(0); hh.push_back(h_init);
        eps_work.push_back(0); S.push_back({}); dSdt.push_back({});
        D.push_back(0); eps_act.push_back(1e30); sigmax.push_back(0);
        Pf.push_back(0); Rart.push_back(0); dscale.push_back(1.0);
        mat.push_back(cur_mat); fixed.push_back(fix ? 1 : 0);
        n++;
    }

    // Flaw thresholds of sph.hpp:117-128 (same mt19937 stream), on the host.
    void seed_damage(double dx, unsigned seed = 12345) {
        std::vector<sph_material> cm;
        for (const Material& m : materials) cm.push_back(m.to_c());
        check(sph_seed_flaws_single(n, mat.data(), cm.data(), (int32_t)cm.size(), dx, seed, eps_act.data()));
    }

    void init() {
        if (!ctx_) create();
        push();
        check(sph_init(ctx_));
        pull();
    }

    double timestep() {
        need();
        if (sync) push();
        double dt = 0;
        check(sph_timestep(ctx_, b_, &dt));
        return dt;
    }

    void step(double dt) {
        need();
        if (sync && n && dt >= 0) {
            // push, step and pull in one call whose host copies overlap the step
            write_fixed_flags();
            std::vector<std::vector<double>> in, out;
            std::vector<const double*> ins;
            std::vector<double*> outs;
            pack_carried(in, ins);
            pull_buffers(out, outs);
            check(sph_step_fields(ctx_, b_, dt, (int32_t)ins.size(), kPushNames, ins.data(), (int32_t)outs.size(),
                                  kPullNames, outs.data(), nullptr));
            t += dt;
            unpack_pulled(out);
            return;
        }
        if (sync) push();
        check(sph_step(ctx_, dt));
        t += dt;
        if (sync) pull();
    }

    void compute_density_h(int iters = 2) {
        need();
        if (sync) push();
        check(sph_compute_density_h(ctx_, iters));
        if (sync) pull();
    }

    void compute_forces() {
        need();
        if (sync) push();
        check(sph_compute_forces(ctx_));
        if (sync) pull();
    }

    // Extension: nsteps steps with each step's CFL dt taken on the device
    // (no host round trip inside), stopping at t_end when t_end > 0.
    void run(int nsteps, double t_end = 0.0) {
        need();
        if (sync) push();
        check(sph_run(ctx_, nsteps, t_end));
        sph_impact_info inf;
        check(sph_impact_info_get(ctx_, b_, &inf));
        t = inf.t;
        if (sync) pull();
    }

    // Copy every field from the device into the mirror (one batched call).
    void pull() {
        need();
        std::vector<std::vector<double>> buf;
        std::vector<double*> outs;
        pull_buffers(buf, outs);
        if (n) check(sph_read_fields(ctx_, b_, (int32_t)outs.size(), kPullNames, outs.data()));
        unpack_pulled(buf);
    }

    // Copy the carried fields of the mirror to the device (the state a step
    // reads: positions, velocities, old derivatives, u, h, mass, stress,
    // damage, flaws, fixed flags), in one batched call.
    void push() {
        need();
        std::vector<std::vector<double>> buf;
        std::vector<const double*> ins;
        pack_carried(buf, ins);
        if (n) check(sph_write_fields(ctx_, b_, (int32_t)ins.size(), kPushNames, ins.data()));
        write_fixed_flags();
    }

    sph_ctx* context() const { return ctx_; }
    int32_t impact() const { return b_; }

private:
    sph_ctx* ctx_ = nullptr;
    int32_t b_ = -1;

    static constexpr int kNumPush = 27, kNumPull = 36;
    static constexpr const char* kPushNames[kNumPush] = {
        "x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz",
        "dSxx", "dSyy", "dSzz", "dSxy", "dSxz", "dSyz", "mass", "u", "dudt", "hh", "D", "eps_act"};
    static constexpr const char* kPullNames[kNumPull] = {
        "x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz",
        "dSxx", "dSyy", "dSzz", "dSxy", "dSxz", "dSyz", "mass", "rho", "u", "dudt", "P", "cs", "csig",
        "hh", "eps_work", "D", "eps_act", "sigmax", "Pf", "Rart", "dscale"};

    // the mirror's carried fields as kPushNames columns
    void pack_carried(std::vector<std::vector<double>>& buf, std::vector<const double*>& ins) const {
        buf.assign(kNumPush, std::vector<double>((size_t)n));
        for (int i = 0; i < n; i++) {
            buf[0][i] = pos[i].x; buf[1][i] = pos[i].y; buf[2][i] = pos[i].z;
            buf[3][i] = vel[i].x; buf[4][i] = vel[i].y; buf[5][i] = vel[i].z;
            buf[6][i] = acc[i].x; buf[7][i] = acc[i].y; buf[8][i] = acc[i].z;
            for (int c = 0; c < 6; c++) {
                buf[9 + c][i] = comp(S[i], c);
                buf[15 + c][i] = comp(dSdt[i], c);
            }
        }
        const std::vector<double>* scal[] = {&mass, &u, &dudt, &hh, &D, &eps_act};
        for (int q = 0; q < 6; q++) buf[21 + q] = *scal[q];
        ins.resize(kNumPush);
        for (int f = 0; f < kNumPush; f++) ins[f] = buf[f].data();
    }
    void pull_buffers(std::vector<std::vector<double>>& buf, std::vector<double*>& outs) const {
        buf.assign(kNumPull, std::vector<double>((size_t)n));
        outs.resize(kNumPull);
        for (int f = 0; f < kNumPull; f++) outs[f] = buf[f].data();
    }
    // kPullNames columns into the mirror, then the fixed flags and grid info
    void unpack_pulled(const std::vector<std::vector<double>>& buf) {
        for (int i = 0; i < n; i++) {
            pos[i] = Vec3(buf[0][i], buf[1][i], buf[2][i]);
            vel[i] = Vec3(buf[3][i], buf[4][i], buf[5][i]);
            acc[i] = Vec3(buf[6][i], buf[7][i], buf[8][i]);
            for (int c = 0; c < 6; c++) {
                comp(S[i], c) = buf[9 + c][i];
                comp(dSdt[i], c) = buf[15 + c][i];
            }
        }
        std::vector<double>* scal[] = {&mass, &rho, &u, &dudt, &P, &cs, &csig, &hh, &eps_work,
                                       &D, &eps_act, &sigmax, &Pf, &Rart, &dscale};
        for (int q = 0; q < 15; q++) *scal[q] = buf[21 + q];
        std::vector<uint8_t> f(n);
        if (n) check(sph_read_fixed(ctx_, b_, f.data()));
        for (int i = 0; i < n; i++) fixed[i] = (char)f[i];
        sph_impact_info inf;
        check(sph_impact_info_get(ctx_, b_, &inf));
        for (int a = 0; a < 3; a++) nc[a] = inf.nc[a];
        h_max = inf.h_max;
    }
    void write_fixed_flags() {
        std::vector<uint8_t> f(n);
        for (int i = 0; i < n; i++) f[i] = fixed[i] ? 1 : 0;
        if (n) check(sph_write_fixed(ctx_, b_, f.data()));
    }

    static void check(int rc) {
        if (rc != SPH_OK) throw std::runtime_error(std::string("deorbit_sph: ") + sph_last_error());
    }
    void need() const {
        if (!ctx_) throw std::runtime_error("System: call init() first");
    }

    void create() {
        check(sph_create(&ctx_, precision, device));
        for (const Material& m : materials) {
            sph_material c = m.to_c();
            int32_t id;
            check(sph_add_material(ctx_, &c, &id));
        }
        sph_params p;
        sph_params_default(&p);
        p.eta = eta; p.h_init = h_init; p.alpha = alpha; p.beta = beta; p.eps = eps;
        p.alpha_u = alpha_u; p.cfl = cfl; p.eps_as = eps_as; p.as_n = as_n;
        p.damage_on = damage_on ? 1 : 0;
        int32_t pr[3] = {per[0], per[1], per[2]};
        check(sph_impact_create(ctx_, &p, dlo, dhi, pr, &b_));
        std::vector<double> x(n), y(n), z(n), vx(n), vy(n), vz(n);
        std::vector<uint8_t> f(n);
        for (int i = 0; i < n; i++) {
            x[i] = pos[i].x; y[i] = pos[i].y; z[i] = pos[i].z;
            vx[i] = vel[i].x; vy[i] = vel[i].y; vz[i] = vel[i].z;
            f[i] = fixed[i] ? 1 : 0;
        }
        if (n)
            check(sph_impact_add_particles(ctx_, b_, n, x.data(), y.data(), z.data(), vx.data(), vy.data(),
                                           vz.data(), mass.data(), u.data(), mat.data(), f.data()));
    }

    static double& comp(Sym3& s, int c) {
        return c == 0 ? s.xx : c == 1 ? s.yy : c == 2 ? s.zz : c == 3 ? s.xy : c == 4 ? s.xz : s.yz;
    }
    static double comp(const Sym3& s, int c) {
        return c == 0 ? s.xx : c == 1 ? s.yy : c == 2 ? s.zz : c == 3 ? s.xy : c == 4 ? s.xz : s.yz;
    }
};

}  // namespace deorbit_sph

#ifndef DEORBIT_SPH_NO_GLOBAL_NAMES
using deorbit_sph::dot;
using deorbit_sph::Material;
using deorbit_sph::norm;
using deorbit_sph::norm2;
using deorbit_sph::Sym3;
using deorbit_sph::System;
using deorbit_sph::Vec3;
#endif
