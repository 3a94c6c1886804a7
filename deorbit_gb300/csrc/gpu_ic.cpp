// gpu_ic -- the reference's production GPU driver (hydrocodes/sph/gpu_ic.cpp)
// on the CUDA library: same command line, IC format, progress line, snapshot
// files and exit codes, so its callers (boundary_daemon.py:230-248,
// validate_craters.py:48-49) run unchanged.
//
//   gpu_ic <ic.bin> <dx> <t_end> [walltime] [--frac] [--snap DT]
//          [--precision fp64|mixed] [--device N] [--checkpoint DT] [--restart chk.bin] [--profile]
//          [--grazing THETA,V[,CPPR[,D]]]
//
// --grazing generates the campaign's grazing IC in place (the IC that
// boundary_daemon.build_grazing_ic writes, boundary_daemon.py:119-158: basalt
// half-space, iron sphere of diameter D at THETA deg and V m/s, CPPR lattice
// cells per impactor radius; defaults 8 and 1000) instead of reading ic.bin,
// and dx is the generated lattice spacing (the ic.bin and dx arguments are
// then placeholders, e.g. "- 0").
//
// IC (run_ic.cpp:4-6): f8 header [xlo xhi ylo yhi zlo zhi n], then n x 10 f8
// [x y z vx vy vz mass u mat fixed]; mat 0 basalt, 1 iron, 2 basalt (the
// trackable impactor of gpu_ic.cpp:59).  Snapshots gpu_snap_NNN.bin: int64 n,
// then n x 10 f8 [x y z vx vy vz u rho h mat] (gpu_ic.cpp:118-123), written at
// the first step with t >= the next snapshot time.  Every 25 steps and at the
// end a progress line with the projectile (mat >= 1) centroid, mean speed,
// mean vz, melt fraction (u > 1e6 J/kg) and u max (gpu_ic.cpp:112-117); the
// reductions run on the device.
//
// Physics follows the CPU solver's semantics (sph.hpp): the Metal driver's
// own departures -- gravity (--g), velocity damping (--damp), a fixed cell
// grid, one density iteration -- are not part of it; --g or --damp with a
// non-default value is rejected.  Extensions: the precision form, lossless
// checkpoints in run_ic's format (--checkpoint, written atomically) and
// restart from one (--restart).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "deorbit_sph.h"

namespace {

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int fail(const char* what) {
    std::printf("error: %s: %s\n", what, sph_last_error());
    return 1;
}

#define CK(call)                               \
    do {                                       \
        if ((call) != SPH_OK) return fail(#call); \
    } while (0)

void usage() {
    std::printf("usage: gpu_ic ic.bin dx t_end [walltime] [--frac] [--snap DT] [--precision fp64|mixed] "
                "[--device N] [--checkpoint DT] [--restart chk.bin] [--profile] [--grazing THETA,V[,CPPR[,D]]]\n");
}

}  // namespace

int main(int argc, char** argv) {
    bool frac = false, profile = false;
    double gz = 0.0, damp = 1.0, snap_dt = 0.05, chk_dt = 0.0;
    int precision = SPH_MIXED, device = 0;
    const char* restart = nullptr;
    const char* grazing = nullptr;
    std::vector<char*> av;
    for (int i = 0; i < argc; i++) {
        std::string s = argv[i];
        if (s == "--frac") frac = true;
        else if (s == "--profile") profile = true;
        else if (s == "--g" && i + 1 < argc) gz = std::atof(argv[++i]);
        else if (s == "--damp" && i + 1 < argc) damp = std::atof(argv[++i]);
        else if (s == "--snap" && i + 1 < argc) snap_dt = std::atof(argv[++i]);
        else if (s == "--checkpoint" && i + 1 < argc) chk_dt = std::atof(argv[++i]);
        else if (s == "--restart" && i + 1 < argc) restart = argv[++i];
        else if (s == "--grazing" && i + 1 < argc) grazing = argv[++i];
        else if (s == "--device" && i + 1 < argc) device = std::atoi(argv[++i]);
        else if (s == "--precision" && i + 1 < argc) {
            std::string p = argv[++i];
            if (p == "fp64") precision = SPH_FP64;
            else if (p == "mixed") precision = SPH_MIXED;
            else { usage(); return 1; }
        } else av.push_back(argv[i]);
    }
    if (av.size() < 4) {
        usage();
        return 1;
    }
    if (gz != 0.0 || damp != 1.0) {
        std::printf("error: --g / --damp are terms of the Metal driver only; the CPU solver's physics has neither\n");
        return 1;
    }
    const char* icf = av[1];
    double dx = std::atof(av[2]);
    sph_grazing_spec gs;
    sph_grazing_spec_default(&gs);
    if (grazing) {
        double f[4] = {0, 0, 8, 1000.0};
        int nf = std::sscanf(grazing, "%lf,%lf,%lf,%lf", &f[0], &f[1], &f[2], &f[3]);
        if (nf < 2 || f[2] < 1) {
            usage();
            return 1;
        }
        gs.theta_deg = f[0];
        gs.v = f[1];
        gs.cppr = (int32_t)f[2];
        gs.D = f[3];
        gs.tgt_mat = 0;  // basalt
        gs.imp_mat = 1;  // iron
        dx = gs.D / 2.0 / gs.cppr;
    }
    const double t_end = std::atof(av[3]);
    const double walltime = av.size() > 4 ? std::atof(av[4]) : 1e30;
    if (!(dx > 0) || !(snap_dt > 0)) {
        usage();
        return 1;
    }

    sph_ctx* ctx = nullptr;
    CK(sph_create(&ctx, precision, device));
    sph_material m;
    int32_t id;
    CK(sph_material_standard(1, &m));  // 0 basalt
    CK(sph_add_material(ctx, &m, &id));
    CK(sph_material_standard(0, &m));  // 1 iron
    CK(sph_add_material(ctx, &m, &id));
    CK(sph_material_standard(1, &m));  // 2 basalt impactor
    CK(sph_add_material(ctx, &m, &id));
    sph_params p;
    sph_params_default(&p);
    p.eta = 1.3;
    p.h_init = 1.3 * dx;
    p.alpha = 1.0;
    p.beta = 2.0;
    p.eps = 0.01;
    p.cfl = 0.2;
    p.eps_as = frac ? 0.3 : 0.0;
    p.damage_on = frac ? 1 : 0;

    int32_t b = -1;
    double t = 0.0;
    if (restart) {
        double dx_ck = 0.0;  // flaws, damage and stress come from the checkpoint
        CK(sph_load_checkpoint(ctx, restart, &p, &b, &dx_ck));
    } else if (grazing) {
        CK(sph_impact_create_grazing(ctx, &p, &gs, &b, &dx, nullptr));
        if (frac) CK(sph_impact_seed_damage(ctx, b, dx, 12345));
    } else {
        CK(sph_load_ic(ctx, icf, &p, &b));
        if (frac) CK(sph_impact_seed_damage(ctx, b, dx, 12345));
    }
    sph_impact_info inf;
    CK(sph_impact_info_get(ctx, b, &inf));
    t = inf.t;
    const int64_t n = inf.n;
    std::vector<int32_t> mat(n);
    CK(sph_read_mat(ctx, b, mat.data()));
    int64_t n_iron = 0;
    for (int64_t i = 0; i < n; i++) n_iron += mat[i] == 1;
    std::printf("loaded %s: n=%lld (%lld iron)  dx=%.0f  frac=%d  g=%.2f\n",
                restart ? restart : (grazing ? "grazing IC (generated)" : icf),
                (long long)n, (long long)n_iron, dx, frac ? 1 : 0, gz);
    if (profile) CK(sph_set_profiling(ctx, 1));
    CK(sph_init(ctx));
    sph_conservation c0;
    CK(sph_conservation_get(ctx, b, &c0));
    std::printf("init done, E0=%.4e\n", c0.energy);
    std::fflush(stdout);

    auto report = [&](double tt, long long step, double wsec) -> int {
        sph_diagnostics d;
        if (sph_impact_diagnostics(ctx, b, 1, 255, 1.0e6, &d) != SPH_OK) return fail("diagnostics");
        const double melt = d.count > 0 ? 100.0 * (double)d.melted / (double)d.count : 0.0;
        std::printf("  t=%.4f step=%lld proj: x=%.0f z=%.0f |v|=%.0f vz=%.0f melt=%.0f%% umax=%.1e [%.0fs]\n", tt,
                    step, d.mean_pos[0], d.mean_pos[2], d.mean_speed, d.mean_vel[2], melt, d.u_max, wsec);
        std::fflush(stdout);
        return 0;
    };

    const double wall0 = now();
    long long step = 0;
    int isnap = 0;
    double next_snap = t + snap_dt, next_chk = chk_dt > 0 ? t + chk_dt : 1e300;
    double dt_last = 0.0;
    while (t < t_end) {
        // run to the next report (every 25 steps) in one device loop, in
        // shorter runs near a snapshot time so the snapshot is taken at the
        // first step that reaches it
        long long k = 25 - step % 25;
        if (dt_last > 0.0) {
            const double room = std::fmin(next_snap, next_chk) - t;
            long long ks = (long long)std::floor(0.8 * room / dt_last);
            if (ks < 1) ks = 1;
            if (ks < k) k = ks;
        }
        CK(sph_run(ctx, (int32_t)k, t_end));
        CK(sph_impact_info_get(ctx, b, &inf));
        if (inf.steps == step) {
            std::printf("error: the run did not advance (n=%lld, t=%.6e)\n", (long long)n, t);
            return 1;
        }
        step = inf.steps;
        t = inf.t;
        dt_last = inf.dt;
        if (step % 25 == 0 || t >= t_end) {
            if (report(t, step, now() - wall0)) return 1;
        }
        if (t >= next_snap) {
            char fn[64];
            std::snprintf(fn, sizeof fn, "gpu_snap_%03d.bin", isnap++);
            CK(sph_write_snapshot(ctx, b, fn));
            next_snap += snap_dt;
        }
        if (t >= next_chk) {
            CK(sph_write_checkpoint(ctx, b, "gpu_chk.bin", dx));
            next_chk += chk_dt;
        }
        if (now() - wall0 > walltime) {
            std::printf("walltime hit\n");
            break;
        }
    }
    sph_conservation c1;
    CK(sph_conservation_get(ctx, b, &c1));
    const double el = now() - wall0;
    std::printf("DONE: %lld steps to t=%.4f  %.1f ms/step  E drift=%.2e\n", step, t,
                step > 0 ? 1000.0 * el / (double)step : 0.0, c0.energy != 0 ? (c1.energy - c0.energy) / c0.energy : 0.0);
    if (profile) {
        const char* names[SPH_K_COUNT] = {"kick", "sort", "grid", "list", "density", "eos", "list2",
                                          "force", "damage", "finish", "dt", "other"};
        std::printf("PROFILE (ms/step):");
        for (int q = 0; q < SPH_K_COUNT; q++) {
            double ms = 0;
            int64_t nl = 0;
            CK(sph_kernel_stats(ctx, q, &ms, &nl));
            if (nl) std::printf(" %s=%.2f", names[q], step > 0 ? ms / (double)step : 0.0);
        }
        std::printf("\n");
    } else {
        std::printf("PROFILE (ms/step): total=%.2f\n", step > 0 ? 1000.0 * el / (double)step : 0.0);
    }
    sph_destroy(ctx);
    return 0;
}
