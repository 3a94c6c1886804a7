// A driver in the style of the reference's cpu_dump.cpp, written against the
// System facade (deorbit_sph_system.hpp) instead of sph.hpp: sheared,
// compressed two-material cube, seeded flaws, `steps` CFL steps, then one
// density + force evaluation; writes n and 14 float64 fields per particle
// (x y z vx vy vz u rho hh D Sxy ax dudt eps_act).
//
//   facade_driver <L> <steps> <out.bin> [mixed]
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "deorbit_sph_system.hpp"

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s L steps out.bin [mixed]\n", argv[0]);
        return 1;
    }
    const int L = std::atoi(argv[1]);
    const int steps = std::atoi(argv[2]);
    const bool mixed = argc > 4 && std::strcmp(argv[4], "mixed") == 0;
    try {
        System S(mixed ? SPH_MIXED : SPH_FP64);
        S.materials.push_back(Material::basalt());
        S.materials.push_back(Material::iron());
        S.eta = 1.3;
        S.eps_as = 0.3;
        S.damage_on = true;
        const double dx = 30.0;
        S.h_init = S.eta * dx;
        const double lo = -L * dx / 2.0, hi = L * dx / 2.0;
        S.set_domain(lo - dx, hi + dx, false, lo - dx, hi + dx, false, lo - dx, hi + dx, false);
        const double R = 5.0 * dx;
        for (int i = 0; i < L; i++)
            for (int j = 0; j < L; j++)
                for (int k = 0; k < L; k++) {
                    const double x = lo + (i + 0.5) * dx, y = lo + (j + 0.5) * dx, z = lo + (k + 0.5) * dx;
                    const bool iron = (x * x + y * y + z * z) < R * R;
                    S.cur_mat = iron ? 1 : 0;
                    S.add({x, y, z}, {80.0 * (y / hi), 0.0, -40.0 * (z / hi)},
                          (iron ? 7800.0 : 2700.0) * dx * dx * dx, 2.0e5 * (1.0 + x / hi), false);
                }
        S.seed_damage(dx);
        S.init();
        for (int s = 0; s < steps; s++) {
            const double dt = S.timestep();
            S.step(dt);
        }
        S.compute_density_h();
        S.compute_forces();
        FILE* f = std::fopen(argv[3], "wb");
        if (!f) return 1;
        const long n = S.n;
        std::fwrite(&n, sizeof(long), 1, f);
        for (int i = 0; i < S.n; i++) {
            const double r[14] = {S.pos[i].x, S.pos[i].y, S.pos[i].z, S.vel[i].x, S.vel[i].y, S.vel[i].z,
                                  S.u[i], S.rho[i], S.hh[i], S.D[i], S.S[i].xy, S.acc[i].x, S.dudt[i],
                                  S.eps_act[i]};
            std::fwrite(r, sizeof(double), 14, f);
        }
        std::fclose(f);
        double vmax = 0;
        for (int i = 0; i < S.n; i++) vmax = std::max(vmax, norm(S.vel[i]));
        std::printf("n=%d t=%.6e vmax=%.3f nc=%d,%d,%d\n", S.n, S.t, vmax, S.nc[0], S.nc[1], S.nc[2]);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
