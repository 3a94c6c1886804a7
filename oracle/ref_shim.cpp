// ref_shim.cpp -- C entry points over the reference's own System (TEST ONLY).
//
// Compiled by oracle/Makefile against the UNMODIFIED reference headers
// (hydrocodes/sph/sph.hpp, vec3.hpp, hydrocodes/common/eos.hpp), which are read
// where they lie; nothing from the reference is copied into this repository.
// The resulting oracle/_ref/libsphref.so lets tests and the golden-vector
// generator drive the reference solver on the same inputs as the C oracle.
#include "sph.hpp"

#include <cstdint>
#include <cstring>
#include <string>

#include "sph_oracle.h"  // only for the plain-data orc_material / orc_params layouts

namespace {

Material to_material(const orc_material* m) {
    Material r;
    r.type = m->type == ORC_IDEAL ? Material::IDEAL : Material::TILLOTSON;
    r.gamma = m->gamma;
    r.rho0 = m->rho0; r.a = m->a; r.b = m->b; r.A = m->A; r.B = m->B;
    r.alpha = m->alpha; r.beta = m->beta; r.u0 = m->u0; r.uiv = m->uiv; r.ucv = m->ucv;
    r.G = m->G; r.Y = m->Y; r.Emod = m->Emod; r.wm = m->wm; r.wk = m->wk;
    return r;
}

double* vec3_component(std::vector<Vec3>& v, int c, size_t i) {
    return c == 0 ? &v[i].x : (c == 1 ? &v[i].y : &v[i].z);
}

// Visit one named per-particle scalar of the System: returns false if unknown.
template <class F>
bool with_field(System& S, const std::string& nm, F f) {
    const size_t n = (size_t)S.n;
    auto vec = [&](std::vector<Vec3>& v, int c) { for (size_t i = 0; i < n; i++) f(i, *vec3_component(v, c, i)); };
    auto sca = [&](std::vector<double>& v) { for (size_t i = 0; i < n; i++) f(i, v[i]); };
    auto sym = [&](std::vector<Sym3>& v, int c) {
        for (size_t i = 0; i < n; i++) {
            double* p = c == 0 ? &v[i].xx : c == 1 ? &v[i].yy : c == 2 ? &v[i].zz
                      : c == 3 ? &v[i].xy : c == 4 ? &v[i].xz : &v[i].yz;
            f(i, *p);
        }
    };
    if (nm == "x") vec(S.pos, 0); else if (nm == "y") vec(S.pos, 1); else if (nm == "z") vec(S.pos, 2);
    else if (nm == "vx") vec(S.vel, 0); else if (nm == "vy") vec(S.vel, 1); else if (nm == "vz") vec(S.vel, 2);
    else if (nm == "ax") vec(S.acc, 0); else if (nm == "ay") vec(S.acc, 1); else if (nm == "az") vec(S.acc, 2);
    else if (nm == "mass") sca(S.mass); else if (nm == "rho") sca(S.rho); else if (nm == "u") sca(S.u);
    else if (nm == "dudt") sca(S.dudt); else if (nm == "P") sca(S.P); else if (nm == "cs") sca(S.cs);
    else if (nm == "csig") sca(S.csig); else if (nm == "hh") sca(S.hh); else if (nm == "eps_work") sca(S.eps_work);
    else if (nm == "D") sca(S.D); else if (nm == "eps_act") sca(S.eps_act); else if (nm == "sigmax") sca(S.sigmax);
    else if (nm == "Pf") sca(S.Pf); else if (nm == "Rart") sca(S.Rart); else if (nm == "dscale") sca(S.dscale);
    else if (nm == "Sxx") sym(S.S, 0); else if (nm == "Syy") sym(S.S, 1); else if (nm == "Szz") sym(S.S, 2);
    else if (nm == "Sxy") sym(S.S, 3); else if (nm == "Sxz") sym(S.S, 4); else if (nm == "Syz") sym(S.S, 5);
    else if (nm == "dSxx") sym(S.dSdt, 0); else if (nm == "dSyy") sym(S.dSdt, 1); else if (nm == "dSzz") sym(S.dSdt, 2);
    else if (nm == "dSxy") sym(S.dSdt, 3); else if (nm == "dSxz") sym(S.dSdt, 4); else if (nm == "dSyz") sym(S.dSdt, 5);
    else return false;
    return true;
}

}  // namespace

extern "C" {

void* ref_create() { return new System(); }
void ref_destroy(void* p) { delete static_cast<System*>(p); }

int ref_add_material(void* p, const orc_material* m) {
    System& S = *static_cast<System*>(p);
    S.materials.push_back(to_material(m));
    return (int)S.materials.size() - 1;
}

void ref_set_params(void* p, const orc_params* q) {
    System& S = *static_cast<System*>(p);
    S.eta = q->eta; S.h_init = q->h_init; S.alpha = q->alpha; S.beta = q->beta; S.eps = q->eps;
    S.alpha_u = q->alpha_u; S.cfl = q->cfl; S.eps_as = q->eps_as; S.as_n = q->as_n;
    S.damage_on = q->damage_on != 0;
}

void ref_set_domain(void* p, double xl, double xh, int px, double yl, double yh, int py,
                    double zl, double zh, int pz) {
    static_cast<System*>(p)->set_domain(xl, xh, px != 0, yl, yh, py != 0, zl, zh, pz != 0);
}

void ref_add_many(void* p, int n, const double* x, const double* y, const double* z,
                  const double* vx, const double* vy, const double* vz, const double* m,
                  const double* u, const int32_t* mat, const uint8_t* fixed) {
    System& S = *static_cast<System*>(p);
    for (int i = 0; i < n; i++) {
        if (mat) S.cur_mat = mat[i];
        S.add({x[i], y[i], z[i]}, {vx[i], vy[i], vz[i]}, m[i], u[i], fixed ? fixed[i] != 0 : false);
    }
}

int ref_n(void* p) { return static_cast<System*>(p)->n; }

int ref_get_field(void* p, const char* name, double* out) {
    return with_field(*static_cast<System*>(p), name, [&](size_t i, double& v) { out[i] = v; }) ? 0 : -1;
}
int ref_set_field(void* p, const char* name, const double* in) {
    return with_field(*static_cast<System*>(p), name, [&](size_t i, double& v) { v = in[i]; }) ? 0 : -1;
}
void ref_get_mat(void* p, int32_t* out) {
    System& S = *static_cast<System*>(p);
    for (int i = 0; i < S.n; i++) out[i] = S.mat[i];
}
void ref_set_fixed(void* p, const uint8_t* in) {
    System& S = *static_cast<System*>(p);
    for (int i = 0; i < S.n; i++) S.fixed[i] = (char)in[i];
}

void ref_seed_damage(void* p, double dx, uint32_t seed) { static_cast<System*>(p)->seed_damage(dx, seed); }
void ref_init(void* p) { static_cast<System*>(p)->init(); }
double ref_timestep(void* p) { return static_cast<System*>(p)->timestep(); }
void ref_step(void* p, double dt) { static_cast<System*>(p)->step(dt); }
void ref_compute_density_h(void* p, int iters) { static_cast<System*>(p)->compute_density_h(iters); }
void ref_compute_forces(void* p) { static_cast<System*>(p)->compute_forces(); }
void ref_compute_strain_stress(void* p) { static_cast<System*>(p)->compute_strain_stress(); }
void ref_grow_damage(void* p, double dt) { static_cast<System*>(p)->grow_damage(dt); }
void ref_yield_limit(void* p, int i) { static_cast<System*>(p)->yield_limit(i); }
void ref_build_cells(void* p) { static_cast<System*>(p)->build_cells(); }

void ref_grid(void* p, int32_t nc[3], double cw[3], double* h_max) {
    System& S = *static_cast<System*>(p);
    for (int a = 0; a < 3; a++) { nc[a] = S.nc[a]; cw[a] = S.cw[a]; }
    *h_max = S.h_max;
}
int64_t ref_ncells(void* p) { return (int64_t)static_cast<System*>(p)->cells.size(); }
void ref_cell_csr(void* p, int32_t* start, int32_t* ids) {
    System& S = *static_cast<System*>(p);
    int32_t k = 0;
    for (size_t c = 0; c < S.cells.size(); c++) {
        start[c] = k;
        for (int j : S.cells[c]) ids[k++] = j;
    }
    start[S.cells.size()] = k;
}

int64_t ref_neighbors(void* p, int kind, int32_t* counts, int32_t* ids, int64_t cap) {
    System& S = *static_cast<System*>(p);
    int64_t total = 0;
    for (int i = 0; i < S.n; i++) {
        int cnt = 0;
        S.for_neighbors(i, [&](int j) {
            double r = norm(S.sep(S.pos[i], S.pos[j]));
            bool take;
            if (kind == ORC_NBR_DENSITY) {
                take = r < 2.0 * S.hh[i];
            } else {
                double hbar = 0.5 * (S.hh[i] + S.hh[j]);
                take = !(j == i || r >= 2.0 * hbar || r == 0);
            }
            if (take) {
                if (ids && total < cap) ids[total] = j;
                total++;
                cnt++;
            }
        });
        if (counts) counts[i] = cnt;
    }
    return total <= cap ? total : -total;
}

// eos.hpp known answers on arbitrary (rho, u) pairs
void ref_eos_batch(const orc_material* m, int n, const double* rho, const double* u, double* P,
                   double* cs) {
    Material M = to_material(m);
    for (int i = 0; i < n; i++) {
        P[i] = M.pressure(rho[i], u[i]);
        cs[i] = M.sound_speed(rho[i], u[i]);
    }
}
void ref_kernels(int n, const double* r, const double* h, double* W, double* dW) {
    for (int i = 0; i < n; i++) { W[i] = kW(r[i], h[i]); dW[i] = kdWdr(r[i], h[i]); }
}
void ref_eig_max(int n, const double* s6, double* out) {
    for (int i = 0; i < n; i++) {
        Sym3 s{s6[6 * i + 0], s6[6 * i + 1], s6[6 * i + 2], s6[6 * i + 3], s6[6 * i + 4], s6[6 * i + 5]};
        out[i] = eig_max(s);
    }
}
// material constructors of eos.hpp:42-50 (to pin the oracle's copies)
void ref_std_material(int which, orc_material* out) {
    Material m = which == 0 ? Material::iron() : which == 1 ? Material::basalt()
               : which == 2 ? Material::water() : Material::aluminum();
    std::memset(out, 0, sizeof(*out));
    out->type = m.type == Material::IDEAL ? ORC_IDEAL : ORC_TILLOTSON;
    out->gamma = m.gamma;
    out->rho0 = m.rho0; out->a = m.a; out->b = m.b; out->A = m.A; out->B = m.B;
    out->alpha = m.alpha; out->beta = m.beta; out->u0 = m.u0; out->uiv = m.uiv; out->ucv = m.ucv;
    out->G = m.G; out->Y = m.Y; out->Emod = m.Emod; out->wm = m.wm; out->wk = m.wk;
}

}  // extern "C"
