// euler_ref_shim.cpp -- C entry points over the reference's own CPU Euler
// solver (TEST ONLY).
//
// Compiled by oracle/Makefile from the UNMODIFIED reference source
// hydrocodes/euler/hydro_cpu.cpp (and the hydrocodes/common/eos.hpp it
// includes), read where it lies; nothing from the reference is copied into
// this repository.  The reference's driver `main` is renamed so that its
// solver functions (Lop, vonmises, grow_damage, update_af, maxspeed,
// step_rk2, implicit_visc) and file-scope settings can be driven on arbitrary grids.  The
// resulting oracle/_ref/libeulerref.so lets the golden-vector generator and
// the oracle tests run the reference and the C oracle on the same inputs.
#define main deorbit_hydro_cpu_main
#include "hydro_cpu.cpp"
#undef main

#include <cstring>
#include <string>

#include "euler_oracle.h"  // only for the plain-data orc_material / eorc_params layouts

namespace {

struct RefGrid {
    Grid g;
    DU d;
    orc_material mat;
    eorc_params prm;
    std::vector<double> ref_r0, ref_p0;  // this grid's hydrostatic reference (set_ref), empty when off
    long visc_iters = 0;                 // this grid's share of the reference's VISC_IT counter
    RefGrid(int nx, int ny, int nz, double dx) : g(nx, ny, nz, dx), d(nx * ny * nz) {}
};

Material to_material(const orc_material* m) {
    Material r;
    r.type = m->type == ORC_IDEAL ? Material::IDEAL : Material::TILLOTSON;
    r.gamma = m->gamma;
    r.rho0 = m->rho0; r.a = m->a; r.b = m->b; r.A = m->A; r.B = m->B;
    r.alpha = m->alpha; r.beta = m->beta; r.u0 = m->u0; r.uiv = m->uiv; r.ucv = m->ucv;
    r.G = m->G; r.Y = m->Y; r.Emod = m->Emod; r.wm = m->wm; r.wk = m->wk;
    return r;
}

// The reference keeps material and switches in file-scope variables: load
// this grid's before every call.
void load(const RefGrid* R) {
    MAT = to_material(&R->mat);
    GAM = R->mat.gamma;
    const eorc_params& p = R->prm;
    GZ = p.gz; TDEC = p.tdec; ETA_AF = p.eta_af; C_ACT = p.c_act; P_COH = p.p_coh; P_ACT = p.p_act;
    RHO_CFL = p.rho_cfl; DAMP = p.damp; RHO_VAC = p.rho_vac; AXISYM = p.axisym != 0; ROCK = p.rock != 0;
    Y_I0 = p.y_i0; MU_I = p.mu_i; MU_D = p.mu_d; Y_D0 = p.y_d0; Y_M = p.y_m; Y_BINGHAM = p.y_bingham;
    VISC_IMP = p.visc_imp != 0;
    VOID_CONS = p.void_cons != 0;
    VOID_AMB = p.void_amb;
    REF_R0 = R->ref_r0;
    REF_P0 = R->ref_p0;
    AF_REG = p.af_reg != 0; C_REG = p.c_reg; AF_SAT = p.af_sat; AF_PREL = p.af_prel != 0;
    AF_SEEDDP = p.af_seeddp != 0;
}

std::vector<double>* field(Grid& g, const std::string& nm) {
    if (nm == "r") return &g.r;
    if (nm == "mu") return &g.mu;
    if (nm == "mv") return &g.mv;
    if (nm == "mw") return &g.mw;
    if (nm == "E") return &g.E;
    if (nm == "Sxx") return &g.Sxx;
    if (nm == "Syy") return &g.Syy;
    if (nm == "Szz") return &g.Szz;
    if (nm == "Sxy") return &g.Sxy;
    if (nm == "Sxz") return &g.Sxz;
    if (nm == "Syz") return &g.Syz;
    if (nm == "D") return &g.D;
    if (nm == "af") return &g.af;
    if (nm == "rc") return &g.rc;
    if (nm == "vib") return &g.vib;
    if (nm == "Pmax") return &g.Pmax;
    return nullptr;
}

std::vector<double>* rhs(DU& d, const std::string& nm) {
    if (nm == "r") return &d.r;
    if (nm == "mu") return &d.mu;
    if (nm == "mv") return &d.mv;
    if (nm == "mw") return &d.mw;
    if (nm == "E") return &d.E;
    if (nm == "Sxx") return &d.Sxx;
    if (nm == "Syy") return &d.Syy;
    if (nm == "Szz") return &d.Szz;
    if (nm == "Sxy") return &d.Sxy;
    if (nm == "Sxz") return &d.Sxz;
    if (nm == "Syz") return &d.Syz;
    if (nm == "D") return &d.D;
    if (nm == "rc") return &d.rc;
    if (nm == "vib") return &d.vib;
    return nullptr;
}

// The reference's own defaults of its settings, read once at load time
// before any grid has changed them.
eorc_params capture_defaults() {
    eorc_params p;
    std::memset(&p, 0, sizeof p);
    p.gz = GZ; p.tdec = TDEC; p.eta_af = ETA_AF; p.c_act = C_ACT; p.p_coh = P_COH; p.p_act = P_ACT;
    p.rho_cfl = RHO_CFL; p.damp = DAMP; p.rho_vac = RHO_VAC; p.axisym = AXISYM; p.rock = ROCK;
    p.y_i0 = Y_I0; p.mu_i = MU_I; p.mu_d = MU_D; p.y_d0 = Y_D0; p.y_m = Y_M; p.y_bingham = Y_BINGHAM;
    p.af_reg = AF_REG; p.c_reg = C_REG; p.af_sat = AF_SAT; p.af_prel = AF_PREL; p.af_seeddp = AF_SEEDDP;
    p.void_amb = VOID_AMB;
    p.void_cons = VOID_CONS;
    p.visc_imp = VISC_IMP;
    return p;
}
const eorc_params kDefaults = capture_defaults();

}  // namespace

extern "C" {

// The reference's default settings (to check the oracle's defaults against).
void eref_params_default(eorc_params* p) { *p = kDefaults; }

void* eref_create(int nx, int ny, int nz, double dx) {
    RefGrid* R = new RefGrid(nx, ny, nz, dx);
    std::memset(&R->mat, 0, sizeof R->mat);  // the reference's default MAT: ideal gas, gamma 1.4
    R->mat.type = ORC_IDEAL;
    R->mat.gamma = 1.4;
    R->prm = kDefaults;
    return R;
}
void eref_destroy(void* h) { delete (RefGrid*)h; }
void eref_set_material(void* h, const orc_material* m) { ((RefGrid*)h)->mat = *m; }
void eref_set_params(void* h, const eorc_params* p) { ((RefGrid*)h)->prm = *p; }
double* eref_field(void* h, const char* name) {
    auto* v = field(((RefGrid*)h)->g, name);
    return v ? v->data() : nullptr;
}
double* eref_rhs(void* h, const char* name) {
    auto* v = rhs(((RefGrid*)h)->d, name);
    return v ? v->data() : nullptr;
}
void eref_lop(void* h) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    Lop(R->g, R->d);
}
void eref_vonmises(void* h, int reg) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    vonmises(R->g, reg != 0);
}
void eref_grow_damage(void* h, double dt) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    grow_damage(R->g, dt);
}
void eref_update_af(void* h, double dt) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    update_af(R->g, dt);
}
double eref_maxspeed(void* h) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    return maxspeed(R->g);
}
void eref_step_rk2(void* h, double dt) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    const long it0 = VISC_IT;
    step_rk2(R->g, dt);
    R->visc_iters += VISC_IT - it0;
}
void eref_implicit_visc(void* h, double dt) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    const long it0 = VISC_IT;
    implicit_visc(R->g, dt);
    R->visc_iters += VISC_IT - it0;
}
long eref_visc_iters(void* h) { return ((RefGrid*)h)->visc_iters; }
int eref_run(void* h, double cfl, double t_end, int max_steps, double* t_out) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    double t = 0;
    int s = 0;
    const long it0 = VISC_IT;
    while (t < t_end && (max_steps < 0 || s < max_steps)) {  // the drivers' loop, hydro_cpu.cpp:452
        double dt = cfl * R->g.dx / maxspeed(R->g);
        if (t + dt > t_end) dt = t_end - t;
        step_rk2(R->g, dt);
        t += dt;
        s++;
    }
    R->visc_iters += VISC_IT - it0;
    if (t_out) *t_out = t;
    return s;
}
void eref_set_ref(void* h) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    set_ref(R->g);
    R->ref_r0 = REF_R0;
    R->ref_p0 = REF_P0;
}
void eref_clear_ref(void* h) {
    RefGrid* R = (RefGrid*)h;
    R->ref_r0.clear();
    R->ref_p0.clear();
}
// The reference driver itself (its renamed main): a mode with its command
// line, printing to stdout as the reference binary does.
int eref_main(int argc, char** argv) { return deorbit_hydro_cpu_main(argc, argv); }

double eref_pcell(void* h, int c) {
    RefGrid* R = (RefGrid*)h;
    load(R);
    return Pcell(R->g, c);
}

}  // extern "C"
