// serve_harness.cpp -- the native server's host logic (deorbit_gb300/csrc/serve.cpp,
// sph_serve_* of libdeorbit_sph.so) driven on the CPU against a stand-in engine
// that counts steps the way the engine's step limits do and charges a fixed
// number of device bytes per particle.  Each case prints lines of "key values..."
// that tests/test_serve_host.py checks.
//
//   serve_harness <case>     case: fifo | oversized | chunks | future | seeding
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "engine.hpp"

namespace {

struct Counting : dsph::EngineBase {
    struct Imp { int64_t n = 0, steps = 0, limit = 0; bool committed = false; int64_t nflaws = -1; };
    std::map<int, Imp> imps;
    int next = 0;
    int64_t bytes_per_particle = 100;
    std::vector<int64_t> runs;             // chunk sizes
    std::vector<std::vector<int>> run_sets;  // residents of each chunk
    int inits = 0;
    std::vector<sph_material> mats;

    [[noreturn]] static void unused(const char* f) { throw std::runtime_error(std::string("unused: ") + f); }
    int64_t resident() const {
        int64_t n = 0;
        for (auto& kv : imps) n += kv.second.n;
        return n;
    }

    int precision() const override { return SPH_MIXED; }
    int add_material(const sph_material& m) override { mats.push_back(m); return (int)mats.size() - 1; }
    int impact_create(const sph_params&, const double*, const double*, const int32_t*) override {
        imps[next] = Imp();
        return next++;
    }
    int impact_create_generated(const sph_params&, std::shared_ptr<const dsph::GrazingLayout>) override { unused(__func__); }
    void impact_set_domain(int, const double*, const double*, const int32_t*) override { unused(__func__); }
    void impact_set_params(int, const sph_params&) override { unused(__func__); }
    sph_params impact_get_params(int) override { unused(__func__); }
    void impact_add_particles(int b, int64_t n, const double*, const double*, const double*, const double*,
                              const double*, const double*, const double*, const double*, const int32_t*,
                              const uint8_t*) override {
        imps.at(b).n += n;
    }
    void impact_seed_damage(int, double, uint32_t) override { unused(__func__); }
    int64_t impact_seed_flaws_multi(int, double, uint32_t) override { unused(__func__); }
    void impact_set_h0(int, const double*) override {}
    std::map<int, int64_t> flaw_log;  // impact -> flaws handed over (0: single-flaw eps_act only)
    void impact_set_flaws(int b, const double*, const int64_t* ptr, const double*, int64_t nflaws) override {
        imps.at(b).nflaws = ptr ? nflaws : 0;
        flaw_log[b] = imps.at(b).nflaws;
    }
    std::vector<sph_material> materials() override { return mats; }
    int64_t device_bytes() override { return resident() * bytes_per_particle; }
    int64_t device_bytes_after_adding(int64_t n) override { return (resident() + n) * bytes_per_particle; }
    void impact_set_time(int, double) override { unused(__func__); }
    void impact_set_step_limit(int b, int64_t s) override { imps.at(b).limit = s; }
    void impact_remove(int b) override { imps.erase(b); }
    int impact_count() override { return (int)imps.size(); }
    sph_impact_info impact_info(int b) override {
        sph_impact_info i{};
        i.n = imps.at(b).n;
        i.steps = imps.at(b).steps;
        return i;
    }
    void get_domain(int, double*, double*, int32_t*) override { unused(__func__); }
    void init() override {
        inits++;
        for (auto& kv : imps) kv.second.committed = true;
    }
    double timestep(int) override { unused(__func__); }
    void step(double) override { unused(__func__); }
    void run(int nsteps, double) override {
        runs.push_back(nsteps);
        std::vector<int> ids;
        for (auto& kv : imps) {
            ids.push_back(kv.first);
            kv.second.steps = std::min(kv.second.limit, kv.second.steps + nsteps);
        }
        run_sets.push_back(ids);
    }
    void compute_density_h(int) override { unused(__func__); }
    void compute_forces() override { unused(__func__); }
    void synchronize() override {}
    int64_t impact_n(int b) override { return imps.at(b).n; }
    int64_t impact_steps(int b) override { return imps.at(b).steps; }
    void read_field(int, const char*, double*) override { unused(__func__); }
    void write_field(int, const char*, const double*) override { unused(__func__); }
    void read_fields(int b, int nf, const char* const*, double* const* outs) override {
        for (int f = 0; f < nf; f++)
            for (int64_t i = 0; i < imps.at(b).n; i++) outs[f][i] = (double)(b * 1000 + f);
    }
    void write_fields(int, int, const char* const*, const double* const*) override { unused(__func__); }
    double step_fields(int, double, int, const char* const*, const double* const*, int, const char* const*,
                       double* const*) override {
        unused(__func__);
        return 0;
    }
    void read_mat(int, int32_t*) override { unused(__func__); }
    void read_fixed(int, uint8_t*) override { unused(__func__); }
    void write_fixed(int, const uint8_t*) override { unused(__func__); }
    sph_conservation conservation(int) override { unused(__func__); }
    void diagnostics(int, int, int, double, double*) override { unused(__func__); }
    void eos_eval(int, int64_t, const double*, const double*, double*, double*) override { unused(__func__); }
    void debug_ref_cells(int, int32_t*, double*, int32_t*, int64_t, int32_t*) override { unused(__func__); }
    int64_t debug_neighbors(int, int, int32_t*, int32_t*, int64_t) override { unused(__func__); }
    int64_t debug_flaws(int, int64_t*, double*, int64_t) override { unused(__func__); }
    void set_tuning(int, double) override { unused(__func__); }
    void set_option(const char*, double) override { unused(__func__); }
    double get_option(const char*) override { unused(__func__); }
    int64_t launches() override { return 0; }
    void phase_times(double*) override { unused(__func__); }
    void set_profiling(int) override { unused(__func__); }
    void kernel_stats(int, double*, int64_t*) override { unused(__func__); }
    void kernel_stats_reset() override { unused(__func__); }
    void event_record(int) override { unused(__func__); }
    double event_elapsed(int, int) override { unused(__func__); }
};

struct Ctx {
    sph_ctx ctx;
    Counting* eng;
    Ctx() {
        auto e = std::make_unique<Counting>();
        eng = e.get();
        ctx.eng = std::move(e);
        sph_material m{};
        m.type = SPH_EOS_TILLOTSON;
        m.wm = 9.0;
        m.wk = 4.0e35;
        eng->add_material(m);
    }
};

void ok(int rc) {
    if (rc != SPH_OK) {
        std::fprintf(stderr, "error %d: %s\n", rc, sph_last_error());
        std::exit(2);
    }
}

struct Particles {
    std::vector<double> x, zero;
    std::vector<int32_t> mat;
    explicit Particles(int64_t n) : x(n), zero(n, 0.0), mat(n, 0) {
        for (int64_t i = 0; i < n; i++) x[i] = (double)i;
    }
};

int64_t submit(sph_server* s, int64_t n, int64_t steps, double arrival, int flaws = SPH_SERVE_FLAWS_NONE) {
    static sph_params p{};
    sph_params_default(&p);
    Particles q(n);
    sph_request r{};
    r.params = &p;
    for (int a = 0; a < 3; a++) { r.lo[a] = -1; r.hi[a] = (double)n + 1; }
    r.n = n;
    r.x = r.y = r.z = q.x.data();
    r.vx = r.vy = r.vz = r.u = q.zero.data();
    r.mass = q.zero.data();
    r.mat = q.mat.data();
    r.flaws = flaws;
    r.flaw_dx = 1.0;
    r.flaw_seed = 12345;
    r.steps = steps;
    r.arrival = arrival;
    int64_t id = -1;
    ok(sph_serve_submit(s, &r, &id));
    return id;  // the caller's arrays may go away: the server copied them
}

sph_serve_record info(sph_server* s, int64_t id) {
    sph_serve_record r{};
    ok(sph_serve_request_info(s, id, &r));
    return r;
}

// polls until every request is done; returns the finishing order
std::vector<int64_t> drain(sph_server* s, int64_t total) {
    std::vector<int64_t> order;
    int64_t ids[64];
    for (int guard = 0; guard < 100000 && (int64_t)order.size() < total; guard++) {
        int32_t nd = 0;
        ok(sph_serve_poll(s, 0.01, ids, 64, &nd));
        for (int i = 0; i < nd; i++) order.push_back(ids[i]);
    }
    return order;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 1;
    const std::string c = argv[1];
    Ctx C;
    sph_server* s = nullptr;
    ok(sph_serve_create(&C.ctx, 2500.0 * 100, 4, "x,rho", &s));
    if (c == "fifo") {
        // three requests of 1000 particles, a budget of 2500: the third waits
        int64_t a = submit(s, 1000, 6, 0.0), b = submit(s, 1000, 6, 0.0), d = submit(s, 1000, 6, 0.0);
        int64_t ids[8];
        int32_t nd = 0;
        ok(sph_serve_poll(s, 0.0, ids, 8, &nd));
        std::printf("after_first_poll %d %d %d\nresident %zu\n", info(s, a).state, info(s, b).state,
                    info(s, d).state, C.eng->imps.size());
        auto order = drain(s, 3);
        std::printf("order %lld %lld %lld\n", (long long)order[0], (long long)order[1], (long long)order[2]);
        std::printf("third_admitted_after %d\n",
                    info(s, d).admitted >= std::max(info(s, a).finished, info(s, b).finished) ? 1 : 0);
    } else if (c == "oversized") {
        int64_t big = submit(s, 10000, 3, 0.0), small = submit(s, 10, 3, 0.0);
        int64_t ids[8];
        int32_t nd = 0;
        ok(sph_serve_poll(s, 0.0, ids, 8, &nd));
        std::printf("after_first_poll %d %d\n", info(s, big).state, info(s, small).state);
        drain(s, 2);
        std::printf("small_after_big %d\n", info(s, small).admitted >= info(s, big).finished ? 1 : 0);
    } else if (c == "chunks") {
        int64_t r1 = submit(s, 100, 5, 0.0), r2 = submit(s, 100, 9, 0.0);
        drain(s, 2);
        std::printf("runs");
        for (auto v : C.eng->runs) std::printf(" %lld", (long long)v);
        sph_serve_summary st{};
        ok(sph_serve_stats(s, &st));
        std::printf("\nparticle_steps %.0f\ndone %lld\nresidents_left %zu\n", st.particle_steps,
                    (long long)st.done, C.eng->imps.size());
        std::vector<double> x(100), rho(100);
        ok(sph_serve_result(s, r1, "x", x.data()));
        ok(sph_serve_result(s, r1, "rho", rho.data()));
        std::printf("result_fields %.0f %.0f\n", x[0], rho[99]);
        std::printf("unkept_field_rc %d\n", sph_serve_result(s, r2, "vx", x.data()));
        ok(sph_serve_release(s, r1));
        sph_serve_record gone{};
        std::printf("released_rc %d\n", sph_serve_request_info(s, r1, &gone));
    } else if (c == "future") {
        double now = 0;
        ok(sph_serve_now(s, &now));
        int64_t late = submit(s, 100, 2, now + 0.05);
        int64_t ids[8];
        int32_t nd = 0;
        ok(sph_serve_poll(s, 0.0, ids, 8, &nd));
        std::printf("not_yet %d\nruns %zu\n", info(s, late).state, C.eng->runs.size());
        drain(s, 1);
        sph_serve_summary st{};
        ok(sph_serve_stats(s, &st));
        std::printf("admitted_after_arrival %d\ndone %lld\np50_nonneg %d\nparticle_steps %.0f\n",
                    info(s, late).admitted >= info(s, late).arrival ? 1 : 0, (long long)st.done,
                    st.p50_latency_s >= 0 ? 1 : 0, st.particle_steps);
    } else if (c == "seeding") {
        // flaws are seeded by the worker before admission and handed to the engine
        int64_t a = submit(s, 500, 2, 0.0, SPH_SERVE_FLAWS_MULTI);
        int64_t b = submit(s, 200, 2, 0.0, SPH_SERVE_FLAWS_SINGLE);
        int64_t ids[8];
        int32_t nd = 0;
        ok(sph_serve_poll(s, 0.0, ids, 8, &nd));
        const int ia = info(s, a).impact, ib = info(s, b).impact;
        std::printf("flaws %lld %lld\n", (long long)C.eng->flaw_log.at(ia), (long long)C.eng->flaw_log.at(ib));
        drain(s, 2);
    }
    ok(sph_serve_destroy(s));
    return 0;
}
