// serve.cpp -- continuous-batching server for impact runs behind the C ABI
// (sph_serve_*).  One engine context serves a stream of requests: a request
// (one impact: particles, parameters, flaw seeding, step count, arrival time)
// is admitted as soon as it has arrived and its particles fit the device-memory
// budget beside the resident impacts -- measured from the engine's own
// allocations and its per-particle footprint at the current neighbour-list
// capacity -- initialised in place while the residents keep their state, and
// advanced with every other resident impact (each with its own CFL dt and step
// limit) in chunks of device-controlled steps.  A finished request's fields are
// read back into host memory and its slot and memory released, which admits
// the next one.
//
// A pool of worker threads (half the host's hardware threads, at most 8)
// prepares queued requests on the host, oldest first (flaw seeding: the
// multi-flaw law draws ~N ln N thresholds) while the serving thread keeps the
// GPU busy, so admission costs only the upload and the impact's first
// evaluation.  All engine calls stay on the serving thread (the thread that
// calls sph_serve_poll); sph_serve_submit may be called from any thread.
//
// The campaign driver of the reference runs one gpu_ic process per impact
// (boundary_daemon.py:215-255); this server is the in-process replacement that
// keeps impacts of different sizes resident together.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "engine.hpp"

using dsph::EngineBase;
using dsph::SphError;

namespace dsph {
void set_error_message(const std::string& m);
}

namespace {

struct Req {
    int64_t id = 0;
    sph_params prm{};
    double lo[3]{}, hi[3]{};
    int32_t per[3]{};
    int64_t n = 0;
    std::vector<double> x, y, z, vx, vy, vz, mass, u, h0;
    std::vector<int32_t> mat;
    std::vector<uint8_t> fixed;
    int32_t flaws = SPH_SERVE_FLAWS_NONE;
    double flaw_dx = 0;
    uint32_t flaw_seed = 0;
    int64_t steps = 0;
    double arrival = 0;
    std::vector<sph_material> mats;  // the context's materials at submission
    // prepared by the worker
    std::vector<double> eps_act, feps;
    std::vector<int64_t> fptr;
    bool claimed = false;  // a worker is preparing it
    bool ready = false;
    // lifecycle (serving thread)
    int32_t state = SPH_SERVE_QUEUED;
    int impact = -1;
    double admitted = -1, finished = -1;
    std::vector<std::vector<double>> result;
};

const char* const kDefaultFields[] = {"x", "y", "z", "vx", "vy", "vz", "u", "rho", "P", "D"};

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// host-side flaw seeding of one request (the worker's job)
void prepare(Req& r) {
    if (r.flaws == SPH_SERVE_FLAWS_SINGLE) {
        r.eps_act.resize(r.n);
        dsph::seed_single_flaws(r.n, r.mat.data(), r.mats.data(), (int)r.mats.size(), r.flaw_dx, r.flaw_seed,
                                r.eps_act.data());
    } else if (r.flaws == SPH_SERVE_FLAWS_MULTI) {
        r.eps_act.resize(r.n);
        r.fptr.assign(r.n + 1, 0);
        double* fe = nullptr;
        int64_t nf = dsph::seed_multi_flaws(r.n, r.mat.data(), r.mats.data(), (int)r.mats.size(), r.flaw_dx,
                                            r.flaw_seed, r.fptr.data(), &fe, r.eps_act.data());
        r.feps.assign(fe, fe + nf);
        free(fe);
    }
}

}  // namespace

struct sph_server {
    sph_ctx* ctx = nullptr;
    double budget = 0;
    int chunk = 4;
    std::vector<std::string> fields;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::shared_ptr<Req>> queue;       // submitted, not admitted (submission order)
    std::map<int, std::shared_ptr<Req>> active;    // resident, by impact id
    std::map<int64_t, std::shared_ptr<Req>> all;   // every request not yet released
    int64_t next_id = 0;
    bool stop = false;
    std::vector<std::thread> workers;  // flaw seeding of queued requests, in parallel
    // statistics
    double particle_steps = 0, busy_s = 0;
    double admit_wait_s = 0;  // admission blocked on a request still being seeded
    double host_s = 0;        // admission, initialisation and retirement between rounds
    double first_arrival = -1, last_finish = -1;
    std::vector<double> latencies;
    int64_t peak_bytes = 0;

    void work() {
        std::unique_lock<std::mutex> lk(mu);
        while (!stop) {
            std::shared_ptr<Req> r;
            for (auto& q : queue)
                if (!q->claimed) { r = q; break; }
            if (!r) {
                cv.wait(lk);
                continue;
            }
            r->claimed = true;  // the oldest unclaimed request first
            lk.unlock();
            try {
                prepare(*r);
            } catch (...) {
                r->flaws = -1;  // reported when the request is admitted
            }
            lk.lock();
            r->ready = true;
            cv.notify_all();
        }
    }
};

namespace {

int guard(const std::function<void()>& f) {
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

void need(const void* p, const char* what) {
    if (!p) throw SphError(SPH_ERR_ARG, std::string("null pointer: ") + what);
}

// Makes the context's device current for the scope; restores the caller's.
struct DevScope {
    int prev = -1;
    explicit DevScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DevScope() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
        cudaGetLastError();
    }
};

std::shared_ptr<Req> find(sph_server* s, int64_t id) {
    auto it = s->all.find(id);
    if (it == s->all.end()) throw SphError(SPH_ERR_ARG, "unknown request id");
    return it->second;
}

// Admits arrived, prepared requests in submission order while they fit the
// budget (the first one always fits an empty server).  Returns how many.
int admit(sph_server* s, double now) {
    EngineBase& E = *s->ctx->eng;
    int admitted = 0;
    for (;;) {
        std::shared_ptr<Req> r;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->queue.empty()) break;
            r = s->queue.front();
            if (r->arrival > now) break;
            // the workers are behind: wait for them rather than idle the GPU on
            // a request that has arrived (bounded by the seeding time of one request)
            if (!r->ready) {
                const auto w0 = std::chrono::steady_clock::now();
                s->cv.wait(lk, [&] { return r->ready; });
                s->admit_wait_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
            }
        }
        const int64_t bytes = E.device_bytes_after_adding(r->n);
        if (!s->active.empty() && (double)bytes > s->budget) break;  // FIFO: wait for memory
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->queue.pop_front();
        }
        if (r->flaws < 0) {
            r->state = SPH_SERVE_FAILED;
            r->finished = now;
            continue;
        }
        const int b = E.impact_create(r->prm, r->lo, r->hi, r->per);
        E.impact_add_particles(b, r->n, r->x.data(), r->y.data(), r->z.data(), r->vx.data(), r->vy.data(),
                               r->vz.data(), r->mass.data(), r->u.data(), r->mat.data(), r->fixed.data());
        if (r->flaws != SPH_SERVE_FLAWS_NONE)
            E.impact_set_flaws(b, r->eps_act.data(), r->flaws == SPH_SERVE_FLAWS_MULTI ? r->fptr.data() : nullptr,
                               r->feps.data(), (int64_t)r->feps.size());
        if (!r->h0.empty()) E.impact_set_h0(b, r->h0.data());
        E.impact_set_step_limit(b, r->steps);
        // host copies are no longer needed once the impact holds them
        std::vector<double>().swap(r->eps_act);
        std::vector<double>().swap(r->feps);
        std::vector<int64_t>().swap(r->fptr);
        r->impact = b;
        r->admitted = now;
        r->state = SPH_SERVE_RESIDENT;
        s->active[b] = r;
        admitted++;
    }
    if (admitted) E.init();  // initialises only the newly admitted impacts
    s->peak_bytes = std::max<int64_t>(s->peak_bytes, E.device_bytes());
    return admitted;
}

}  // namespace

extern "C" {

int sph_serve_create(sph_ctx* ctx, double hbm_budget_bytes, int32_t chunk, const char* fields,
                     sph_server** out) {
    return guard([&] {
        need(out, "out");
        *out = nullptr;
        if (!ctx || !ctx->eng) throw SphError(SPH_ERR_ARG, "null context");
        if (!(hbm_budget_bytes > 0) || chunk < 1) throw SphError(SPH_ERR_ARG, "budget must be > 0 and chunk >= 1");
        auto s = std::make_unique<sph_server>();
        s->ctx = ctx;
        s->budget = hbm_budget_bytes;
        s->chunk = chunk;
        if (fields && *fields) {
            std::string f(fields), cur;
            for (char c : f + ",") {
                if (c == ',' || c == ' ') {
                    if (!cur.empty()) s->fields.push_back(cur);
                    cur.clear();
                } else {
                    cur += c;
                }
            }
        } else {
            for (const char* f : kDefaultFields) s->fields.push_back(f);
        }
        s->t0 = std::chrono::steady_clock::now();
        sph_server* raw = s.get();
        const unsigned hc = std::thread::hardware_concurrency();
        const int nw = (int)std::max(1u, std::min(8u, hc > 2 ? hc / 2 : 1u));
        for (int w = 0; w < nw; w++) s->workers.emplace_back([raw] { raw->work(); });
        *out = s.release();
    });
}

int sph_serve_destroy(sph_server* s) {
    return guard([&] {
        if (!s) return;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv.notify_all();
        for (auto& w : s->workers)
            if (w.joinable()) w.join();
        if (s->ctx && s->ctx->eng) {
            DevScope dv(s->ctx->device);
            for (auto& kv : s->active) {
                try {
                    s->ctx->eng->impact_remove(kv.first);
                } catch (...) {
                }
            }
        }
        delete s;
    });
}

int sph_serve_now(sph_server* s, double* t) {
    return guard([&] {
        need(s, "server");
        need(t, "t");
        *t = now_s(s->t0);
    });
}

int sph_serve_submit(sph_server* s, const sph_request* q, int64_t* id) {
    return guard([&] {
        need(s, "server");
        need(q, "request");
        need(q->params, "params");
        if (q->n < 1) throw SphError(SPH_ERR_ARG, "a request needs particles");
        need(q->x, "x"); need(q->y, "y"); need(q->z, "z");
        need(q->vx, "vx"); need(q->vy, "vy"); need(q->vz, "vz");
        need(q->mass, "mass"); need(q->u, "u");
        if (q->steps < 1) throw SphError(SPH_ERR_ARG, "steps must be >= 1");
        if (q->flaws < SPH_SERVE_FLAWS_NONE || q->flaws > SPH_SERVE_FLAWS_MULTI) throw SphError(SPH_ERR_ARG, "flaws");
        auto r = std::make_shared<Req>();
        r->prm = *q->params;
        for (int a = 0; a < 3; a++) {
            r->lo[a] = q->lo[a];
            r->hi[a] = q->hi[a];
            r->per[a] = q->periodic[a];
        }
        const int64_t n = q->n;
        r->n = n;
        auto cp = [n](std::vector<double>& d, const double* src) { d.assign(src, src + n); };
        cp(r->x, q->x); cp(r->y, q->y); cp(r->z, q->z);
        cp(r->vx, q->vx); cp(r->vy, q->vy); cp(r->vz, q->vz);
        cp(r->mass, q->mass); cp(r->u, q->u);
        if (q->h0) cp(r->h0, q->h0);
        r->mat.assign(n, 0);
        if (q->mat) r->mat.assign(q->mat, q->mat + n);
        r->fixed.assign(n, 0);
        if (q->fixed) r->fixed.assign(q->fixed, q->fixed + n);
        r->flaws = q->flaws;
        r->flaw_dx = q->flaw_dx;
        r->flaw_seed = q->flaw_seed;
        r->steps = q->steps;
        r->mats = s->ctx->eng->materials();
        for (int64_t i = 0; i < n; i++)
            if (r->mat[i] < 0 || r->mat[i] >= (int32_t)r->mats.size())
                throw SphError(SPH_ERR_ARG, "material id not in the context");
        const double now = now_s(s->t0);
        r->arrival = q->arrival >= 0 ? q->arrival : now;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r->id = s->next_id++;
            if (s->first_arrival < 0 || r->arrival < s->first_arrival) s->first_arrival = r->arrival;
            s->queue.push_back(r);
            s->all[r->id] = r;
        }
        s->cv.notify_all();
        if (id) *id = r->id;
    });
}

int sph_serve_poll(sph_server* s, double max_wait_s, int64_t* done_ids, int32_t cap, int32_t* ndone) {
    return guard([&] {
        need(s, "server");
        need(ndone, "ndone");
        *ndone = 0;
        DevScope dv(s->ctx->device);
        EngineBase& E = *s->ctx->eng;
        const double th0 = now_s(s->t0);
        admit(s, th0);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->host_s += now_s(s->t0) - th0;
        }
        if (s->active.empty()) {
            // idle: wait (bounded) for the next arrival
            double next = -1;
            {
                std::lock_guard<std::mutex> lk(s->mu);
                if (!s->queue.empty()) next = s->queue.front()->arrival;
            }
            if (next >= 0 && max_wait_s > 0) {
                const double d = std::min(max_wait_s, next - now_s(s->t0));
                if (d > 0) std::this_thread::sleep_for(std::chrono::duration<double>(d));
            }
            return;
        }
        int64_t steps = s->chunk;
        int64_t n_res = 0;
        for (auto& kv : s->active) {  // host step counts: no device round trip per impact
            steps = std::min<int64_t>(steps, kv.second->steps - E.impact_steps(kv.first));
            n_res += E.impact_n(kv.first);
        }
        steps = std::max<int64_t>(steps, 1);
        const double tb = now_s(s->t0);
        E.run((int)steps, 0.0);
        E.synchronize();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->busy_s += now_s(s->t0) - tb;
            s->particle_steps += (double)n_res * (double)steps;
        }
        // retire finished requests: results to host memory, slot and memory released
        const double tr0 = now_s(s->t0);
        struct HostTime {  // retirement time, added however the scope ends
            sph_server* s;
            double t0;
            ~HostTime() {
                std::lock_guard<std::mutex> lk(s->mu);
                s->host_s += now_s(s->t0) - t0;
            }
        } host_time{s, tr0};
        std::vector<int> fin;
        for (auto& kv : s->active)
            if (E.impact_steps(kv.first) >= kv.second->steps) fin.push_back(kv.first);
        for (int b : fin) {
            auto r = s->active[b];
            const int nf = (int)s->fields.size();
            r->result.assign(nf, std::vector<double>(r->n));
            std::vector<const char*> names(nf);
            std::vector<double*> outs(nf);
            for (int f = 0; f < nf; f++) {
                names[f] = s->fields[f].c_str();
                outs[f] = r->result[f].data();
            }
            E.read_fields(b, nf, names.data(), outs.data());
            E.impact_remove(b);
            s->active.erase(b);
            std::lock_guard<std::mutex> lk(s->mu);
            r->finished = now_s(s->t0);
            r->state = SPH_SERVE_DONE;
            s->latencies.push_back(r->finished - r->arrival);
            s->last_finish = std::max(s->last_finish, r->finished);
            if (done_ids && *ndone < cap) done_ids[*ndone] = r->id;
            (*ndone)++;
        }
    });
}

int sph_serve_request_info(sph_server* s, int64_t id, sph_serve_record* out) {
    return guard([&] {
        need(s, "server");
        need(out, "out");
        std::lock_guard<std::mutex> lk(s->mu);
        auto r = find(s, id);
        out->n = r->n;
        out->steps = r->steps;
        out->state = r->state;
        out->impact = r->impact;
        out->arrival = r->arrival;
        out->admitted = r->admitted;
        out->finished = r->finished;
    });
}

int sph_serve_result(sph_server* s, int64_t id, const char* field, double* out) {
    return guard([&] {
        need(s, "server");
        need(field, "field");
        need(out, "out");
        std::shared_ptr<Req> r;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r = find(s, id);
        }
        if (r->state != SPH_SERVE_DONE) throw SphError(SPH_ERR_STATE, "request not finished");
        for (size_t f = 0; f < s->fields.size(); f++)
            if (s->fields[f] == field) {
                std::memcpy(out, r->result[f].data(), sizeof(double) * (size_t)r->n);
                return;
            }
        throw SphError(SPH_ERR_ARG, std::string("field not kept by this server: ") + field);
    });
}

int sph_serve_release(sph_server* s, int64_t id) {
    return guard([&] {
        need(s, "server");
        std::lock_guard<std::mutex> lk(s->mu);
        auto r = find(s, id);
        if (r->state != SPH_SERVE_DONE && r->state != SPH_SERVE_FAILED)
            throw SphError(SPH_ERR_STATE, "only finished requests are released");
        s->all.erase(id);
    });
}

int sph_serve_stats(sph_server* s, sph_serve_summary* out) {
    return guard([&] {
        need(s, "server");
        need(out, "out");
        std::memset(out, 0, sizeof(*out));
        std::lock_guard<std::mutex> lk(s->mu);
        std::vector<double> lat = s->latencies;
        out->done = (int64_t)lat.size();
        out->queued = (int64_t)s->queue.size();
        out->resident = (int64_t)s->active.size();
        if (!lat.empty()) {
            std::sort(lat.begin(), lat.end());
            // linear interpolation between order statistics (numpy's default percentile)
            auto pct = [&](double p) {
                const double x = p / 100.0 * (double)(lat.size() - 1);
                const size_t i = (size_t)x;
                const double f = x - (double)i;
                return i + 1 < lat.size() ? lat[i] + f * (lat[i + 1] - lat[i]) : lat[i];
            };
            out->p50_latency_s = pct(50);
            out->p99_latency_s = pct(99);
            double m = 0;
            for (double v : lat) m += v;
            out->mean_latency_s = m / (double)lat.size();
        }
        out->particle_steps = s->particle_steps;
        const double wall = s->last_finish - s->first_arrival;
        out->throughput = wall > 0 ? s->particle_steps / wall : 0;
        out->busy_throughput = s->busy_s > 0 ? s->particle_steps / s->busy_s : 0;
        out->busy_s = s->busy_s;
        out->peak_device_bytes = (double)s->peak_bytes;
        out->admit_wait_s = s->admit_wait_s;
        out->host_s = s->host_s;
    });
}

}  // extern "C"
