// The request loop (sph_gb300/csrc/sph_serve.cpp) on the CPU, against a fake
// of the pool's C ABI: scenes are particle counts against a capacity, a step
// advances every resident scene's step count (taking a fixed wall time, as a
// GPU epoch would), admissions and removals apply at the next step as in the
// real pool.  Test infrastructure: tests/test_server_host.py compiles this
// file with sph_serve.cpp (g++) and runs its scenarios.
//
// Scenarios (argv[1]), each printing one JSON line:
//   complete   25 scenes of 100 particles x 30 steps, capacity 1000
//   capacity   10 such scenes with capacity 350 (three fit at once), and six
//              scenes with 10..60 steps: residency over time, joins mid-run
//   lookahead  small (100 steps), big, small with capacity 920: admission order
//   backpressure  ten scenes against a queue bound of three while nothing can
//              be admitted (capacity 0), then capacity for all of them
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../include/sph_gb300.h"

struct FakeScene {
    unsigned n, steps, done;
    bool resident, removed;
};

struct sph_pool {
    std::atomic<unsigned long long> capacity{0};
    std::map<int, FakeScene> scenes;
    int next = 1;
    std::string err;
    // what the tests inspect
    std::vector<unsigned> admitted_sizes;   // admission order
    unsigned max_resident = 0;
    unsigned long long max_used = 0;
    bool joined_mid_run = false;            // a scene became resident while another had progressed
    std::chrono::microseconds step_time{2000};
};

static unsigned long long used(const sph_pool* p)
{
    unsigned long long u = 0;
    for (auto& kv : p->scenes)
        if (!kv.second.removed) u += kv.second.n;
    return u;
}

extern "C" {

int sph_pool_add_scene(sph_pool* p, const sph_scene_desc*, const double*, const double*, unsigned n, const double*,
                       unsigned, unsigned steps, int* id)
{
    if (used(p) + n > p->capacity) {
        p->err = "pool full";
        return SPH_ERR_CAPACITY;
    }
    *id = p->next++;
    p->scenes[*id] = FakeScene{n, steps, 0, false, false};
    p->admitted_sizes.push_back(n);
    return SPH_OK;
}

int sph_pool_remove_scene(sph_pool* p, int id)
{
    auto it = p->scenes.find(id);
    if (it == p->scenes.end()) return SPH_ERR_INVALID;
    it->second.removed = true;
    return SPH_OK;
}

int sph_pool_step(sph_pool* p, int nsteps)
{
    // the re-layout: removals leave, admissions become resident
    bool progressed = false;
    for (auto it = p->scenes.begin(); it != p->scenes.end();) {
        if (it->second.removed) { it = p->scenes.erase(it); continue; }
        progressed |= it->second.resident && it->second.done > 0;
        ++it;
    }
    unsigned res = 0;
    for (auto& kv : p->scenes) {
        if (!kv.second.resident && progressed) p->joined_mid_run = true;
        kv.second.resident = true;
        ++res;
    }
    if (res > p->max_resident) p->max_resident = res;
    if (used(p) > p->max_used) p->max_used = used(p);
    for (int k = 0; k < nsteps; ++k)
        for (auto& kv : p->scenes)
            if (kv.second.done < kv.second.steps) ++kv.second.done;
    std::this_thread::sleep_for(p->step_time);
    return SPH_OK;
}

int sph_pool_poll(sph_pool* p, int* ids, int max, int* n)
{
    int k = 0;
    for (auto& kv : p->scenes)
        if (kv.second.resident && !kv.second.removed && kv.second.done >= kv.second.steps) {
            if (ids && k < max) ids[k] = kv.first;
            ++k;
        }
    *n = k;
    return SPH_OK;
}

int sph_pool_query(sph_pool* p, int id, sph_stats* out, int* done)
{
    auto it = p->scenes.find(id);
    if (it == p->scenes.end()) return SPH_ERR_INVALID;
    std::memset(out, 0, sizeof *out);
    out->steps = it->second.done;
    out->num_fluid = it->second.n;
    if (done) *done = it->second.done >= it->second.steps;
    return SPH_OK;
}

int sph_pool_download(sph_pool* p, int id, int, double* out)
{
    auto it = p->scenes.find(id);
    if (it == p->scenes.end()) return SPH_ERR_INVALID;
    for (unsigned i = 0; i < 3 * it->second.n; ++i) out[i] = (double)id;
    return SPH_OK;
}

const char* sph_pool_last_error(const sph_pool* p) { return p ? p->err.c_str() : "null pool"; }

}  // extern "C"

static void submit(sph_server* s, unsigned n, unsigned steps, std::vector<long long>* ids)
{
    std::vector<double> x(3 * (size_t)n, 0.0);
    sph_scene_desc d;
    std::memset(&d, 0, sizeof d);
    long long id = 0;
    if (sph_server_submit(s, &d, x.data(), nullptr, n, nullptr, 0, steps, &id) == SPH_OK) ids->push_back(id);
}

static void report(const char* name, sph_server* s, sph_pool* p)
{
    sph_server_stats st;
    sph_server_get_stats(s, &st);
    std::printf("{\"scenario\": \"%s\", \"submitted\": %llu, \"admitted\": %llu, \"completed\": %llu, \"queued\": %llu, "
                "\"resident\": %llu, \"particle_steps\": %.1f, \"p50\": %.6f, \"p99\": %.6f, \"max_resident\": %u, "
                "\"max_used\": %llu, \"capacity\": %llu, \"joined_mid_run\": %d, \"rejected\": %llu, "
                "\"queued_bytes\": %llu, \"order\": [",
                name, st.submitted, st.admitted, st.completed, st.queued, st.resident, st.particle_steps,
                st.p50_latency_s, st.p99_latency_s, p->max_resident, p->max_used, p->capacity.load(),
                p->joined_mid_run ? 1 : 0, st.rejected, st.queued_bytes);
    for (size_t k = 0; k < p->admitted_sizes.size(); ++k)
        std::printf("%s%u", k ? ", " : "", p->admitted_sizes[k]);
    std::printf("]}\n");
}

int main(int argc, char** argv)
{
    const std::string sc = argc > 1 ? argv[1] : "";
    sph_pool pool;
    sph_server_desc sd;
    sph_server_desc_init(&sd);
    sd.epoch_steps = 10;
    std::vector<long long> ids;
    sph_server* s = nullptr;
    if (sc == "complete") {
        pool.capacity = 1000;
        sd.keep_results = 1;
        sph_server_create(&pool, &sd, &s);
        for (int k = 0; k < 25; ++k) submit(s, 100, 30, &ids);
    } else if (sc == "capacity") {
        pool.capacity = 350;
        sph_server_create(&pool, &sd, &s);
        for (int k = 0; k < 10; ++k) submit(s, 100, 30, &ids);
        for (unsigned st = 10; st <= 60; st += 10) submit(s, 100, st, &ids);
    } else if (sc == "lookahead") {
        pool.capacity = 920;
        sph_server_create(&pool, &sd, &s);
        submit(s, 50, 100, &ids);
        submit(s, 900, 10, &ids);
        submit(s, 50, 10, &ids);
    } else if (sc == "backpressure") {
        pool.capacity = 0;
        sd.max_queued_bytes = 3ull * 100 * 3 * sizeof(double);
        sph_server_create(&pool, &sd, &s);
        for (int k = 0; k < 10; ++k) submit(s, 100, 30, &ids);
        report("backpressure_full", s, &pool);
        pool.capacity = 1000;
    } else {
        std::fprintf(stderr, "unknown scenario\n");
        return 2;
    }
    int idle = 0;
    sph_server_drain(s, 30.0, &idle);
    if (!idle) return 3;
    if (sc == "complete") {
        // every request reported complete once, with its kept result
        std::vector<sph_request_info> info(64);
        int n = 0;
        sph_server_completed(s, info.data(), 64, &n);
        int bad = 0;
        std::vector<double> x(300);
        for (int k = 0; k < n; ++k) {
            if (info[k].state != SPH_REQUEST_DONE || info[k].steps_done != 30 || !(info[k].latency_s > 0)) ++bad;
            if (sph_server_fetch(s, info[k].id, SPH_FIELD_POSITION, x.data()) != SPH_OK) ++bad;
        }
        int n2 = 0;
        sph_server_completed(s, info.data(), 64, &n2);
        std::printf("{\"reported\": %d, \"bad\": %d, \"reported_again\": %d}\n", n, bad, n2);
    }
    report(sc.c_str(), s, &pool);
    sph_server_destroy(s);
    return 0;
}
