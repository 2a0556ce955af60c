// Request loop serving DFSPH scenes from one device-resident pool (host side,
// above the C ABI; no counterpart in the reference, which runs one scene per
// process).
//
// Clients submit scenes from any thread (sph_server_submit copies them and
// returns at once).  One driver thread owns the pool's stepping and repeats:
//
//   1. enqueue one epoch of pool steps (CUDA graph launches; the pool first
//      applies the admissions and removals made since the last epoch);
//   2. while the GPU runs the epoch, admit queued requests in arrival order
//      with a look-ahead (a request that does not fit the pool's capacity
//      stays queued and later, smaller ones may pass it): host-side work only
//      (grid planning, staging), so it overlaps the device;
//   3. poll the pool (waits for the epoch), retire completed scenes (their
//      latency is completion minus submission; with keep_results their final
//      positions and velocities are copied out first) and remove them.
//
// Requests that arrive while others run join at the next epoch boundary, so
// resident scenes keep stepping while the scene set changes (continuous
// batching); each scene's results are those of the scene alone (the pool's
// reductions do not depend on what else is resident).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/sph_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long long id = 0;
    sph_scene_desc d{};
    std::vector<double> x, v, b;
    unsigned n = 0, nb = 0, steps = 0;
    Clock::time_point t_submit;
    size_t bytes() const { return (x.size() + v.size() + b.size()) * sizeof(double); }
};

struct Record {
    sph_request_info info{};
    double t_submit = 0.0;     // seconds on the server's clock
    std::vector<double> x, v;  // final state (keep_results)
};

}  // namespace

struct sph_server {
    sph_pool* pool = nullptr;
    sph_server_desc desc{};
    Clock::time_point t0;

    std::mutex m;                       // everything below
    std::condition_variable cv;         // submissions, stop, progress
    std::deque<Request> queue;
    std::unordered_map<int, long long> resident;    // pool scene id -> request id
    std::unordered_map<long long, Record> records;  // every request by id
    std::vector<long long> completed_unread;
    std::vector<double> latencies;
    long long next_id = 1;
    unsigned long long submitted = 0, admitted = 0, completed = 0, failed = 0, epochs = 0, rejected = 0;
    unsigned long long queued_bytes = 0;   // host bytes of the queued requests
    double particle_steps_done = 0.0;
    bool stop = false;
    bool driver_failed = false;
    std::string err;
    std::thread driver;

    void run();
    bool admit_locked();
    void retire(int pool_id, std::unique_lock<std::mutex>& lk);
};

namespace {

void set_err(sph_server* s, const std::string& m)
{
    s->err = m;
}

}  // namespace

// Admission: the first `lookahead` queued requests, in arrival order, each
// admitted if it fits the pool now.  Returns whether any was admitted.
bool sph_server::admit_locked()
{
    bool any = false;
    unsigned tried = 0;
    for (auto it = queue.begin(); it != queue.end() && tried < desc.lookahead;) {
        ++tried;
        Request& r = *it;
        int sid = -1;
        const int rc = sph_pool_add_scene(pool, &r.d, r.x.data(), r.v.empty() ? nullptr : r.v.data(), r.n,
                                          r.nb ? r.b.data() : nullptr, r.nb, r.steps, &sid);
        if (rc == SPH_ERR_CAPACITY) {
            ++it;
            continue;
        }
        Record& rec = records[r.id];
        if (rc != SPH_OK) {
            rec.info.state = SPH_REQUEST_FAILED;
            ++failed;
            completed_unread.push_back(r.id);
        } else {
            rec.info.state = SPH_REQUEST_RESIDENT;
            resident[sid] = r.id;
            ++admitted;
            any = true;
        }
        queued_bytes -= r.bytes();
        it = queue.erase(it);
    }
    return any;
}

// A completed scene: statistics, latency, optional copy of its state, removal.
void sph_server::retire(int pool_id, std::unique_lock<std::mutex>& lk)
{
    auto it = resident.find(pool_id);
    if (it == resident.end()) return;
    const long long rid = it->second;
    resident.erase(it);
    sph_stats st{};
    int done = 0;
    sph_pool_query(pool, pool_id, &st, &done);
    const double lat = std::chrono::duration<double>(Clock::now() - t0).count() - records[rid].t_submit;
    const unsigned n = records[rid].info.num_fluid;
    std::vector<double> x, v;
    bool kept = false;
    if (desc.keep_results && n) {
        x.resize(3 * (size_t)n);
        v.resize(3 * (size_t)n);
        lk.unlock();  // downloads wait for the device; submitters need not
        kept = sph_pool_download(pool, pool_id, SPH_FIELD_POSITION, x.data()) == SPH_OK &&
               sph_pool_download(pool, pool_id, SPH_FIELD_VELOCITY, v.data()) == SPH_OK;
        lk.lock();
    }
    Record& rec = records[rid];  // (the map may have grown meanwhile)
    rec.info.state = SPH_REQUEST_DONE;
    rec.info.steps_done = st.steps;
    rec.info.status = st.status;
    rec.info.latency_s = lat;
    if (kept) {
        rec.x.swap(x);
        rec.v.swap(v);
    }
    sph_pool_remove_scene(pool, pool_id);
    latencies.push_back(lat);
    particle_steps_done += (double)n * (double)st.steps;
    ++completed;
    completed_unread.push_back(rid);
}

void sph_server::run()
{
    std::vector<int> done(256);
    std::unique_lock<std::mutex> lk(m);
    for (;;) {
        admit_locked();
        if (resident.empty()) {
            if (stop) break;
            cv.wait_for(lk, std::chrono::milliseconds(5));
            continue;
        }
        if (stop) break;
        // 1. the epoch (admissions made above become resident first)
        lk.unlock();
        int rc = sph_pool_step(pool, (int)desc.epoch_steps);
        lk.lock();
        if (rc != SPH_OK) {
            driver_failed = true;
            set_err(this, std::string("sph_pool_step: ") + sph_pool_last_error(pool));
            break;
        }
        ++epochs;
        // 2. admissions while the epoch runs on the device
        admit_locked();
        // 3. completed scenes (the poll waits for the epoch)
        int nd = 0;
        lk.unlock();
        rc = sph_pool_poll(pool, done.data(), (int)done.size(), &nd);
        if (rc == SPH_OK && nd > (int)done.size()) {
            done.resize((size_t)nd);
            rc = sph_pool_poll(pool, done.data(), (int)done.size(), &nd);
        }
        lk.lock();
        if (rc != SPH_OK) {
            driver_failed = true;
            set_err(this, std::string("sph_pool_poll: ") + sph_pool_last_error(pool));
            break;
        }
        for (int k = 0; k < nd && k < (int)done.size(); ++k) retire(done[k], lk);
        cv.notify_all();
    }
    cv.notify_all();
}

extern "C" {

int sph_server_desc_init(sph_server_desc* d)
{
    if (!d) return SPH_ERR_INVALID;
    std::memset(d, 0, sizeof *d);
    d->epoch_steps = 10;
    d->lookahead = 8;
    d->keep_results = 0;
    return SPH_OK;
}

int sph_server_create(sph_pool* pool, const sph_server_desc* desc, sph_server** out)
{
    if (!pool || !out) return SPH_ERR_INVALID;
    *out = nullptr;
    sph_server* s = new (std::nothrow) sph_server();
    if (!s) return SPH_ERR_INVALID;
    if (desc) s->desc = *desc;
    else sph_server_desc_init(&s->desc);
    if (s->desc.epoch_steps == 0 || s->desc.lookahead == 0) {
        delete s;
        return SPH_ERR_INVALID;
    }
    s->pool = pool;
    s->t0 = Clock::now();
    try {
        s->driver = std::thread([s] { s->run(); });
    } catch (...) {
        delete s;
        return SPH_ERR_INVALID;
    }
    *out = s;
    return SPH_OK;
}

int sph_server_destroy(sph_server* s)
{
    if (!s) return SPH_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->driver.joinable()) s->driver.join();
    delete s;
    return SPH_OK;
}

int sph_server_submit(sph_server* s, const sph_scene_desc* d, const double* x, const double* v, unsigned n,
                      const double* bx, unsigned nb, unsigned steps, long long* request_id)
{
    if (!s || !d || !request_id || !x || !n || (nb && !bx)) return SPH_ERR_INVALID;
    Request r;
    try {
        r.d = *d;
        r.x.assign(x, x + 3 * (size_t)n);
        if (v) r.v.assign(v, v + 3 * (size_t)n);
        if (nb) r.b.assign(bx, bx + 3 * (size_t)nb);
    } catch (...) {
        return SPH_ERR_CAPACITY;
    }
    r.n = n;
    r.nb = nb;
    r.steps = steps;
    r.t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->m);
        if (s->stop || s->driver_failed) {
            set_err(s, "the server has stopped");
            return SPH_ERR_INVALID;
        }
        if (s->desc.max_queued_bytes && s->queued_bytes + r.bytes() > s->desc.max_queued_bytes) {
            ++s->rejected;
            set_err(s, "request queue full (max_queued_bytes)");
            return SPH_ERR_CAPACITY;
        }
        s->queued_bytes += r.bytes();
        r.id = s->next_id++;
        Record& rec = s->records[r.id];
        rec.info.id = r.id;
        rec.info.state = SPH_REQUEST_QUEUED;
        rec.info.num_fluid = n;
        rec.info.steps = steps;
        rec.t_submit = std::chrono::duration<double>(r.t_submit - s->t0).count();
        *request_id = r.id;
        s->queue.push_back(std::move(r));
        ++s->submitted;
    }
    s->cv.notify_all();
    return SPH_OK;
}

int sph_server_completed(sph_server* s, sph_request_info* out, int max, int* n)
{
    if (!s || !n || (max > 0 && !out)) return SPH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->m);
    int k = 0;
    for (; k < max && k < (int)s->completed_unread.size(); ++k) out[k] = s->records[s->completed_unread[k]].info;
    s->completed_unread.erase(s->completed_unread.begin(), s->completed_unread.begin() + k);
    *n = k;
    return SPH_OK;
}

int sph_server_query(sph_server* s, long long id, sph_request_info* out)
{
    if (!s || !out) return SPH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->m);
    auto it = s->records.find(id);
    if (it == s->records.end()) {
        set_err(s, "unknown request id");
        return SPH_ERR_INVALID;
    }
    *out = it->second.info;
    return SPH_OK;
}

int sph_server_fetch(sph_server* s, long long id, int field, double* out)
{
    if (!s || !out || (field != SPH_FIELD_POSITION && field != SPH_FIELD_VELOCITY)) return SPH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->m);
    auto it = s->records.find(id);
    if (it == s->records.end() || it->second.info.state != SPH_REQUEST_DONE) {
        set_err(s, "request has not completed");
        return SPH_ERR_INVALID;
    }
    const std::vector<double>& src = field == SPH_FIELD_POSITION ? it->second.x : it->second.v;
    if (src.empty()) {
        set_err(s, "no kept result (keep_results off)");
        return SPH_ERR_INVALID;
    }
    std::memcpy(out, src.data(), src.size() * sizeof(double));
    return SPH_OK;
}

int sph_server_release(sph_server* s, long long id)
{
    if (!s) return SPH_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->m);
    auto it = s->records.find(id);
    if (it == s->records.end()) return SPH_ERR_INVALID;
    std::vector<double>().swap(it->second.x);
    std::vector<double>().swap(it->second.v);
    return SPH_OK;
}

int sph_server_drain(sph_server* s, double timeout_s, int* idle)
{
    if (!s || !idle) return SPH_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->m);
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    while (!(s->queue.empty() && s->resident.empty()) && !s->driver_failed && Clock::now() < until)
        s->cv.wait_until(lk, until);
    *idle = s->queue.empty() && s->resident.empty() ? 1 : 0;
    return s->driver_failed ? SPH_ERR_CUDA : SPH_OK;
}

int sph_server_get_stats(sph_server* s, sph_server_stats* out)
{
    if (!s || !out) return SPH_ERR_INVALID;
    std::memset(out, 0, sizeof *out);
    std::vector<std::pair<int, long long>> res;
    std::vector<double> lat;
    {
        std::lock_guard<std::mutex> lk(s->m);
        out->submitted = s->submitted;
        out->admitted = s->admitted;
        out->completed = s->completed;
        out->failed = s->failed;
        out->queued = s->queue.size();
        out->rejected = s->rejected;
        out->queued_bytes = s->queued_bytes;
        out->resident = s->resident.size();
        out->epochs = s->epochs;
        out->particle_steps = s->particle_steps_done;
        res.assign(s->resident.begin(), s->resident.end());
        lat = s->latencies;
        for (auto& q : res) q.second = (long long)s->records[q.second].info.num_fluid;
    }
    out->wall_s = std::chrono::duration<double>(Clock::now() - s->t0).count();
    // steps resident scenes have run so far
    for (auto& q : res) {
        sph_stats st{};
        int done = 0;
        if (sph_pool_query(s->pool, q.first, &st, &done) == SPH_OK) out->particle_steps += (double)q.second * st.steps;
    }
    out->particle_steps_per_s = out->wall_s > 0 ? out->particle_steps / out->wall_s : 0.0;
    if (!lat.empty()) {
        std::sort(lat.begin(), lat.end());
        // linear interpolation between closest ranks
        auto pct = [&](double p) {
            const double r = p / 100.0 * (double)(lat.size() - 1);
            const size_t lo = (size_t)r, hi = std::min(lo + 1, lat.size() - 1);
            return lat[lo] + (lat[hi] - lat[lo]) * (r - (double)lo);
        };
        out->p50_latency_s = pct(50.0);
        out->p99_latency_s = pct(99.0);
        double sum = 0.0;
        for (double t : lat) sum += t;
        out->mean_latency_s = sum / (double)lat.size();
    }
    return SPH_OK;
}

const char* sph_server_last_error(const sph_server* s)
{
    if (!s) return "null server";
    return s->err.c_str();
}

}  // extern "C"
