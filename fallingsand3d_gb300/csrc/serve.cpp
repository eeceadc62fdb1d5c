// Serving loop: a seeded Poisson stream of simulation requests served by one
// batch with continuous batching.  Requests that arrive while a segment runs
// are admitted (generated on the device, overlapping the running segment) as
// soon as the memory budget allows and join at the next segment; finished
// worlds are hashed, retired and their memory reused.  Latency is measured
// from a request's arrival to its result being visible on the host.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "fs3d_common.h"
#include "pcg.h"

using namespace fs3d;

extern "C" {

fs3d_status fs3d_serve_plan(const fs3d_serve_params* p, int64_t capacity, fs3d_serve_request* reqs,
                            int64_t* n_reqs) {
    if (!p || !n_reqs || p->lambda <= 0.0 || p->duration_s <= 0.0 || capacity < 0 || (capacity > 0 && !reqs))
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_serve_plan: bad args");
    static const int kDims[7] = {16, 24, 32, 48, 64, 96, 128};
    const int lo = p->min_steps > 0 ? p->min_steps : 10, hi = p->max_steps > 0 ? p->max_steps : 1000;
    if (hi < lo) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_serve_plan: max_steps < min_steps");
    Pcg32 r(p->master_seed, 0xC4u);
    double t = 0.0;
    int64_t n = 0;
    const int64_t cap = p->max_requests > 0 ? p->max_requests : INT64_MAX;
    for (;;) {
        // exponential inter-arrival time from a 32-bit draw in (0, 1)
        const double u = ((double)r.next() + 0.5) / 4294967296.0;
        t += -log(u) / p->lambda;
        if (t > p->duration_s || n >= cap) break;
        int d[3];
        for (int& v : d) v = kDims[r.bounded(7u)];
        const double v = ((double)r.next() + 0.5) / 4294967296.0;
        int steps = (int)floor(exp(log((double)lo) + v * (log((double)hi) - log((double)lo))));
        steps = steps < lo ? lo : (steps > hi ? hi : steps);
        if (n < capacity) {
            fs3d_serve_request& q = reqs[n];
            memset(&q, 0, sizeof(q));
            q.arrival_s = t;
            q.X = d[0];
            q.Y = d[1];
            q.Z = d[2];
            q.n_steps = steps;
            q.seed = fmix64(p->master_seed ^ (0x5E7E000000000000ull + (uint64_t)n));
        }
        ++n;
    }
    *n_reqs = n;
    return FS3D_OK;
}

fs3d_status fs3d_serve_run(const fs3d_serve_params* p, int64_t n, fs3d_serve_request* reqs, fs3d_serve_stats* st) {
    if (!p || !reqs || !st || n < 0) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_serve_run: bad args");
    memset(st, 0, sizeof(*st));
    fs3d_config cfg = fs3d_default_config();
    if (p->steps_per_segment > 0) cfg.steps_per_segment = p->steps_per_segment;
    fs3d_batch* b = nullptr;
    fs3d_status s = fs3d_batch_create(p->hbm_budget ? p->hbm_budget : ((size_t)150 << 30), &cfg, &b);
    if (s != FS3D_OK) return s;
    {
        // warm-up outside the clock: the first launch of each kernel loads it,
        // and the stream-ordered pool grows on its first large allocations
        void* stream = nullptr;
        fs3d_batch_stream(b, &stream);
        void* warm = nullptr;
        const size_t warm_bytes = (size_t)1 << 30;
        if (cudaMallocAsync(&warm, warm_bytes, (cudaStream_t)stream) == cudaSuccess)
            cudaFreeAsync(warm, (cudaStream_t)stream);
        uint64_t t = 0, h = 0;
        int done = 0;
        s = fs3d_batch_admit_generated(b, 16, 16, 16, 1, 0, 1, &t);
        if (s == FS3D_OK) s = fs3d_batch_run_segment(b);
        if (s == FS3D_OK) s = fs3d_batch_sync(b, -1);
        if (s == FS3D_OK) s = fs3d_batch_poll(b, t, &done, &h);
        if (s == FS3D_OK) s = fs3d_batch_retire(b, t, nullptr);
        if (s == FS3D_OK) s = fs3d_batch_sync(b, -1);
        if (s != FS3D_OK) {
            fs3d_batch_destroy(b);
            return s;
        }
    }
    const int64_t seg_timeout_ns = (int64_t)(p->segment_timeout_ms > 0 ? p->segment_timeout_ms : 10000) * 1000000;
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    auto now_s = [&] { return std::chrono::duration<double>(clk::now() - t0).count(); };
    std::deque<int64_t> queue;
    std::unordered_map<uint64_t, int64_t> live;  // ticket -> request
    int64_t next = 0, completed = 0;
    std::vector<double> lat;
    lat.reserve((size_t)n);
    size_t peak_bytes = 0;
    int64_t peak_live = 0;
    double vu = 0.0;
    bool segment_in_flight = false;
    std::vector<uint64_t> tk, fin;  // live tickets, finished tickets
    std::vector<int> dn;
    std::vector<uint64_t> hs;
    while (completed < n && s == FS3D_OK) {
        const double now = now_s();
        while (next < n && reqs[next].arrival_s <= now) queue.push_back(next++);
        // admit in arrival order while the budget allows
        while (!queue.empty()) {
            fs3d_serve_request& q = reqs[queue.front()];
            uint64_t ticket = 0;
            const fs3d_status a = fs3d_batch_admit_generated(b, q.X, q.Y, q.Z, q.seed, 0, q.n_steps, &ticket);
            if (a == FS3D_ERR_BUDGET) {
                // with no world live the batch holds no memory: this request
                // needs more than the whole budget and would wait forever
                if (live.empty())
                    s = set_error(FS3D_ERR_BUDGET, "fs3d_serve_run: request " + std::to_string(queue.front()) +
                                                       " needs more memory than the whole budget");
                break;
            }
            if (a != FS3D_OK) {
                s = a;
                break;
            }
            q.admitted_s = now_s();
            live[ticket] = queue.front();
            queue.pop_front();
        }
        if (s != FS3D_OK) break;
        int64_t lw = 0;
        size_t used = 0;
        fs3d_batch_stats(b, &lw, nullptr, &used, nullptr);
        peak_live = std::max(peak_live, lw);
        peak_bytes = std::max(peak_bytes, used);
        if (segment_in_flight) {
            // arrivals during the segment were admitted above; now wait for it,
            // within the deadline (a segment that does not end in time ends the run)
            s = fs3d_batch_sync(b, seg_timeout_ns);
            segment_in_flight = false;
            if (s != FS3D_OK) break;
            // every live world polled at once: the finished ones are hashed
            // together (one launch, one wait) and retired together
            tk.clear();
            for (const auto& kv : live) tk.push_back(kv.first);
            dn.assign(tk.size(), 0);
            hs.assign(tk.size(), 0);
            s = fs3d_batch_poll_many(b, (int)tk.size(), tk.data(), dn.data(), p->with_hash ? hs.data() : nullptr);
            if (s != FS3D_OK) break;
            const double fin_s = now_s();
            fin.clear();
            for (size_t i = 0; i < tk.size(); ++i) {
                if (!dn[i]) continue;
                fs3d_serve_request& q = reqs[live[tk[i]]];
                q.hash = hs[i];
                q.finished_s = fin_s;
                lat.push_back((q.finished_s - q.arrival_s) * 1e3);
                vu += (double)q.X * q.Y * q.Z * q.n_steps;
                ++completed;
                live.erase(tk[i]);
                fin.push_back(tk[i]);
            }
            if (!fin.empty()) s = fs3d_batch_retire_many(b, (int)fin.size(), fin.data(), nullptr);
            continue;
        }
        if (!live.empty()) {
            s = fs3d_batch_run_segment(b);
            segment_in_flight = s == FS3D_OK;
            ++st->segments;
        } else if (next < n) {
            // idle until the next arrival
            const double wait = reqs[next].arrival_s - now_s();
            if (wait > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds((int64_t)(wait * 1e6) - 100));
        }
    }
    st->wall_s = now_s();
    if (s == FS3D_ERR_TIMEOUT) {
        // A segment still running past the deadline: the batch is not torn
        // down (its teardown would wait for that work) and its memory stays
        // allocated.  A segment that ended but reported a kernel's bounded
        // wait giving up leaves nothing running, so the batch is released.
        void* stream = nullptr;
        fs3d_batch_stream(b, &stream);
        if (cudaStreamQuery((cudaStream_t)stream) == cudaSuccess) fs3d_batch_destroy(b);
        cudaGetLastError();
        return s;
    }
    fs3d_batch_destroy(b);
    if (s != FS3D_OK) return s;
    st->requests = n;
    st->completed = completed;
    st->peak_live_worlds = peak_live;
    st->peak_bytes = peak_bytes;
    st->voxel_updates = vu;
    st->voxel_updates_per_s = st->wall_s > 0 ? vu / st->wall_s : 0.0;
    const double window = n > 0 ? reqs[n - 1].arrival_s : 0.0;
    st->offered_voxel_updates_per_s = window > 0 ? vu / window : 0.0;
    if (!lat.empty()) {
        std::sort(lat.begin(), lat.end());
        auto pct = [&](double f) { return lat[std::min(lat.size() - 1, (size_t)(f * (double)(lat.size() - 1) + 0.5))]; };
        st->p50_ms = pct(0.50);
        st->p99_ms = pct(0.99);
        st->max_ms = lat.back();
        double sum = 0;
        for (double v : lat) sum += v;
        st->mean_ms = sum / (double)lat.size();
    }
    return FS3D_OK;
}

}  // extern "C"
