// fs3d_batch: many independent worlds of mixed sizes in one device pool (bit
// plane format), stepped together.  A segment is one CUDA graph: a persistent
// kernel per size class runs each of its worlds through all of the segment's
// steps (plus, for worlds too large for any class, steps_per_segment launches
// of the per-step kernel), then a small kernel advances every world's step
// counter in the device table.  The graph reads the world and work-item
// tables from device memory, so worlds join (admit) and leave (retire)
// between segments without a re-capture, and an unchanged batch reuses the
// tables as they stand.  Each world keeps its own step counter, so its
// trajectory is the same whether it runs alone or inside any mix.
//
// Streams: `stream` runs segments; `upload` the host-to-device copies of
// admit_many; `side` the admission conversions and single retirements;
// `readback` the read-back conversions of retire_many; `download` their
// device-to-host copies.  Events order them against the segments and each
// other, and no stream waits for work its next item does not need, so both
// directions of the host link run while a segment computes.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "fs3d_common.h"
#include "planes.h"

using namespace fs3d;

namespace {

struct BWorld {
    int X = 0, Y = 0, Z = 0, nw = 0;
    // the classes that hold the world (they depend on its dims only), looked up once
    mutable int cls_smem = -2, cls_gm = -2;
    uint64_t seed = 0, t = 0;
    int64_t remaining = 0;
    uint4* rows = nullptr;
    std::shared_ptr<void> arena;  // set when rows live in a block shared by the worlds of one admit_many
    uint8_t* statics = nullptr;
    uint8_t* lflags = nullptr;  // layer flags after the planes (same allocation)
    bool flags_valid = false;   // set from the cells at admission, then kept by every resident segment
    size_t bytes = 0;
    bool done = false;
    cudaEvent_t ready = nullptr;     // admission finished (side stream)
    std::shared_ptr<CUevent_st> finished;  // recorded after the segment that took its last step (shared)
    bool hash_valid = false;
    uint64_t hash = 0;
    uint64_t admit_id = 0;                       // admission whose static-material check is pending (0: none)
    int admit_index = 0;                         // the world's place in that admission
    std::shared_ptr<CUevent_st> admitted;       // planes written by admit_many (shared by its worlds)
    std::shared_ptr<CUevent_st> statics_ready;  // static byte copy written
};

// An admit_many whose conversion is enqueued and whose per-world static
// material flags are still on their way to the host: the worlds run from
// their planes meanwhile; a world holding a material >= 4 gets its byte copy
// (from the staging bytes) when the flags are read.
struct PendingAdmit {
    uint64_t id = 0;
    cudaEvent_t done = nullptr;  // flags copied (admission stream)
    int* flags = nullptr;        // page-locked, one per world
    size_t flags_cap = 0;
    uint8_t* staging = nullptr;  // the admitted bytes on the device
    void* table = nullptr;       // conversion and copy tables
    const int* flags_dev = nullptr;  // the flags in `table`
    std::shared_ptr<CUevent_st> reader;  // last read-back that took static bytes from `staging`
    int slot = -1;                       // the admission staging buffer holding the bytes
    std::shared_ptr<CUevent_st> converted;  // after the conversion that read them
    std::vector<uint64_t> tickets;
    std::vector<int64_t> byte_off, cells;
};

std::shared_ptr<CUevent_st> shared_event() {
    cudaEvent_t ev = nullptr;
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return {};
    return std::shared_ptr<CUevent_st>(ev, [](CUevent_st* x) { cudaEventDestroy(x); });
}

template <class T>
struct PinnedArray {
    // two page-locked host images, written in turn (one may still be being
    // uploaded while the next segment's tables are built), and the device copy
    T* hb[2] = {nullptr, nullptr};
    T* dvb[2] = {nullptr, nullptr};  // the images' device views (null: not addressable by the device)
    T* h = nullptr;                  // the image in use
    T* hv = nullptr;                 // its device view
    int cur = 0;
    T* d = nullptr;
    size_t cap = 0;
    void select(int i) {
        cur = i;
        h = hb[i];
        hv = dvb[i];
    }
    // copies the first n entries of the image in use to the device: a kernel
    // reading the page-locked image (no copy engine) when it can
    cudaError_t upload(size_t n, cudaStream_t st) const {
        return hv ? copy_small_async(d, hv, sizeof(T) * n, st)
                  : cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, st);
    }
    fs3d_status reserve(size_t n) {
        if (n <= cap) return FS3D_OK;
        size_t c = cap ? cap : 64;
        while (c < n) c *= 2;
        T *nh0 = nullptr, *nh1 = nullptr, *nd = nullptr;
        FS3D_CUDA(cudaMallocHost((void**)&nh0, sizeof(T) * c));
        cudaError_t e = cudaMallocHost((void**)&nh1, sizeof(T) * c);
        if (e == cudaSuccess) e = cudaMalloc((void**)&nd, sizeof(T) * c);
        if (e != cudaSuccess) {
            cudaFreeHost(nh0);
            if (nh1) cudaFreeHost(nh1);
            return cuda_fail(e, "cudaMalloc(batch tables)");
        }
        cudaFreeHost(hb[0]);
        cudaFreeHost(hb[1]);
        cudaFree(d);
        hb[0] = nh0;
        hb[1] = nh1;
        dvb[0] = reinterpret_cast<T*>(device_view(nh0));
        dvb[1] = reinterpret_cast<T*>(device_view(nh1));
        h = hb[cur];
        hv = dvb[cur];
        d = nd;
        cap = c;
        return FS3D_OK;
    }
    void release() {
        cudaFreeHost(hb[0]);
        cudaFreeHost(hb[1]);
        cudaFree(d);
        hb[0] = hb[1] = h = hv = d = nullptr;
        dvb[0] = dvb[1] = nullptr;
        cap = 0;
    }
};

}  // namespace

struct fs3d_batch {
    size_t budget = 0, used = 0;
    fs3d_config cfg{};
    cudaStream_t stream = nullptr, side = nullptr;
    std::map<uint64_t, BWorld> worlds;
    uint64_t next_ticket = 1;
    PinnedArray<PlaneWorld> tw;
    PinnedArray<PlaneItem> ti;
    PinnedArray<int> tn;  // meta: {per-step items, resident count per class, offset per class, worlds}
    PinnedArray<int> to;  // resident worlds (indices into tw) by class, largest first
    int* counter = nullptr;  // work counters of the resident kernels, one per class
    int* err = nullptr;      // set by a kernel whose bounded wait gave up
    cudaEvent_t fork = nullptr, join[kAllClasses + 1] = {};
    cudaStream_t branch[kAllClasses + 1] = {};  // capture branches of a segment: one per class, then the per-step chain
    cudaEvent_t tables_free[2] = {};  // the upload from each table image has run
    int tab_cur = 0;                  // the table image of the last build
    cudaEvent_t last_segment = nullptr;
    std::vector<std::shared_ptr<CUevent_st>> pending_ready;  // admissions the next segment must wait for
    cudaStream_t readback = nullptr;              // read-backs of retire_many
    cudaStream_t upload = nullptr;                // host -> device copies of admit_many
    cudaStream_t download = nullptr;              // device -> host copies of retire_many

    std::deque<PendingAdmit> pending_admits;      // in admission order
    uint64_t next_admit_id = 1;
    std::vector<std::pair<int*, size_t>> flag_pool;  // page-locked flag buffers free for reuse
    // page-locked staging of the small job tables (a copy from pageable memory
    // would wait for the copies queued before it); a chunk is reused once the
    // event recorded after its upload has completed
    struct HostChunk {
        char* p = nullptr;
        uint8_t* dv = nullptr;  // device view of p (null: not addressable by the device)
        size_t cap = 0;
        cudaEvent_t uploaded = nullptr;
    };
    std::vector<HostChunk> host_chunks;
    // memory of retired worlds (and staging buffers) freed once the read-back
    // that reads it has run: no stream has to wait for another
    struct DeferredFree {
        std::shared_ptr<CUevent_st> after;
        std::vector<std::shared_ptr<void>> arenas;
        std::vector<void*> ptrs;
    };
    std::deque<DeferredFree> deferred;
    // Staging bytes of admit_many (uploads) and retire_many (downloads):
    // kStagingRing persistent buffers each, used in turn.  A buffer is taken
    // again once the events of its previous use (kStagingRing calls back) have
    // run: no per-call allocation of hundreds of MB, and no stream waits on
    // the calls just before.
    struct StagingSlot {
        uint8_t* p = nullptr;
        size_t cap = 0;
        std::vector<std::shared_ptr<CUevent_st>> busy;  // the uses still to run
        uint64_t admit_id = 0;                          // admission whose bytes these are
    };
    static constexpr int kStagingRing = 3;
    StagingSlot up_ring[kStagingRing], rb_ring[kStagingRing];
    int up_turn = 0, rb_turn = 0;
    // segment graphs without and with the per-step kernel's launches (the
    // second only when some world is too large to be resident)
    cudaGraphExec_t graph = nullptr, graph_steps = nullptr;
    void* graph_worlds = nullptr;  // table pointers baked into the graphs
    void* graph_items = nullptr;
    void* graph_order = nullptr;
    // classes with worlds in the current tables (bit c), and those the graphs launch
    uint32_t class_mask = ~0u, graph_mask = 0;
    int grid = 0;
    int promote = 0;  // single-CTA resident worlds run this many classes wider (autotuned)
    unsigned long long* hash_dev = nullptr;
    unsigned long long* processed_dev = nullptr;  // cell-steps the resident kernels evaluated
    uint64_t segments = 0;
    uint64_t dense_cell_steps = 0;   // every cell of every stepped world, per step
    uint64_t stepped_cell_steps = 0; // of those, taken by the per-step kernel (always evaluated)
    // The device tables as the last segment left them (each world advanced by
    // its steps) are the next segment's tables while no world is admitted or
    // retired, changes class, or takes fewer steps than a full segment:
    // `reuse_left` more segments may launch without rebuilding them.
    bool tables_stale = true;
    bool prepared = false;  // fs3d_batch_prepare built the next segment's tables
    uint64_t reuse_left = 0;
    std::vector<BWorld*> running;  // the worlds of the tables, in table order
    size_t table_items = 0;        // per-step kernel items in the tables
    uint64_t table_dense = 0, table_stepped = 0;  // cell-steps per segment of the tables
};

namespace {

// Worlds younger than this (by their own step counter: a world admitted at
// step 500 has been stepped 500 times) are still mostly moving: the hybrid
// mode keeps them in shared memory, where dense steps are cheap.
// (2048 mixed worlds: 64-step segments at ages 0 / 64 / 128 / 192 take
// 5.1 / 2.7 / 1.9 / 1.9 ms in shared memory and 8.5 / 3.4 / 1.6 / 1.3 ms
// from L2, which wins from age 128 on.)
constexpr uint64_t kYoungSteps = 128;

// Segment class of a running world (-1: the per-step kernel) under the
// batch's mode: 1 shared-memory classes, 2 global-memory classes, 3 hybrid
// (young worlds in shared memory when they fit, settled ones in global
// memory), 0 none.  `promote` moves worlds to wider classes: the shared-memory
// single-CTA classes in mode 1, the global-memory classes in modes 2 and 3
// (the hybrid mode tunes on settled worlds, which run in global memory).
int segment_class(const fs3d_batch* b, const BWorld& w) {
    const int mode = b->cfg.use_smem;
    auto smem = [&]() {
        if (w.cls_smem == -2) w.cls_smem = resident_class(w.X, w.Y, w.Z);
        int c = w.cls_smem;
        if (mode == 1 && c >= 0 && c < kSingleCtaClasses) c = std::min(c + b->promote, kSingleCtaClasses - 1);
        return c;
    };
    auto gm = [&]() {
        if (w.cls_gm == -2) w.cls_gm = resident_class_gm(w.X, w.Y, w.Z);
        const int c = w.cls_gm;
        return c < 0 ? -1 : kResidentClasses + std::min(c + b->promote, kGmDense - 1);
    };
    if (mode == 1) return smem();
    if (mode == 2) return gm();
    if (mode == 3) {
        if (w.t < kYoungSteps) {
            // a young world that needs a cluster runs instead from L2 with a
            // whole SM (768 threads): dense steps keep its warps busy, and no
            // cluster barrier or y-slab imbalance holds it up.  The smallest
            // worlds run in 256-thread CTAs: their dense steps take half the
            // passes there (2048 fresh worlds: 2.79 ms per first segment
            // against 3.02 ms in 128-thread CTAs; moving the 256-thread worlds
            // up to 768 threads too measured 3.09 ms)
            const int c = smem();
            if (c >= 0 && c < kSingleCtaClasses) return c == 0 ? 1 : c;
            if (w.Y <= 4096) return kResidentClasses + kGmDense;
            return c >= 0 ? c : gm();
        }
        const int first = gm();
        return first >= 0 ? first : smem();
    }
    return -1;
}

fs3d_status wait_stream(cudaStream_t st, int64_t timeout_ns) {
    if (timeout_ns < 0) {
        FS3D_CUDA(cudaStreamSynchronize(st));
        return FS3D_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t e = cudaStreamQuery(st);
        if (e == cudaSuccess) return FS3D_OK;
        if (e != cudaErrorNotReady) return cuda_fail(e, "cudaStreamQuery");
        if (std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count() >=
            timeout_ns)
            return set_error(FS3D_ERR_TIMEOUT, "batch stream did not finish within the timeout");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
}

void free_world(fs3d_batch* b, BWorld& w) {
    if (w.arena)
        w.arena.reset();  // the block is freed with its last world
    else if (w.rows)
        cudaFreeAsync(w.rows, b->side);
    if (w.statics) cudaFreeAsync(w.statics, b->side);
    if (w.ready) cudaEventDestroy(w.ready);
    w.finished.reset();
    w.admitted.reset();
    w.statics_ready.reset();
    w.rows = nullptr;
    w.statics = nullptr;
    w.ready = nullptr;
}

// Stream-ordered allocation from the device's default pool (freed blocks stay
// cached: its release threshold is raised when a batch is created).
template <class T>
cudaError_t stream_alloc(T** p, size_t n, cudaStream_t st) {
    return cudaMallocAsync(reinterpret_cast<void**>(p), n, st);
}

// Test hook (fs3d_test_inject): admissions whose world memory allocation is
// refused as out of memory, without asking the device.
std::atomic<int> g_inject_alloc_failures{0};

// The allocation of an admission's world memory (planes and layer flags).
template <class T>
cudaError_t admission_alloc(T** p, size_t n, cudaStream_t st) {
    int left = g_inject_alloc_failures.load();
    while (left > 0 && !g_inject_alloc_failures.compare_exchange_weak(left, left - 1)) {
    }
    if (left > 0) return cudaErrorMemoryAllocation;
    return stream_alloc(p, n, st);
}

// A page-locked buffer of at least n flags, from the batch's pool.
int* take_flags(fs3d_batch* b, size_t n, size_t* cap) {
    for (size_t i = 0; i < b->flag_pool.size(); ++i)
        if (b->flag_pool[i].second >= n) {
            const auto f = b->flag_pool[i];
            b->flag_pool.erase(b->flag_pool.begin() + (std::ptrdiff_t)i);
            *cap = f.second;
            return f.first;
        }
    const size_t c = std::max<size_t>(n, 1024);
    int* f = nullptr;
    if (cudaMallocHost((void**)&f, c * sizeof(int)) != cudaSuccess) return nullptr;
    *cap = c;
    return f;
}

// The next buffer of a staging ring, of at least n bytes, for stream st: st
// waits for the buffer's previous uses (it grows, on st, when too small).
fs3d_batch::StagingSlot* take_slot(fs3d_batch::StagingSlot* ring, int& turn, size_t n, cudaStream_t st,
                                   cudaError_t* e) {
    fs3d_batch::StagingSlot& sl = ring[turn];
    turn = (turn + 1) % fs3d_batch::kStagingRing;
    *e = cudaSuccess;
    for (auto& ev : sl.busy)
        if (*e == cudaSuccess) *e = cudaStreamWaitEvent(st, ev.get(), 0);
    sl.busy.clear();
    if (*e == cudaSuccess && sl.cap < n) {
        if (sl.p) cudaFreeAsync(sl.p, st);
        sl.p = nullptr;
        sl.cap = 0;
        *e = cudaMallocAsync(reinterpret_cast<void**>(&sl.p), n, st);
        if (*e == cudaSuccess) sl.cap = n;
    }
    return &sl;
}

// Marks a staging buffer in use until an event recorded now on st has run
// (or, with no event, waits for st here).
void mark_busy(fs3d_batch::StagingSlot* sl, cudaStream_t st) {
    std::shared_ptr<CUevent_st> ev = shared_event();
    if (ev && cudaEventRecord(ev.get(), st) == cudaSuccess)
        sl->busy.push_back(ev);
    else
        cudaStreamSynchronize(st);
}

// Frees the deferred memory whose read-backs have run (all of it with `wait`).
void drain_deferred(fs3d_batch* b, bool wait) {
    while (!b->deferred.empty()) {
        fs3d_batch::DeferredFree& d = b->deferred.front();
        const cudaError_t q = wait ? cudaEventSynchronize(d.after.get()) : cudaEventQuery(d.after.get());
        if (q == cudaErrorNotReady) break;
        d.arenas.clear();  // a block goes back to the pool with its last world
        for (void* p : d.ptrs) cudaFreeAsync(p, b->side);
        b->deferred.pop_front();
    }
}

// A page-locked chunk of at least n bytes whose last upload has run (index
// into b->host_chunks); upload_chunk copies it to the device and marks it in use.
int take_chunk(fs3d_batch* b, size_t n) {
    for (size_t i = 0; i < b->host_chunks.size(); ++i) {
        auto& c = b->host_chunks[i];
        if (c.cap >= n && cudaEventQuery(c.uploaded) == cudaSuccess) return (int)i;
    }
    fs3d_batch::HostChunk c;
    c.cap = std::max<size_t>(n, (size_t)1 << 16);
    if (cudaMallocHost((void**)&c.p, c.cap) != cudaSuccess) return -1;
    c.dv = device_view(c.p);
    if (cudaEventCreateWithFlags(&c.uploaded, cudaEventDisableTiming) != cudaSuccess) {
        cudaFreeHost(c.p);
        return -1;
    }
    b->host_chunks.push_back(c);
    return (int)b->host_chunks.size() - 1;
}

// (a kernel reads the page-locked chunk: a copy-engine transfer here would
// queue behind the hundreds of MB other streams move over the host link, and
// hold up the conversion or segment that needs the table)
cudaError_t upload_chunk(fs3d_batch* b, int i, void* dst, size_t n, cudaStream_t st) {
    const fs3d_batch::HostChunk& c = b->host_chunks[(size_t)i];
    cudaError_t e = c.dv ? copy_small_async(dst, c.dv, n, st) : cudaMemcpyAsync(dst, c.p, n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(b->host_chunks[(size_t)i].uploaded, st);
    return e;
}

// Completes the pending admissions with id <= upto, oldest first: reads their
// static-material flags (waiting for them with `wait`, else stopping at the
// first not yet on the host), gives each flagged world its byte copy and
// frees the staging bytes.
fs3d_status finalize_admits(fs3d_batch* b, uint64_t upto, bool wait) {
    while (!b->pending_admits.empty() && b->pending_admits.front().id <= upto) {
        PendingAdmit& p = b->pending_admits.front();
        const cudaError_t q = wait ? cudaEventSynchronize(p.done) : cudaEventQuery(p.done);
        if (q == cudaErrorNotReady) break;
        if (q != cudaSuccess) return cuda_fail(q, "admission");
        std::vector<BWorld*> flagged;
        fs3d_status s = FS3D_OK;
        for (size_t a = 0; a < p.tickets.size(); ++a) {
            auto it = b->worlds.find(p.tickets[a]);
            if (it == b->worlds.end()) continue;
            BWorld& w = it->second;
            w.admit_id = 0;
            if (!p.flags[a] || s != FS3D_OK) continue;
            const size_t cells = (size_t)p.cells[a];
            cudaError_t e = stream_alloc(&w.statics, cells, b->side);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(w.statics, p.staging + p.byte_off[a], cells, cudaMemcpyDeviceToDevice, b->side);
            if (e != cudaSuccess) {
                s = cuda_fail(e, "static material copy");
                continue;
            }
            w.bytes += cells;
            b->used += cells;
            flagged.push_back(&w);
        }
        std::shared_ptr<CUevent_st> ready;
        if (!flagged.empty()) {
            ready = shared_event();
            if (ready && cudaEventRecord(ready.get(), b->side) == cudaSuccess)
                for (BWorld* w : flagged) w->statics_ready = ready;
            else
                ready.reset();
        }
        // the staging buffer is free again once the conversion and the static
        // copies (admission stream) and any read-back that took static bytes
        // from it have run; the tables (with the flags) likewise
        if (p.slot >= 0) {
            fs3d_batch::StagingSlot* sl = &b->up_ring[p.slot];
            if (p.converted) sl->busy.push_back(p.converted);
            if (!flagged.empty()) {
                if (ready)
                    sl->busy.push_back(ready);
                else
                    cudaStreamSynchronize(b->side);
            }
            if (p.reader) sl->busy.push_back(p.reader);
            if (sl->admit_id == p.id) sl->admit_id = 0;
        }
        if (p.reader) {
            fs3d_batch::DeferredFree d;
            d.after = p.reader;
            d.ptrs = {p.table};
            b->deferred.push_back(std::move(d));
        } else {
            cudaFreeAsync(p.table, b->side);
        }
        b->flag_pool.emplace_back(p.flags, p.flags_cap);
        cudaEventDestroy(p.done);
        b->pending_admits.pop_front();
        if (s != FS3D_OK) return s;
    }
    return FS3D_OK;
}

// One segment on stream `a`: the resident kernel of every class (worlds that
// fit in shared memory take all their steps in one launch) and
// steps_per_segment launches of the per-step kernel (the larger worlds).
// With `fork` each goes to its own branch stream so they run concurrently.
// resident-kernel launches of one segment under a mode (enqueue_segment's),
// of the classes in `mask`
int resident_launches(int mode, uint32_t mask) {
    uint32_t launched = 0;
    if (mode == 1 || mode == 3) launched |= (1u << kResidentClasses) - 1u;
    if (mode == 2 || mode == 3) launched |= ((1u << kGmClasses) - 1u) << kResidentClasses;
    return __builtin_popcount(launched & mask);
}

fs3d_status enqueue_segment(fs3d_batch* b, cudaStream_t a, bool fork, bool with_steps) {
    if (fork) {
        FS3D_CUDA(cudaEventRecord(b->fork, a));
        for (cudaStream_t br : b->branch) FS3D_CUDA(cudaStreamWaitEvent(br, b->fork, 0));
    }
    fs3d_status s = FS3D_OK;
    const int mode = b->cfg.use_smem;
    // The launch order is the order the SMs fill in.  Young worlds: the large
    // ones first (the dense global-memory class, then the shared-memory
    // classes widest first), since they take the longest; settled worlds: the
    // global-memory classes smallest CTA first, whose chains are the longest.
    // In a graph the branches' kernels are all pending at once and the launch
    // order alone does not decide which grid is placed first: the dense class
    // carries the greatest priority.
    // Classes without a world in the tables are not launched (the graph is
    // captured again when that set changes).
    auto has = [&](int cls) { return (b->class_mask >> cls) & 1u; };
    auto gm = [&](int c) {
        if (!has(kResidentClasses + c)) return FS3D_OK;
        return launch_plane_segment_gm(c, b->tw.d, b->to.d, b->tn.d, b->counter + kResidentClasses + c, b->err,
                                       fork ? b->branch[kResidentClasses + c] : a, b->processed_dev,
                                       mode == 3 && c == kGmDense);
    };
    if (mode == 3) s = gm(kGmDense);
    if (mode == 1 || mode == 3)
        for (int c = kResidentClasses - 1; c >= 0 && s == FS3D_OK; --c)
            if (has(c))
                s = launch_plane_segment_resident(c, b->tw.d, b->to.d, b->tn.d, b->counter + c, b->err,
                                                  fork ? b->branch[c] : a, b->processed_dev);
    if (mode == 2 || mode == 3)
        for (int c = 0; c < kGmClasses && s == FS3D_OK; ++c)
            if (c != kGmDense || mode == 2) s = gm(c);
    for (int k = 0; with_steps && k < b->cfg.steps_per_segment && s == FS3D_OK; ++k)
        s = launch_plane_step(b->tw.d, b->ti.d, b->tn.d, b->grid, k, fork ? b->branch[kAllClasses] : a);
    if (s != FS3D_OK) return s;
    if (fork)
        for (int c = 0; c <= kAllClasses; ++c) {
            FS3D_CUDA(cudaEventRecord(b->join[c], b->branch[c]));
            FS3D_CUDA(cudaStreamWaitEvent(a, b->join[c], 0));
        }
    return launch_advance_worlds(b->tw.d, b->tn.d, a);
}

fs3d_status capture_one(fs3d_batch* b, bool with_steps, cudaGraphExec_t* out) {
    if (*out) {
        cudaGraphExecDestroy(*out);
        *out = nullptr;
    }
    cudaStream_t cs;
    FS3D_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    fs3d_status s = FS3D_OK;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        s = enqueue_segment(b, cs, true, with_steps);
        e = cudaStreamEndCapture(cs, &g);
    }
    if (e == cudaSuccess && s == FS3D_OK) e = cudaGraphInstantiate(out, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (s != FS3D_OK) return s;
    if (e != cudaSuccess) return cuda_fail(e, "segment graph capture");
    return FS3D_OK;
}

fs3d_status capture_graph(fs3d_batch* b) {
    fs3d_status s = capture_one(b, false, &b->graph);
    if (s == FS3D_OK) s = capture_one(b, true, &b->graph_steps);
    if (s != FS3D_OK) return s;
    b->graph_worlds = b->tw.d;
    b->graph_items = b->ti.d;
    b->graph_order = b->to.d;
    b->graph_mask = b->class_mask;
    return FS3D_OK;
}

}  // namespace

namespace fs3d {
void set_inject_alloc_failures(int n) { g_inject_alloc_failures.store(n > 0 ? n : 0); }
}  // namespace fs3d

extern "C" {

fs3d_status fs3d_batch_create(size_t budget, const fs3d_config* cfg, fs3d_batch** out) {
    if (!out || budget == 0) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_create: bad args");
    *out = nullptr;
    fs3d_batch* b = new fs3d_batch();
    b->budget = budget;
    b->cfg = cfg ? *cfg : fs3d_default_config();
    if (b->cfg.steps_per_segment <= 0) b->cfg.steps_per_segment = 64;
    if (b->cfg.steps_per_segment > 4096) b->cfg.steps_per_segment = 4096;
    const int resident = plane_step_ctas_per_sm();
    const int per_sm = b->cfg.ctas_per_sm > 0 && b->cfg.ctas_per_sm < resident ? b->cfg.ctas_per_sm : resident;
    b->grid = sm_count_public() * per_sm;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->readback, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->upload, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->download, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->tables_free[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->last_segment, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->hash_dev, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->processed_dev, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->processed_dev, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->counter, sizeof(int) * kAllClasses);
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->err, sizeof(int) * kErrInts);
    if (e == cudaSuccess) e = cudaMemset(b->err, 0, sizeof(int) * kErrInts);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int c = 0; c <= kAllClasses && e == cudaSuccess; ++c) {
        e = cudaEventCreateWithFlags(&b->join[c], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->branch[c], cudaStreamNonBlocking);
    }
    if (e == cudaSuccess) {
        // keep freed pool memory cached so admissions after retirements are cheap
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    fs3d_status s = e == cudaSuccess ? FS3D_OK : cuda_fail(e, "fs3d_batch_create");
    if (s == FS3D_OK) s = b->tn.reserve(kMetaInts);
    // size the tables for a few thousand worlds and capture the segment graph
    // now, so the first segments of a run (or a server) pay neither a pinned
    // allocation nor a capture
    if (s == FS3D_OK) s = b->tw.reserve(4096);
    if (s == FS3D_OK) s = b->ti.reserve(1 << 16);
    if (s == FS3D_OK) s = b->to.reserve(4096);
    if (s == FS3D_OK && b->cfg.use_graphs) s = capture_graph(b);
    if (s != FS3D_OK) {
        fs3d_batch_destroy(b);
        return s;
    }
    *out = b;
    return FS3D_OK;
}

}  // extern "C"

namespace {

// any byte >= 4 (a static material that must be kept for read-back)
bool has_static_material(const uint8_t* g, size_t n) {
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t v;
        memcpy(&v, g + i, 8);
        if (v & 0xFCFCFCFCFCFCFCFCull) return true;
    }
    for (; i < n; ++i)
        if (g[i] >= 4) return true;
    return false;
}

// Admits a world given as host bytes (g != NULL) or generated on the device
// from its seed (g == NULL: the mixed-size batch world of that seed).  With
// `wait` the call returns only after the host grid has been copied.
fs3d_status admit(fs3d_batch* b, const uint8_t* g, int X, int Y, int Z, uint64_t seed, uint64_t start_step,
                  int64_t n_steps, uint64_t* ticket, bool wait = true) {
    if (!b || !ticket || X <= 0 || Y <= 0 || Z <= 0 || X > kPlaneMaxX || Y > 65536 || Z > 65536 || n_steps < 0)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_admit: bad args (X must be 1..2048)");
    if (!g && Y < 4) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_admit_generated: needs Y >= 4");
    const size_t n = (size_t)X * Y * Z;
    const bool stat = g ? has_static_material(g, n) : false;
    BWorld w;
    w.X = X;
    w.Y = Y;
    w.Z = Z;
    w.nw = plane_nw(X);
    w.seed = seed;
    w.t = start_step;
    w.remaining = n_steps;
    w.done = n_steps == 0;
    w.bytes = plane_bytes(X, Y, Z) + layer_flag_bytes(Y) + (stat ? n : 0) + sizeof(PlaneWorld);
    if (b->used + w.bytes > b->budget)
        return set_error(FS3D_ERR_BUDGET, "fs3d_batch_admit: world does not fit in the memory budget now");
    uint8_t* staging = nullptr;
    FS3D_CUDA(admission_alloc(&w.rows, plane_bytes(X, Y, Z) + layer_flag_bytes(Y), b->side));
    w.lflags = reinterpret_cast<uint8_t*>(w.rows) + plane_bytes(X, Y, Z);
    fs3d_status s = FS3D_OK;
    cudaError_t e = cudaSuccess;
    if (g) {
        e = stream_alloc(&staging, n, b->side);
        if (e == cudaSuccess) e = cudaMemcpyAsync(staging, g, n, cudaMemcpyHostToDevice, b->side);
        s = e == cudaSuccess ? planes_from_bytes(staging, X, Y, Z, w.rows, b->side) : cuda_fail(e, "admit upload");
        if (stat)
            w.statics = staging;
        else if (staging)
            cudaFreeAsync(staging, b->side);
    } else {
        s = planes_generate_batch_world(seed, X, Y, Z, w.rows, b->side);
    }
    // layer flags from the cells: the first two steps evaluate only the
    // row-pairs that can change
    if (s == FS3D_OK) s = layer_flags_from_cells(w.rows, w.lflags, X, Y, Z, start_step, b->side);
    w.flags_valid = s == FS3D_OK;
    if (s == FS3D_OK) {
        e = cudaEventCreateWithFlags(&w.ready, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(w.ready, b->side);
        // the caller's buffer may be reused as soon as this returns; a world
        // generated on the device has no host buffer and is not waited for
        if (e == cudaSuccess && g && wait) e = cudaEventSynchronize(w.ready);
        if (e != cudaSuccess) s = cuda_fail(e, "admit event");
    }
    if (s != FS3D_OK) {
        free_world(b, w);
        return s;
    }
    b->used += w.bytes;
    *ticket = b->next_ticket++;
    b->worlds.emplace(*ticket, w);
    b->tables_stale = true;
    return FS3D_OK;
}

}  // namespace

extern "C" {

fs3d_status fs3d_batch_admit(fs3d_batch* b, const uint8_t* g, int X, int Y, int Z, uint64_t seed,
                             uint64_t start_step, int64_t n_steps, uint64_t* ticket) {
    if (!g) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_admit: NULL grid");
    return admit(b, g, X, Y, Z, seed, start_step, n_steps, ticket);
}

fs3d_status fs3d_batch_admit_generated(fs3d_batch* b, int X, int Y, int Z, uint64_t seed, uint64_t start_step,
                                       int64_t n_steps, uint64_t* ticket) {
    return admit(b, nullptr, X, Y, Z, seed, start_step, n_steps, ticket);
}

}  // extern "C"

namespace {

// Rebuilds the segment tables from the running worlds (their segment class,
// steps and kept layer flags), uploads them and works out how many following
// segments may reuse them as the device advances them.
fs3d_status build_tables(fs3d_batch* b) {
    const int S = b->cfg.steps_per_segment;
    b->running.clear();
    b->table_items = 0;
    b->table_dense = b->table_stepped = 0;
    b->reuse_left = 0;
    // the other table image: it may be rewritten once its upload (two builds
    // back) has run, while the last build's upload may still be pending
    b->tab_cur ^= 1;
    FS3D_CUDA(cudaEventSynchronize(b->tables_free[b->tab_cur]));
    b->tw.select(b->tab_cur);
    b->ti.select(b->tab_cur);
    b->tn.select(b->tab_cur);
    b->to.select(b->tab_cur);
    // resident class of every running world (-1: stepped by the per-step kernel)
    std::vector<std::pair<int, BWorld*>> run;
    size_t ni = 0, ns = 0;
    for (auto& kv : b->worlds) {
        BWorld& w = kv.second;
        if (w.done) continue;
        const int c = segment_class(b, w);
        run.emplace_back(c, &w);
        if (c >= 0)
            ++ns;
        else
            ni += (size_t)plane_items_for(w.Y, w.Z, w.nw);
    }
    const size_t nw_ = run.size();
    if (nw_ == 0) return FS3D_OK;
    // growing the tables frees device arrays a running segment may still read
    if (nw_ > b->tw.cap || ni > b->ti.cap || ns > b->to.cap) FS3D_CUDA(cudaStreamSynchronize(b->stream));
    fs3d_status s = b->tw.reserve(nw_);
    if (s == FS3D_OK) s = b->ti.reserve(ni > 0 ? ni : 1);
    if (s == FS3D_OK) s = b->to.reserve(ns > 0 ? ns : 1);
    if (s != FS3D_OK) return s;
    std::vector<int> by_class[kAllClasses];
    size_t ii = 0;
    uint64_t reuse = UINT64_MAX;  // segments these tables hold for, this one included
    for (size_t wi = 0; wi < nw_; ++wi) {
        BWorld& w = *run[wi].second;
        const int steps = (int)(w.remaining < S ? w.remaining : S);
        PlaneWorld& d = b->tw.h[wi];
        memset(&d, 0, sizeof(d));
        d.rows = w.rows;
        d.seed = w.seed;
        d.t = w.t;
        d.X = w.X;
        d.Y = w.Y;
        d.Z = w.Z;
        d.nw = w.nw;
        d.steps = steps;
        d.lg = plane_lg(w.nw);
        // resident segments keep the layer flags; the per-step kernel does not
        if (run[wi].first >= 0) {
            d.lflags = w.lflags;
            d.lflags_fresh = w.flags_valid ? 0 : 1;
            w.flags_valid = w.lflags != nullptr;
        } else {
            w.flags_valid = false;
        }
        const uint64_t cs = (uint64_t)w.X * w.Y * w.Z * (uint64_t)steps;
        b->table_dense += cs;
        if (run[wi].first < 0) b->table_stepped += cs;
        if (run[wi].first >= 0) {
            by_class[run[wi].first].push_back((int)wi);
        } else {
            const int per = 32 >> d.lg, items = plane_items_for(w.Y, w.Z, w.nw);
            for (int a = 0; a < items; ++a) b->ti.h[ii++] = PlaneItem{(int32_t)wi, a * per};
        }
        // full segments while `remaining` lasts; in the hybrid mode a young
        // world changes class once it is kYoungSteps old
        uint64_t hold = (uint64_t)std::max<int64_t>(1, w.remaining / S);
        const uint64_t age = w.t;
        if (b->cfg.use_smem == 3 && age < kYoungSteps) hold = std::min(hold, (kYoungSteps - age + S - 1) / S);
        reuse = std::min(reuse, hold);
        b->running.push_back(&w);
    }
    // per class, largest worlds first, so each launch ends with short work
    int* meta = b->tn.h;
    meta[0] = (int)ii;
    meta[kMetaWorlds] = (int)nw_;
    size_t si = 0;
    for (int c = 0; c < kAllClasses; ++c) {
        std::vector<int>& v = by_class[c];
        std::sort(v.begin(), v.end(), [&](int x, int y) {
            const PlaneWorld &a = b->tw.h[x], &e2 = b->tw.h[y];
            const int64_t ca = (int64_t)a.X * a.Y * a.Z * a.steps, cc = (int64_t)e2.X * e2.Y * e2.Z * e2.steps;
            return ca != cc ? ca > cc : x < y;
        });
        meta[1 + c] = (int)v.size();
        meta[1 + kAllClasses + c] = (int)si;
        for (int x : v) b->to.h[si++] = x;
    }
    uint32_t mask = 0;
    for (int c = 0; c < kAllClasses; ++c)
        if (!by_class[c].empty()) mask |= 1u << c;
    b->class_mask = mask;
    // admissions complete before the segment reads their planes
    for (auto& ev : b->pending_ready) FS3D_CUDA(cudaStreamWaitEvent(b->stream, ev.get(), 0));
    b->pending_ready.clear();
    for (auto& kv : b->worlds)
        if (kv.second.ready) {
            FS3D_CUDA(cudaStreamWaitEvent(b->stream, kv.second.ready, 0));
            cudaEventDestroy(kv.second.ready);
            kv.second.ready = nullptr;
        }
    // the tables go up through small kernels reading the page-locked images,
    // not the copy engines, which may be busy with hundreds of MB of grids
    FS3D_CUDA(b->tw.upload(nw_, b->stream));
    if (ii) FS3D_CUDA(b->ti.upload(ii, b->stream));
    if (si) FS3D_CUDA(b->to.upload(si, b->stream));
    FS3D_CUDA(b->tn.upload(kMetaInts, b->stream));
    FS3D_CUDA(cudaEventRecord(b->tables_free[b->tab_cur], b->stream));
    if (b->cfg.use_graphs && (!b->graph || b->graph_worlds != b->tw.d || b->graph_items != b->ti.d ||
                              b->graph_order != b->to.d || b->graph_mask != b->class_mask)) {
        s = capture_graph(b);
        if (s != FS3D_OK) {
            b->running.clear();
            return s;
        }
    }
    b->table_items = ii;
    b->reuse_left = reuse - 1;
    b->tables_stale = false;
    return FS3D_OK;
}

}  // namespace

extern "C" {

fs3d_status fs3d_batch_prepare(fs3d_batch* b) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_prepare: NULL batch");
    if (b->prepared && !b->tables_stale) return FS3D_OK;
    // an unchanged batch whose tables hold for another segment needs nothing
    if (!b->tables_stale && b->reuse_left > 0 && !b->running.empty()) return FS3D_OK;
    const fs3d_status s = build_tables(b);
    b->prepared = s == FS3D_OK;
    return s;
}

fs3d_status fs3d_batch_run_segment(fs3d_batch* b) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_run_segment: NULL batch");
    const int S = b->cfg.steps_per_segment;
    if (b->prepared && !b->tables_stale) {
        b->prepared = false;  // the tables fs3d_batch_prepare built are this segment's
        if (b->running.empty()) return FS3D_OK;
    } else if (!b->tables_stale && b->reuse_left > 0 && !b->running.empty()) {
        --b->reuse_left;  // the tables on the device are this segment's
    } else {
        b->prepared = false;
        const fs3d_status s = build_tables(b);
        if (s != FS3D_OK) return s;
        if (b->running.empty()) return FS3D_OK;
    }
    b->dense_cell_steps += b->table_dense;
    b->stepped_cell_steps += b->table_stepped;
    const size_t ii = b->table_items;
    if (b->cfg.use_graphs) {
        FS3D_CUDA(cudaGraphLaunch(ii ? b->graph_steps : b->graph, b->stream));
        note_launch((ii ? (uint64_t)S : 0u) + (uint64_t)resident_launches(b->cfg.use_smem, b->graph_mask) + 1u);
    } else {
        const fs3d_status s = enqueue_segment(b, b->stream, false, ii > 0);
        if (s != FS3D_OK) return s;
    }
    FS3D_CUDA(cudaEventRecord(b->last_segment, b->stream));
    std::shared_ptr<CUevent_st> fin;  // one event for every world that finishes in this segment
    for (BWorld* pw : b->running) {
        BWorld& w = *pw;
        const int steps = (int)(w.remaining < S ? w.remaining : S);
        w.t += (uint64_t)steps;
        w.remaining -= steps;
        if (w.remaining == 0) {
            w.done = true;
            if (!fin) {
                cudaEvent_t ev = nullptr;
                FS3D_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
                fin.reset(ev, [](CUevent_st* x) { cudaEventDestroy(x); });
                FS3D_CUDA(cudaEventRecord(ev, b->stream));
            }
            w.finished = fin;
        }
    }
    ++b->segments;
    return FS3D_OK;
}

fs3d_status fs3d_batch_sync(fs3d_batch* b, int64_t timeout_ns) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_sync: NULL batch");
    fs3d_status s = wait_stream(b->stream, timeout_ns);
    if (s != FS3D_OK) return s;
    int err = 0;
    FS3D_CUDA(cudaMemcpy(&err, b->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err)
        return set_error(FS3D_ERR_TIMEOUT,
                         "a shared-memory bulk copy did not complete in time: the segments from that one on "
                         "stepped nothing, so the worlds' states no longer match their step counters");
    s = wait_stream(b->side, timeout_ns);
    if (s == FS3D_OK) s = wait_stream(b->readback, timeout_ns);
    return s == FS3D_OK ? wait_stream(b->download, timeout_ns) : s;
}

fs3d_status fs3d_batch_poll(fs3d_batch* b, uint64_t ticket, int* done, uint64_t* hash) {
    if (!b || !done) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_poll: bad args");
    auto it = b->worlds.find(ticket);
    if (it == b->worlds.end()) return set_error(FS3D_ERR_NOT_FOUND, "fs3d_batch_poll: unknown ticket");
    BWorld& w = it->second;
    *done = 0;
    if (!w.done) return FS3D_OK;
    if (w.admit_id && hash) {
        const fs3d_status f = finalize_admits(b, w.admit_id, true);
        if (f != FS3D_OK) return f;
    }
    if (w.finished) {
        const cudaError_t q = cudaEventQuery(w.finished.get());
        if (q == cudaErrorNotReady) return FS3D_OK;
        if (q != cudaSuccess) return cuda_fail(q, "fs3d_batch_poll");
    }
    if (!w.hash_valid && hash) {
        if (w.ready) FS3D_CUDA(cudaStreamWaitEvent(b->side, w.ready, 0));
        fs3d_status s = planes_hash_async(w.rows, w.statics, w.X, w.Y, w.Z, b->hash_dev, b->side);
        if (s != FS3D_OK) return s;
        unsigned long long h = 0;
        FS3D_CUDA(cudaMemcpyAsync(&h, b->hash_dev, sizeof(h), cudaMemcpyDeviceToHost, b->side));
        FS3D_CUDA(cudaStreamSynchronize(b->side));
        w.hash = h;
        w.hash_valid = true;
    }
    *done = 1;
    if (hash) *hash = w.hash;
    return FS3D_OK;
}

fs3d_status fs3d_batch_poll_many(fs3d_batch* b, int n, const uint64_t* tickets, int* done, uint64_t* hashes) {
    if (!b || n < 0 || (n > 0 && (!tickets || !done)))
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_poll_many: bad args");
    std::vector<BWorld*> need;
    std::vector<int> need_at;
    for (int i = 0; i < n; ++i) {
        auto it = b->worlds.find(tickets[i]);
        if (it == b->worlds.end()) return set_error(FS3D_ERR_NOT_FOUND, "fs3d_batch_poll_many: unknown ticket");
        BWorld& w = it->second;
        done[i] = 0;
        if (!w.done) continue;
        if (w.admit_id && hashes) {
            const fs3d_status f = finalize_admits(b, w.admit_id, true);
            if (f != FS3D_OK) return f;
        }
        if (w.finished) {
            const cudaError_t q = cudaEventQuery(w.finished.get());
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) return cuda_fail(q, "fs3d_batch_poll_many");
        }
        done[i] = 1;
        if (!hashes) continue;
        if (w.hash_valid) {
            hashes[i] = w.hash;
        } else {
            need.push_back(&w);
            need_at.push_back(i);
        }
    }
    if (need.empty()) return FS3D_OK;
    // the hashes of every world still without one: one launch, one wait
    const int k = (int)need.size();
    std::vector<HashJob> jobs((size_t)k);
    for (int j = 0; j < k; ++j) {
        const BWorld& w = *need[(size_t)j];
        if (w.ready) FS3D_CUDA(cudaStreamWaitEvent(b->side, w.ready, 0));
        jobs[(size_t)j] = HashJob{w.rows, w.statics, w.X, w.Y, w.Z, w.nw};
    }
    // the kernel reads its jobs from, and writes the hashes into, one
    // page-locked chunk: no allocation and no copy-engine transfer on the way
    const size_t jobs_bytes = (sizeof(HashJob) * (size_t)k + 15) / 16 * 16;
    const size_t bytes = jobs_bytes + sizeof(unsigned long long) * (size_t)k;
    const int ci = take_chunk(b, bytes);
    if (ci < 0) return set_error(FS3D_ERR_CUDA, "fs3d_batch_poll_many: page-locked chunk");
    fs3d_batch::HostChunk& c = b->host_chunks[(size_t)ci];
    memcpy(c.p, jobs.data(), sizeof(HashJob) * (size_t)k);
    const unsigned long long* out_host = reinterpret_cast<const unsigned long long*>(c.p + jobs_bytes);
    fs3d_status s;
    if (c.dv) {
        s = planes_hash_many(reinterpret_cast<const HashJob*>(c.dv), k,
                             reinterpret_cast<unsigned long long*>(c.dv + jobs_bytes), b->side);
    } else {
        // a chunk the device cannot address: through device memory
        void* table = nullptr;
        FS3D_CUDA(stream_alloc(&table, bytes, b->side));
        cudaError_t e = cudaMemcpyAsync(table, c.p, jobs_bytes, cudaMemcpyHostToDevice, b->side);
        s = e == cudaSuccess ? planes_hash_many(static_cast<const HashJob*>(table), k,
                                                reinterpret_cast<unsigned long long*>(static_cast<char*>(table) +
                                                                                      jobs_bytes),
                                                b->side)
                             : cuda_fail(e, "fs3d_batch_poll_many jobs");
        if (s == FS3D_OK) {
            e = cudaMemcpyAsync(c.p + jobs_bytes, static_cast<char*>(table) + jobs_bytes, bytes - jobs_bytes,
                                cudaMemcpyDeviceToHost, b->side);
            if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_poll_many hashes");
        }
        cudaFreeAsync(table, b->side);
    }
    if (s == FS3D_OK) {
        cudaError_t e = cudaEventRecord(c.uploaded, b->side);  // the chunk is in use until here
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->side);
        if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_poll_many hashes");
    }
    if (s != FS3D_OK) return s;
    for (int j = 0; j < k; ++j) {
        BWorld& w = *need[(size_t)j];
        w.hash = out_host[j];
        w.hash_valid = true;
        hashes[need_at[(size_t)j]] = w.hash;
    }
    return FS3D_OK;
}

}  // extern "C"

namespace {

// Enqueues the read-back (if grid_out) and the release of one world on the
// side stream; `sync` waits for the read-back before returning.
fs3d_status retire(fs3d_batch* b, uint64_t ticket, uint8_t* grid_out, bool sync) {
    auto it = b->worlds.find(ticket);
    if (it == b->worlds.end()) return set_error(FS3D_ERR_NOT_FOUND, "fs3d_batch_retire: unknown ticket");
    BWorld& w = it->second;
    if (w.admit_id) {
        const fs3d_status f = finalize_admits(b, w.admit_id, true);
        if (f != FS3D_OK) return f;
    }
    FS3D_CUDA(cudaStreamWaitEvent(b->side, w.finished ? w.finished.get() : b->last_segment, 0));
    if (w.ready) FS3D_CUDA(cudaStreamWaitEvent(b->side, w.ready, 0));
    fs3d_status s = FS3D_OK;
    if (grid_out) {
        const size_t n = (size_t)w.X * w.Y * w.Z;
        uint8_t* staging = nullptr;
        FS3D_CUDA(stream_alloc(&staging, n, b->side));
        s = planes_to_bytes(w.rows, w.statics, w.X, w.Y, w.Z, staging, b->side);
        cudaError_t e = cudaSuccess;
        if (s == FS3D_OK) e = cudaMemcpyAsync(grid_out, staging, n, cudaMemcpyDeviceToHost, b->side);
        cudaFreeAsync(staging, b->side);
        if (e == cudaSuccess && sync) e = cudaStreamSynchronize(b->side);
        if (s == FS3D_OK && e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_retire readback");
    }
    b->used -= w.bytes;
    free_world(b, w);
    b->worlds.erase(it);
    b->tables_stale = true;
    return s;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// Admits specs[0..k) (k: as many as fit) with one upload per contiguous run,
// one conversion launch and one flag read-back.  With `wait` it returns once
// the callers' grids have been copied and the static-material flags read;
// otherwise once everything is enqueued (the grids must stay unchanged until
// the admission stream has run: fs3d_batch_wait_copies).
fs3d_status admit_many_impl(fs3d_batch* b, int n, const fs3d_world_spec* specs, uint64_t* tickets, int* n_admitted,
                            bool wait) {
    if (!b || n < 0 || (n > 0 && (!specs || !tickets)) || !n_admitted)
        return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_admit_many: bad args");
    *n_admitted = 0;
    // admit in order while the budget allows (static byte copies, found on the
    // device below, are charged on top)
    int k = 0;
    size_t used = b->used;
    for (; k < n; ++k) {
        const fs3d_world_spec& p = specs[k];
        if (!p.grid || p.X <= 0 || p.Y <= 0 || p.Z <= 0 || p.X > kPlaneMaxX || p.Y > 65536 || p.Z > 65536 ||
            p.n_steps < 0)
            return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_admit_many: bad world spec");
        const size_t need = plane_bytes(p.X, p.Y, p.Z) + layer_flag_bytes(p.Y) + sizeof(PlaneWorld);
        if (used + need > b->budget) break;
        used += need;
    }
    if (k == 0) return n ? set_error(FS3D_ERR_BUDGET, "fs3d_batch_admit_many: nothing fits in the budget now") : FS3D_OK;
    // older asynchronous admissions whose flags have arrived are completed
    // first, and memory whose read-backs have run is returned
    drain_deferred(b, false);
    fs3d_status s = finalize_admits(b, UINT64_MAX, false);
    if (s != FS3D_OK) return s;
    PendingAdmit pa;
    pa.id = b->next_admit_id++;
    pa.flags = take_flags(b, (size_t)k, &pa.flags_cap);
    if (!pa.flags) return set_error(FS3D_ERR_CUDA, "fs3d_batch_admit_many: page-locked flag buffer");
    // one staging buffer, one copy per run of contiguous grids, one conversion launch for all
    std::vector<ConvJob> jobs((size_t)k);
    std::vector<int64_t> unit_off((size_t)k);
    std::vector<uint4*> rows((size_t)k, nullptr);
    int64_t bytes_total = 0, units = 0;
    for (int a = 0; a < k; ++a) {
        const fs3d_world_spec& p = specs[a];
        ConvJob& j = jobs[(size_t)a];
        j.statics = nullptr;
        j.static_flag = nullptr;
        j.static_src = nullptr;
        j.byte_off = bytes_total;
        j.X = p.X;
        j.Y = p.Y;
        j.Z = p.Z;
        j.nw = plane_nw(p.X);
        unit_off[(size_t)a] = units;
        pa.tickets.push_back(0);
        pa.byte_off.push_back(bytes_total);
        pa.cells.push_back((int64_t)p.X * p.Y * p.Z);
        bytes_total += ((int64_t)p.X * p.Y * p.Z + 15) / 16 * 16;
        units += (int64_t)p.Y * p.Z * j.nw;
    }
    const size_t jobs_bytes = sizeof(ConvJob) * (size_t)k, off_bytes = sizeof(int64_t) * (size_t)k;
    const size_t flags_off = (jobs_bytes + off_bytes + 15) / 16 * 16;
    const size_t copy_off = (flags_off + sizeof(int) * (size_t)k + 15) / 16 * 16;
    const size_t copy_bytes = sizeof(CopyJob) * (size_t)k + sizeof(int64_t) * (size_t)k;
    const size_t bj_off = (copy_off + copy_bytes + 15) / 16 * 16;  // the conversion's job of each unit block
    const size_t table_bytes = bj_off + sizeof(int) * (size_t)conv_blocks(units);
    // the grid uploads run on their own stream: the next admission's upload
    // does not wait for this one's conversion (which waits for free SMs)
    cudaStream_t up = b->upload;
    {
        // an admission still holding this turn's staging bytes (kStagingRing
        // calls back) is completed first
        const uint64_t holder = b->up_ring[b->up_turn].admit_id;
        if (holder) {
            s = finalize_admits(b, holder, true);
            if (s != FS3D_OK) {
                b->flag_pool.emplace_back(pa.flags, pa.flags_cap);
                return s;
            }
        }
    }
    pa.slot = b->up_turn;
    cudaError_t e = cudaSuccess;
    fs3d_batch::StagingSlot* slot = take_slot(b->up_ring, b->up_turn, (size_t)bytes_total, up, &e);
    pa.staging = slot->p;
    slot->admit_id = pa.id;
    if (e == cudaSuccess) e = stream_alloc(&pa.table, table_bytes, b->side);
    // grids the device can address (page-locked host or device memory) that lie
    // back to back go over in one copy-engine transfer per run (the SMs stay
    // free for segments in flight); other device-addressable grids are gathered
    // by one copy kernel; pageable ones take a copy call each
    std::vector<CopyJob> copies;
    std::vector<int64_t> chunk_off;
    int64_t chunks = 0;
    // one block for all the worlds' planes and layer flags (freed with the last of them)
    std::vector<size_t> row_off((size_t)k);
    size_t block_bytes = 0;
    for (int a = 0; a < k; ++a) {
        row_off[(size_t)a] = block_bytes;
        block_bytes += (plane_bytes(specs[a].X, specs[a].Y, specs[a].Z) + layer_flag_bytes(specs[a].Y) + 255) & ~(size_t)255;
    }
    void* block = nullptr;
    if (e == cudaSuccess) e = admission_alloc(&block, block_bytes, b->side);
    for (int a = 0; a < k; ++a)
        rows[(size_t)a] = reinterpret_cast<uint4*>(static_cast<char*>(block) + row_off[(size_t)a]);
    uint8_t* staging = pa.staging;
    for (int a = 0; a < k && e == cudaSuccess;) {
        const int64_t cells = (int64_t)specs[a].X * specs[a].Y * specs[a].Z;
        const uint8_t* dv = device_view(specs[a].grid);
        int e_run = a + 1;  // [a, e_run): sources and staging both contiguous, no padding between,
                            // all in the first source's allocation
        int64_t run_bytes = cells;
        uintptr_t rs = 0;
        size_t rn = 0;
        const bool ranged = dv && alloc_range(specs[a].grid, &rs, &rn);
        while (ranged && e_run < k) {
            const int64_t c = (int64_t)specs[e_run].X * specs[e_run].Y * specs[e_run].Z;
            const int64_t c_prev = (int64_t)specs[e_run - 1].X * specs[e_run - 1].Y * specs[e_run - 1].Z;
            const uintptr_t g = reinterpret_cast<uintptr_t>(specs[e_run].grid);
            if (specs[e_run].grid != specs[e_run - 1].grid + c_prev ||
                run_bytes != jobs[(size_t)e_run].byte_off - jobs[(size_t)a].byte_off || g + (uintptr_t)c > rs + rn)
                break;
            run_bytes += c;
            ++e_run;
        }
        if (!dv || e_run - a > 1) {
            e = cudaMemcpyAsync(staging + jobs[(size_t)a].byte_off, specs[a].grid, (size_t)run_bytes, cudaMemcpyDefault,
                                up);
        } else {
            copies.push_back(CopyJob{dv, staging + jobs[(size_t)a].byte_off, cells});
            chunk_off.push_back(chunks);
            chunks += (cells + 15) / 16;
        }
        a = e_run;
    }
    int max_Y = 0;
    for (int a = 0; a < k; ++a) {
        ConvJob& j = jobs[(size_t)a];
        j.rows = rows[(size_t)a];
        j.lflags = reinterpret_cast<uint8_t*>(j.rows) + plane_bytes(j.X, j.Y, j.Z);
        j.t0b = (uint32_t)specs[a].start_step & 0xFFu;
        max_Y = std::max(max_Y, j.Y);
    }
    // the conversion (admission stream) follows the uploads
    if (e == cudaSuccess) {
        cudaEvent_t uploaded = nullptr;
        e = cudaEventCreateWithFlags(&uploaded, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(uploaded, up);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->side, uploaded, 0);
        if (uploaded) cudaEventDestroy(uploaded);
    }
    ConvJob* jobs_dev = static_cast<ConvJob*>(pa.table);
    int64_t* off_dev = reinterpret_cast<int64_t*>(static_cast<char*>(pa.table) + jobs_bytes);
    int* flags_dev = reinterpret_cast<int*>(static_cast<char*>(pa.table) + flags_off);
    pa.flags_dev = flags_dev;
    CopyJob* copies_dev = reinterpret_cast<CopyJob*>(static_cast<char*>(pa.table) + copy_off);
    int64_t* chunk_dev = reinterpret_cast<int64_t*>(static_cast<char*>(pa.table) + copy_off + sizeof(CopyJob) * (size_t)k);
    // the whole table (jobs, offsets, zeroed flags, copy jobs) in one upload
    // from a page-locked image, so nothing here waits for the grid uploads
    if (e == cudaSuccess) {
        const size_t image = table_bytes;
        const int ci = take_chunk(b, image);
        if (ci < 0) {
            e = cudaErrorMemoryAllocation;
        } else {
            char* h = b->host_chunks[(size_t)ci].p;
            memcpy(h, jobs.data(), jobs_bytes);
            memcpy(h + jobs_bytes, unit_off.data(), off_bytes);
            memset(h + flags_off, 0, copy_off - flags_off);
            if (!copies.empty()) {
                memcpy(h + copy_off, copies.data(), sizeof(CopyJob) * copies.size());
                memcpy(h + copy_off + sizeof(CopyJob) * (size_t)k, chunk_off.data(), sizeof(int64_t) * chunk_off.size());
            }
            conv_block_jobs(unit_off.data(), k, units, reinterpret_cast<int*>(h + bj_off));
            e = upload_chunk(b, ci, pa.table, image, b->side);
        }
    }
    if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_admit_many upload");
    if (s == FS3D_OK) s = copy_many(copies_dev, chunk_dev, (int)copies.size(), chunks, b->side);
    const int* bj_dev = reinterpret_cast<const int*>(static_cast<char*>(pa.table) + bj_off);
    if (s == FS3D_OK) s = planes_from_bytes_multi(jobs_dev, off_dev, bj_dev, k, units, staging, flags_dev, b->side);
    // layer flags from the cells: the first two steps evaluate only the row-pairs that can change
    if (s == FS3D_OK) s = layer_flags_from_cells_multi(jobs_dev, k, max_Y, b->side);
    // segments may start once the planes are written
    std::shared_ptr<CUevent_st> admitted;
    if (s == FS3D_OK) {
        admitted = shared_event();
        e = admitted ? cudaEventRecord(admitted.get(), b->side) : cudaErrorMemoryAllocation;
        pa.converted = admitted;
        if (e == cudaSuccess) {
            // the flags come down through a small kernel writing the page-locked
            // buffer (a copy-engine transfer would queue behind the read-backs)
            int* fv = reinterpret_cast<int*>(device_view(pa.flags));
            e = fv ? copy_small_async(fv, flags_dev, sizeof(int) * (size_t)k, b->side)
                   : cudaMemcpyAsync(pa.flags, flags_dev, sizeof(int) * (size_t)k, cudaMemcpyDeviceToHost, b->side);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pa.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(pa.done, b->side);
        if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_admit_many conversion");
    }
    if (s != FS3D_OK) {
        cudaStreamSynchronize(b->upload);  // no copy may still be writing the staging bytes
        cudaStreamSynchronize(b->side);
        slot->admit_id = 0;
        if (pa.table) cudaFreeAsync(pa.table, b->side);
        if (block) cudaFreeAsync(block, b->side);
        if (pa.done) cudaEventDestroy(pa.done);
        b->flag_pool.emplace_back(pa.flags, pa.flags_cap);
        return s;
    }
    cudaStream_t side = b->side;
    std::shared_ptr<void> arena(block, [side](void* p) { cudaFreeAsync(p, side); });
    for (int a = 0; a < k; ++a) {
        const fs3d_world_spec& p = specs[a];
        BWorld w;
        w.X = p.X;
        w.Y = p.Y;
        w.Z = p.Z;
        w.nw = plane_nw(p.X);
        w.seed = p.seed;
        w.t = p.start_step;
        w.remaining = p.n_steps;
        w.done = p.n_steps == 0;
        w.rows = rows[(size_t)a];
        w.arena = arena;
        w.lflags = reinterpret_cast<uint8_t*>(w.rows) + plane_bytes(p.X, p.Y, p.Z);
        w.flags_valid = true;
        w.bytes = plane_bytes(p.X, p.Y, p.Z) + layer_flag_bytes(p.Y) + sizeof(PlaneWorld);
        w.admit_id = pa.id;
        w.admit_index = a;
        w.admitted = admitted;
        b->used += w.bytes;
        tickets[a] = b->next_ticket++;
        pa.tickets[(size_t)a] = tickets[a];
        b->worlds.emplace(tickets[a], w);
    }
    b->tables_stale = true;
    b->pending_ready.push_back(admitted);
    const uint64_t id = pa.id;
    b->pending_admits.push_back(std::move(pa));
    // with `wait` the callers' grids may be reused once this returns; without,
    // few admissions stay open (each holds its staging bytes)
    s = wait ? finalize_admits(b, id, true)
             : (b->pending_admits.size() > 4 ? finalize_admits(b, b->pending_admits.front().id, true) : FS3D_OK);
    *n_admitted = k;
    if (s != FS3D_OK) return s;
    return k < n ? set_error(FS3D_ERR_BUDGET, "fs3d_batch_admit_many: the remaining worlds do not fit now") : FS3D_OK;
}

// An event after the read-back's conversion (null if none could be recorded).
std::shared_ptr<CUevent_st> record_read(cudaStream_t rb) {
    std::shared_ptr<CUevent_st> ev = shared_event();
    if (ev && cudaEventRecord(ev.get(), rb) != cudaSuccess) ev.reset();
    return ev;
}

// Retires tickets[0..n): the read-backs (conversion + copy into grids_out[a]
// where given) run on the read-back stream after each world's last segment;
// with `wait` it returns once the outputs hold the grids.  With `keep` the
// worlds stay in the batch (a snapshot of their current state): the next
// segment waits for the read-back's conversion.
fs3d_status retire_many_impl(fs3d_batch* b, int n, const uint64_t* tickets, uint8_t* const* grids_out, bool wait,
                             bool keep = false) {
    if (!b || n < 0 || (n > 0 && !tickets)) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_retire_many: bad args");
    std::vector<std::map<uint64_t, BWorld>::iterator> its;
    its.reserve((size_t)n);
    for (int a = 0; a < n; ++a) {
        auto it = b->worlds.find(tickets[a]);
        if (it == b->worlds.end()) return set_error(FS3D_ERR_NOT_FOUND, "fs3d_batch_retire_many: unknown ticket");
        its.push_back(it);
    }
    {
        std::vector<uint64_t> sorted(tickets, tickets + n);
        std::sort(sorted.begin(), sorted.end());
        if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
            return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_retire_many: a ticket appears twice");
    }
    // admissions whose flags have arrived are completed (static copies made);
    // a world whose admission is still open reads its static bytes, if its
    // flag says it has any, straight from that admission's staging bytes
    {
        const fs3d_status f = finalize_admits(b, UINT64_MAX, false);
        if (f != FS3D_OK) return f;
    }
    drain_deferred(b, false);
    auto pending_of = [&](uint64_t id) -> PendingAdmit* {
        for (PendingAdmit& p : b->pending_admits)
            if (p.id == id) return &p;
        return nullptr;
    };
    std::vector<PendingAdmit*> readers;  // open admissions whose staging bytes this read-back reads
    cudaStream_t rb = b->readback;
    {
        // each world's planes are final after its last segment (a world not
        // done yet: the last segment enqueued so far); admissions and static
        // copies must have run
        std::vector<CUevent_st*> deps;
        auto dep = [&](CUevent_st* ev) {
            if (ev && std::find(deps.begin(), deps.end(), ev) == deps.end()) deps.push_back(ev);
        };
        for (auto it : its) {
            const BWorld& w = it->second;
            dep(w.finished ? w.finished.get() : (b->segments ? b->last_segment : nullptr));
            dep(w.admitted.get());
            dep(w.ready);
            dep(w.statics_ready.get());
        }
        for (CUevent_st* ev : deps) FS3D_CUDA(cudaStreamWaitEvent(rb, ev, 0));
    }
    fs3d_status s = FS3D_OK;
    uint8_t* staging = nullptr;
    void* table = nullptr;
    std::shared_ptr<CUevent_st> read;    // recorded after the conversion
    std::shared_ptr<CUevent_st> copied;  // recorded after the copy kernel (download stream), if one ran
    fs3d_batch::StagingSlot* rb_slot = nullptr;  // the read-back's staging buffer
    if (grids_out) {
        std::vector<ConvJob> jobs;
        std::vector<int64_t> unit_off;
        std::vector<int> who;
        int64_t bytes_total = 0, units = 0;
        for (int a = 0; a < n; ++a) {
            if (!grids_out[a]) continue;
            const BWorld& w = its[(size_t)a]->second;
            ConvJob j;
            j.rows = w.rows;
            j.statics = w.statics;
            j.static_flag = nullptr;
            j.static_src = nullptr;
            if (w.admit_id)
                if (PendingAdmit* pa = pending_of(w.admit_id)) {
                    j.static_flag = pa->flags_dev + w.admit_index;
                    j.static_src = pa->staging + pa->byte_off[(size_t)w.admit_index];
                    if (std::find(readers.begin(), readers.end(), pa) == readers.end()) readers.push_back(pa);
                }
            j.byte_off = bytes_total;
            j.X = w.X;
            j.Y = w.Y;
            j.Z = w.Z;
            j.nw = w.nw;
            jobs.push_back(j);
            unit_off.push_back(units);
            who.push_back(a);
            bytes_total += ((int64_t)w.X * w.Y * w.Z + 15) / 16 * 16;
            units += (int64_t)w.Y * w.Z * w.nw;
        }
        const int k = (int)jobs.size();
        if (k) {
            const size_t jobs_bytes = sizeof(ConvJob) * (size_t)k;
            const size_t copy_off = (jobs_bytes + sizeof(int64_t) * (size_t)k + 15) / 16 * 16;
            const size_t bj_off = (copy_off + (sizeof(CopyJob) + sizeof(int64_t)) * (size_t)k + 15) / 16 * 16;
            const size_t table_bytes = bj_off + sizeof(int) * (size_t)conv_blocks(units);
            cudaError_t e = cudaSuccess;
            rb_slot = take_slot(b->rb_ring, b->rb_turn, (size_t)bytes_total, rb, &e);
            staging = rb_slot->p;
            if (e == cudaSuccess) e = stream_alloc(&table, table_bytes, rb);
            ConvJob* jobs_dev = static_cast<ConvJob*>(table);
            int64_t* off_dev = reinterpret_cast<int64_t*>(static_cast<char*>(table) + jobs_bytes);
            // the copy jobs are only known below: the table goes up in one
            // page-locked image once they are
            if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_retire_many upload");
            int ci = -1;
            const size_t image = table_bytes;
            if (s == FS3D_OK) {
                ci = take_chunk(b, image);
                if (ci < 0) s = set_error(FS3D_ERR_CUDA, "fs3d_batch_retire_many: page-locked table");
            }
            char* h = ci >= 0 ? b->host_chunks[(size_t)ci].p : nullptr;
            if (h) {
                memcpy(h, jobs.data(), jobs_bytes);
                memcpy(h + jobs_bytes, unit_off.data(), sizeof(int64_t) * (size_t)k);
                conv_block_jobs(unit_off.data(), k, units, reinterpret_cast<int*>(h + bj_off));
            }
            std::vector<CopyJob> copies;
            std::vector<int64_t> chunk_off;
            int64_t chunks = 0;
            std::vector<std::pair<int, int64_t>> runs;  // (first job, bytes) of each copy-engine run
            // outputs the device can address are written by one copy kernel,
            // pageable ones take a copy call each; outputs lying back to back
            // go back in one copy-engine transfer per run
            for (int q = 0; q < k && s == FS3D_OK;) {
                uint8_t* out = grids_out[who[(size_t)q]];
                const BWorld& w = its[(size_t)who[(size_t)q]]->second;
                const int64_t cells = (int64_t)w.X * w.Y * w.Z;
                uint8_t* dv = device_view(out);
                int e_run = q + 1;
                int64_t run_bytes = cells;
                uintptr_t rs = 0;
                size_t rn = 0;
                const bool ranged = dv && alloc_range(out, &rs, &rn);
                while (ranged && e_run < k) {
                    const BWorld& w2 = its[(size_t)who[(size_t)e_run]]->second;
                    const BWorld& w1 = its[(size_t)who[(size_t)e_run - 1]]->second;
                    // back to back in both, with no staging padding in between
                    // (a run copy must not write the caller's bytes between
                    // grids), and inside the first output's allocation (one copy
                    // may not span two)
                    const int64_t c1 = (int64_t)w1.X * w1.Y * w1.Z;
                    const uintptr_t g = reinterpret_cast<uintptr_t>(grids_out[who[(size_t)e_run]]);
                    if (grids_out[who[(size_t)e_run]] != grids_out[who[(size_t)e_run - 1]] + c1 ||
                        run_bytes != jobs[(size_t)e_run].byte_off - jobs[(size_t)q].byte_off ||
                        g + (uintptr_t)((int64_t)w2.X * w2.Y * w2.Z) > rs + rn)
                        break;
                    run_bytes += (int64_t)w2.X * w2.Y * w2.Z;
                    ++e_run;
                }
                if (!dv || e_run - q > 1) {
                    runs.emplace_back(q, run_bytes);
                } else {
                    copies.push_back(CopyJob{staging + jobs[(size_t)q].byte_off, dv, cells});
                    chunk_off.push_back(chunks);
                    chunks += (cells + 15) / 16;
                }
                q = e_run;
            }
            CopyJob* copies_dev = reinterpret_cast<CopyJob*>(static_cast<char*>(table) + copy_off);
            int64_t* chunk_dev =
                reinterpret_cast<int64_t*>(static_cast<char*>(table) + copy_off + sizeof(CopyJob) * (size_t)k);
            if (s == FS3D_OK) {
                if (!copies.empty()) {
                    memcpy(h + copy_off, copies.data(), sizeof(CopyJob) * copies.size());
                    memcpy(h + copy_off + sizeof(CopyJob) * (size_t)k, chunk_off.data(), sizeof(int64_t) * chunk_off.size());
                }
                e = upload_chunk(b, ci, table, image, rb);
                if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_retire_many upload");
            }
            const int* bj_dev = reinterpret_cast<const int*>(static_cast<char*>(table) + bj_off);
            if (s == FS3D_OK) s = planes_to_bytes_multi(jobs_dev, off_dev, bj_dev, k, units, staging, rb);
            if (s == FS3D_OK) read = record_read(rb);
            // the downloads run on their own stream: the next read-back's
            // conversion does not wait for this one's copies over the host link
            if (s == FS3D_OK && read) {
                e = cudaStreamWaitEvent(b->download, read.get(), 0);
                if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_retire_many ordering");
            }
            cudaStream_t dl = b->download;
            for (size_t r = 0; r < runs.size() && s == FS3D_OK; ++r) {
                const int q = runs[r].first;
                e = cudaMemcpyAsync(grids_out[who[(size_t)q]], staging + jobs[(size_t)q].byte_off, (size_t)runs[r].second,
                                    cudaMemcpyDefault, dl);
                if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_retire_many readback");
            }
            if (s == FS3D_OK && !copies.empty()) {
                s = copy_many(copies_dev, chunk_dev, (int)copies.size(), chunks, dl);
                // the copy kernel reads its jobs from `table` on the download
                // stream, which the read-back stream never waits for: the table
                // is freed once an event after that kernel has run
                if (s == FS3D_OK) {
                    copied = shared_event();
                    if (copied && cudaEventRecord(copied.get(), dl) != cudaSuccess) copied.reset();
                    if (!copied) cudaStreamSynchronize(dl);
                }
            }
        }
    }
    if (!read) read = record_read(rb);
    if (!read && s == FS3D_OK) s = set_error(FS3D_ERR_CUDA, "fs3d_batch_retire_many: event");
    // the staging buffer is free again after the downloads, the tables after
    // the conversion (and after the copy kernel, when one reads them)
    if (rb_slot) {
        mark_busy(rb_slot, b->download);
        mark_busy(rb_slot, rb);
    }
    if (table && copied) {
        // the conversion (read-back stream) precedes the copy kernel
        // (download stream waits for `read`), so `copied` covers both readers
        fs3d_batch::DeferredFree df;
        df.after = copied;
        df.ptrs = {table};
        b->deferred.push_back(std::move(df));
    } else if (table) {
        cudaFreeAsync(table, rb);
    }
    for (PendingAdmit* pa : readers) pa->reader = read;
    if (keep) {
        // the worlds stay: later segments must not change their planes before
        // the conversion has read them
        if (s == FS3D_OK) {
            const cudaError_t e = read ? cudaStreamWaitEvent(b->stream, read.get(), 0) : cudaStreamSynchronize(rb);
            if (e != cudaSuccess) s = cuda_fail(e, "fs3d_batch_read_many ordering");
        }
        if (wait && s == FS3D_OK) {
            FS3D_CUDA(cudaStreamSynchronize(rb));
            FS3D_CUDA(cudaStreamSynchronize(b->download));
        }
        return s;
    }
    // the worlds' memory goes back once the conversion has read it
    fs3d_batch::DeferredFree d;
    d.after = read;
    for (auto it : its) {
        BWorld& w = it->second;
        b->used -= w.bytes;
        if (w.arena) d.arenas.push_back(std::move(w.arena));
        else if (w.rows) d.ptrs.push_back(w.rows);
        if (w.statics) d.ptrs.push_back(w.statics);
        w.arena.reset();
        w.rows = nullptr;
        w.statics = nullptr;
        free_world(b, w);
        b->worlds.erase(it);
    }
    if (read) {
        b->deferred.push_back(std::move(d));
    } else {
        // no event: the conversion is waited for here
        cudaStreamSynchronize(rb);
        d.arenas.clear();
        for (void* p : d.ptrs) cudaFreeAsync(p, b->side);
    }
    if (!its.empty()) b->tables_stale = true;
    if (wait && s == FS3D_OK) {
        FS3D_CUDA(cudaStreamSynchronize(rb));
        FS3D_CUDA(cudaStreamSynchronize(b->download));
    }
    return s;
}

}  // namespace

extern "C" {

fs3d_status fs3d_batch_admit_many(fs3d_batch* b, int n, const fs3d_world_spec* specs, uint64_t* tickets,
                                  int* n_admitted) {
    return admit_many_impl(b, n, specs, tickets, n_admitted, true);
}

fs3d_status fs3d_batch_admit_many_async(fs3d_batch* b, int n, const fs3d_world_spec* specs, uint64_t* tickets,
                                        int* n_admitted) {
    return admit_many_impl(b, n, specs, tickets, n_admitted, false);
}

fs3d_status fs3d_batch_retire_many(fs3d_batch* b, int n, const uint64_t* tickets, uint8_t* const* grids_out) {
    return retire_many_impl(b, n, tickets, grids_out, true);
}

fs3d_status fs3d_batch_retire_many_async(fs3d_batch* b, int n, const uint64_t* tickets, uint8_t* const* grids_out) {
    return retire_many_impl(b, n, tickets, grids_out, false);
}

fs3d_status fs3d_batch_read_many(fs3d_batch* b, int n, const uint64_t* tickets, uint8_t* const* grids_out) {
    if (!grids_out) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_read_many: NULL outputs");
    return retire_many_impl(b, n, tickets, grids_out, true, true);
}

fs3d_status fs3d_batch_wait_copies(fs3d_batch* b, int64_t timeout_ns) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_wait_copies: NULL batch");
    fs3d_status s = wait_stream(b->readback, timeout_ns);
    if (s == FS3D_OK) s = wait_stream(b->download, timeout_ns);
    if (s == FS3D_OK) s = wait_stream(b->upload, timeout_ns);
    if (s == FS3D_OK) s = wait_stream(b->side, timeout_ns);
    if (s == FS3D_OK) s = finalize_admits(b, UINT64_MAX, false);
    if (s == FS3D_OK) drain_deferred(b, false);
    return s;
}

fs3d_status fs3d_batch_retire(fs3d_batch* b, uint64_t ticket, uint8_t* grid_out) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_retire: NULL batch");
    return retire(b, ticket, grid_out, true);
}

}  // extern "C"

namespace {

// tuned choices per batch shape: the count of live worlds per resident class
// (and of worlds too large to be resident), so a batch of the same make-up
// starts from the measured best
struct Tuning {
    int mode, promote, ctas_per_sm;
    bool operator==(const Tuning& o) const {
        return mode == o.mode && promote == o.promote && ctas_per_sm == o.ctas_per_sm;
    }
};
std::map<std::vector<int>, Tuning> g_tuned;
std::mutex g_tuned_mu;

std::vector<int> batch_shape(const fs3d_batch* b) {
    std::vector<int> h(kResidentClasses + 1, 0);
    for (auto& kv : b->worlds) {
        if (kv.second.done) continue;
        const int c = resident_class(kv.second.X, kv.second.Y, kv.second.Z);
        ++h[(size_t)(c < 0 ? kResidentClasses : c)];
    }
    return h;
}

// applies a launch configuration; the segment graph (which bakes in the
// per-step kernel's grid) is re-captured once the stream is idle
fs3d_status apply_tuning(fs3d_batch* b, const Tuning& t) {
    FS3D_CUDA(cudaStreamSynchronize(b->stream));
    b->cfg.use_smem = t.mode;
    b->promote = t.promote;
    b->tables_stale = true;
    b->grid = sm_count_public() * t.ctas_per_sm;
    return b->cfg.use_graphs ? capture_graph(b) : FS3D_OK;
}

// voxel-updates the next segment will perform
double segment_work(const fs3d_batch* b) {
    double v = 0.0;
    const int S = b->cfg.steps_per_segment;
    for (auto& kv : b->worlds) {
        const BWorld& w = kv.second;
        if (w.done) continue;
        v += (double)w.X * w.Y * w.Z * (double)(w.remaining < S ? w.remaining : S);
    }
    return v;
}

}  // namespace

extern "C" {

fs3d_status fs3d_batch_autotune(fs3d_batch* b, int trial_segments, fs3d_tune_report* out) {
    if (!b || trial_segments <= 0) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_autotune: bad args");
    if (out) memset(out, 0, sizeof(*out));
    const std::vector<int> shape = batch_shape(b);
    auto report = [&](const Tuning& t) {
        if (!out) return;
        out->mode = t.mode;
        out->promote = t.promote;
        out->ctas_per_sm = t.ctas_per_sm;
    };
    {
        std::lock_guard<std::mutex> lock(g_tuned_mu);
        auto it = g_tuned.find(shape);
        if (it != g_tuned.end()) {
            const fs3d_status s = apply_tuning(b, it->second);
            if (s != FS3D_OK) return s;
            report(it->second);
            if (out) out->cached = 1;
            return FS3D_OK;
        }
    }
    // candidates: resident kernels in global or shared memory (when resident
    // segments are on), two class promotions, and the per-step kernel's grid
    // only when some world is too large to be resident in both
    const int resident = plane_step_ctas_per_sm();
    bool stepped = false;
    for (auto& kv : b->worlds)
        if (!kv.second.done && resident_class(kv.second.X, kv.second.Y, kv.second.Z) < 0 &&
            resident_class_gm(kv.second.X, kv.second.Y, kv.second.Z) < 0)
            stepped = true;
    // the hybrid mode picks a world's memory by its age itself; an explicit
    // mode 1 or 2 is tuned between the two
    std::vector<Tuning> cand;
    const int m0 = b->cfg.use_smem;
    const std::vector<int> modes = m0 == 3 ? std::vector<int>{3} : (m0 ? std::vector<int>{2, 1} : std::vector<int>{0});
    for (int m : modes)
        for (int p = 0; p < (m ? 2 : 1); ++p)
            for (int cps : {resident, resident > 1 ? resident / 2 : resident}) {
                const Tuning t{m, p, (stepped || m == 0) ? cps : resident};
                if (std::find(cand.begin(), cand.end(), t) == cand.end()) cand.push_back(t);
            }
    cudaEvent_t e0, e1;
    FS3D_CUDA(cudaEventCreate(&e0));
    FS3D_CUDA(cudaEventCreate(&e1));
    double best_rate = -1.0;
    Tuning best{b->cfg.use_smem, b->promote, b->grid / sm_count_public()};
    fs3d_status s = FS3D_OK;
    int trials = 0, segments = 0;
    for (size_t ci = 0; ci < cand.size() && s == FS3D_OK; ++ci) {
        s = apply_tuning(b, cand[ci]);
        double rate = 0.0;
        for (int r = 0; r < trial_segments + 1 && s == FS3D_OK; ++r) {
            const double work = segment_work(b);
            if (work <= 0.0) break;
            cudaEventRecord(e0, b->stream);
            s = fs3d_batch_run_segment(b);
            ++segments;
            cudaEventRecord(e1, b->stream);
            if (s == FS3D_OK) s = cudaEventSynchronize(e1) == cudaSuccess ? FS3D_OK : cuda_fail(cudaGetLastError(), "autotune");
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0 && ms > 0.0f) rate = std::max(rate, work / ms);  // the first is a warm-up
        }
        if (out && trials < 8) out->trial_vox_per_ms[trials] = rate;
        ++trials;
        if (rate > best_rate) {
            best_rate = rate;
            best = cand[ci];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const fs3d_status sa = apply_tuning(b, best);
    if (s != FS3D_OK) return s;
    if (sa != FS3D_OK) return sa;
    if (best_rate > 0.0) {
        std::lock_guard<std::mutex> lock(g_tuned_mu);
        g_tuned[shape] = best;
    }
    report(best);
    if (out) {
        out->trials = trials;
        out->segments = segments;
        out->best_vox_per_ms = best_rate;
    }
    return FS3D_OK;
}

fs3d_status fs3d_batch_counters(fs3d_batch* b, uint64_t* dense_cell_steps, uint64_t* processed_cell_steps) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_counters: NULL batch");
    FS3D_CUDA(cudaStreamSynchronize(b->stream));
    unsigned long long dev = 0;
    FS3D_CUDA(cudaMemcpy(&dev, b->processed_dev, sizeof(dev), cudaMemcpyDeviceToHost));
    if (dense_cell_steps) *dense_cell_steps = b->dense_cell_steps;
    if (processed_cell_steps) *processed_cell_steps = (uint64_t)dev + b->stepped_cell_steps;
    return FS3D_OK;
}

fs3d_status fs3d_batch_stats(const fs3d_batch* b, int64_t* live_worlds, int64_t* live_cells, size_t* bytes_used,
                             size_t* bytes_budget) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_stats: NULL batch");
    int64_t cells = 0;
    for (auto& kv : b->worlds) cells += (int64_t)kv.second.X * kv.second.Y * kv.second.Z;
    if (live_worlds) *live_worlds = (int64_t)b->worlds.size();
    if (live_cells) *live_cells = cells;
    if (bytes_used) *bytes_used = b->used;
    if (bytes_budget) *bytes_budget = b->budget;
    return FS3D_OK;
}

fs3d_status fs3d_batch_stream(fs3d_batch* b, void** stream) {
    if (!b || !stream) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_stream: bad args");
    *stream = (void*)b->stream;
    return FS3D_OK;
}

fs3d_status fs3d_batch_destroy(fs3d_batch* b) {
    if (!b) return set_error(FS3D_ERR_INVALID_ARG, "fs3d_batch_destroy: NULL batch");
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->readback) cudaStreamSynchronize(b->readback);
    if (b->upload) cudaStreamSynchronize(b->upload);
    if (b->download) cudaStreamSynchronize(b->download);
    if (b->side) cudaStreamSynchronize(b->side);
    finalize_admits(b, UINT64_MAX, true);
    drain_deferred(b, true);
    for (auto& kv : b->worlds) free_world(b, kv.second);
    b->worlds.clear();
    b->pending_ready.clear();
    for (fs3d_batch::StagingSlot* ring : {b->up_ring, b->rb_ring})
        for (int i = 0; i < fs3d_batch::kStagingRing; ++i) {
            if (ring[i].p) cudaFreeAsync(ring[i].p, b->side);
            ring[i].p = nullptr;
            ring[i].busy.clear();
        }
    if (b->side) cudaStreamSynchronize(b->side);
    for (auto& f : b->flag_pool) cudaFreeHost(f.first);
    b->flag_pool.clear();
    for (auto& c : b->host_chunks) {
        cudaEventSynchronize(c.uploaded);
        cudaEventDestroy(c.uploaded);
        cudaFreeHost(c.p);
    }
    b->host_chunks.clear();
    if (b->graph) cudaGraphExecDestroy(b->graph);
    if (b->graph_steps) cudaGraphExecDestroy(b->graph_steps);
    b->tw.release();
    b->ti.release();
    b->tn.release();
    b->to.release();
    cudaFree(b->hash_dev);
    cudaFree(b->counter);
    cudaFree(b->err);
    cudaFree(b->processed_dev);
    if (b->fork) cudaEventDestroy(b->fork);
    for (int c = 0; c <= kAllClasses; ++c) {
        if (b->join[c]) cudaEventDestroy(b->join[c]);
        if (b->branch[c]) cudaStreamDestroy(b->branch[c]);
    }
    for (cudaEvent_t ev : b->tables_free)
        if (ev) cudaEventDestroy(ev);
    if (b->last_segment) cudaEventDestroy(b->last_segment);
    if (b->stream) cudaStreamDestroy(b->stream);
    if (b->side) cudaStreamDestroy(b->side);
    if (b->readback) cudaStreamDestroy(b->readback);
    if (b->upload) cudaStreamDestroy(b->upload);
    if (b->download) cudaStreamDestroy(b->download);
    delete b;
    return FS3D_OK;
}

}  // extern "C"
