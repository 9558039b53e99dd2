// rpm_server.cu -- incremental scene updates and the continuous-batching
// serving loop.
//
// Serving model (DRGBT-style replanning, apps/test_drgbt_random_obstacles.cpp
// and DRGBT.cpp:79-176, as a service): planners submit isValid / distance
// batches and edge batches of any size against resident scenes while moving
// obstacles are updated every few milliseconds.  One worker thread
//   * admits requests in arrival order as device memory of the budget frees up
//     (a request larger than the whole budget is rejected), skipping over
//     requests that do not fit yet so small ones are not held behind large ones;
//   * packs admitted requests -- from any scenes and robots, configuration and
//     edge requests alike -- into one batch per free slot (a slot is a
//     stream): one multi-segment launch for the configuration requests and one
//     multi-segment edge pipeline for the edge requests, so new requests join
//     the next batch while earlier batches still run and batches overlap on
//     the device.  A batch holds at most max_batch_configs units of work (an
//     edge counts 8), an eighth of that on the high-priority slots;
//   * retires batches by CUDA events, frees their memory and time-stamps every
//     request (submit, admit, launch, done).
// Each request's result is what the same check gives alone: configurations are
// evaluated independently, and a batch reads one consistent version of each
// scene.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <thread>
#include <unordered_map>

#include "rpm_ctx_impl.cuh"

namespace rpm {
namespace impl {

// ------------------------------------------------------ incremental update --
// Rows of m updated obstacles: [k][0] = index (bits), [k][1..6] = AABB.
__global__ void k_obstacle_update(float *rows_f, double *rows_d, int n_pad, const float *upd, int m) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const int j = __float_as_int(upd[7 * k]);
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        const float v = upd[7 * k + 1 + c];
        rows_f[c * n_pad + j] = v;
        rows_d[c * n_pad + j] = (double)v;
    }
}

// The next version of a scene: copy the current version device-to-device,
// scatter the m updated AABBs, rebuild the sorted copy, record 'ready'.  Checks issued afterwards wait
// on 'ready'; checks already issued keep reading the version they started on.
// Caller holds ctx->mu.
int scene_update(rpm_ctx *ctx, SceneRec *s, const int32_t *idx, const float *aabb, int32_t m) {
    for (int k = 0; k < m; ++k)
        for (int c = 0; c < 6; ++c) s->aabb[6 * (size_t)idx[k] + c] = aabb[6 * (size_t)k + c];
    if (!ctx->upd_stream) CK(cudaStreamCreateWithFlags(&ctx->upd_stream, cudaStreamNonBlocking));
    const int nxt = (s->cur + 1) % kRing;
    SceneBuf &cur = s->bufs[s->cur];
    SceneBuf &b = s->bufs[nxt];
    // checks still reading the version about to be overwritten finish first
    // (ordered on the device: the host never blocks here)
    stream_wait_users(ctx, b, ctx->upd_stream);
    // the pinned staging of this buffer is free once its last update ran;
    // otherwise this update copies from pageable memory
    const bool staging_free = !b.ready || cudaEventQuery(b.ready) == cudaSuccess;
    const size_t bytes = scene_bytes(*s);
    if (!b.mem) {
        if (cudaMalloc(&b.mem, bytes) != cudaSuccess) return fail(RPM_ERR_NOMEM, "scene version allocation failed");
        bind_scene_buf(*s, b);
    }
    if (!b.ready) CK(cudaEventCreateWithFlags(&b.ready, cudaEventDisableTiming));
    if (b.upd_cap < m) {
        if (b.ready) CK(cudaEventSynchronize(b.ready));   // growing the staging (rare): its last copy must be done
        if (b.upd_host) cudaFreeHost(b.upd_host);
        if (b.upd_dev) cudaFree(b.upd_dev);
        b.upd_cap = std::max(m, 64);
        if (cudaMallocHost(&b.upd_host, (size_t)b.upd_cap * 7 * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&b.upd_dev, (size_t)b.upd_cap * 7 * sizeof(float)) != cudaSuccess)
            return fail(RPM_ERR_NOMEM, "update staging allocation failed");
    }
    std::vector<float> pageable;
    float *stage = b.upd_host;
    if (!staging_free) {
        pageable.resize((size_t)m * 7);
        stage = pageable.data();
    }
    for (int k = 0; k < m; ++k) {
        int32_t j = idx[k];
        std::memcpy(&stage[7 * k], &j, sizeof j);
        for (int c = 0; c < 6; ++c) stage[7 * k + 1 + c] = aabb[6 * (size_t)k + c];
    }
    CK(cudaMemcpyAsync(b.mem, cur.mem, bytes, cudaMemcpyDeviceToDevice, ctx->upd_stream));
    if (m > 0) {
        CK(cudaMemcpyAsync(b.upd_dev, stage, (size_t)m * 7 * sizeof(float), cudaMemcpyHostToDevice, ctx->upd_stream));
        k_obstacle_update<<<(m + 127) / 128, 128, 0, ctx->upd_stream>>>(b.f, b.d, s->n_pad, b.upd_dev, m);
        CK(cudaGetLastError());
        CK(launch_scene_sort(*s, b, ctx->upd_stream));   // same order, new contents and block bounds
    }
    CK(cudaEventRecord(b.ready, ctx->upd_stream));
    b.pending = true;
    s->cur = nxt;
    s->version++;
    return RPM_OK;
}

}  // namespace impl
}  // namespace rpm

using namespace rpm;
using namespace rpm::impl;

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over [0, size) with 256-byte granules (host bookkeeping
// of the device arena).
struct Arena {
    size_t size = 0;
    std::list<std::pair<size_t, size_t>> free_;   // (offset, length), sorted
    void init(size_t n) { size = n; free_.clear(); free_.push_back({0, n}); }
    static size_t round(size_t n) { return (n + 255) & ~(size_t)255; }
    bool alloc(size_t n, size_t &off) {
        n = round(n);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= n) {
                off = it->first;
                it->first += n;
                it->second -= n;
                if (it->second == 0) free_.erase(it);
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t n) {
        n = round(n);
        auto it = free_.begin();
        while (it != free_.end() && it->first < off) ++it;
        it = free_.insert(it, {off, n});
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
        }
    }
};

struct Req {
    uint64_t ticket = 0;
    rpm_request r{};
    int D = 0, L = 0;
    size_t bytes = 0, off = 0;
    rpm_request_timing t{};
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    std::vector<Req *> reqs;
    bool busy = false;
    bool small = false;   // high-priority stream for batches of small requests
};

constexpr int64_t kSmallRequest = 8192;   // configurations (edges count x 8)
// Work per batch: a batch completes as a whole, so its size bounds the latency
// of every request in it.  32,768 units held p99 of requests up to 4,096
// configurations to 3.4 ms at 12,000 req/s of the serving trace (262,144: 9.7 ms)
// for 5 % less throughput at 20,000 req/s.
constexpr int32_t kDefaultBatchWork = 1 << 15;
constexpr double kAgeBoost = 0.050;       // a request waiting this long (s) is served as if small

int64_t work_of(const Req *q) { return q->r.kind == RPM_REQ_EDGES ? 8 * q->r.count : q->r.count; }

}  // namespace

struct rpm_server {
    rpm_ctx *ctx = nullptr;
    rpm_server_config cfg{};
    char *arena_mem = nullptr;
    Arena arena;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> incoming;   // submitted, not yet admitted
    std::deque<Req *> ready;      // admitted, waiting for a slot
    std::vector<Slot> slots;
    std::unordered_map<uint64_t, Req *> reqs;
    uint64_t next_ticket = 1;
    std::thread worker;
    bool stop = false;
    int64_t batches = 0;
};

namespace {

size_t request_bytes(const rpm_request &r, int D, int L) {
    const size_t n = (size_t)r.count;
    if (r.kind == RPM_REQ_EDGES)
        return Arena::round(2 * n * D * sizeof(float)) + Arena::round(n) + Arena::round(n * sizeof(int32_t));
    size_t b = Arena::round(n * D * sizeof(float));
    if (r.valid_host) b += Arena::round(n);
    if (r.dist_host) b += Arena::round(n * sizeof(double));
    if (r.profile_host) b += Arena::round(n * L * sizeof(float));
    return b;
}

// Device pointers of a request's buffers inside the arena.
struct DevBufs {
    float *q = nullptr, *q1 = nullptr, *q2 = nullptr;
    uint8_t *valid = nullptr;
    double *dist = nullptr;
    float *profile = nullptr;
    int32_t *checks = nullptr;
};

DevBufs layout(rpm_server *srv, const Req *q) {
    char *p = srv->arena_mem + q->off;
    const size_t n = (size_t)q->r.count;
    DevBufs d;
    if (q->r.kind == RPM_REQ_EDGES) {
        d.q1 = reinterpret_cast<float *>(p);
        d.q2 = d.q1 + n * q->D;
        p += Arena::round(2 * n * q->D * sizeof(float));
        d.valid = reinterpret_cast<uint8_t *>(p);
        p += Arena::round(n);
        d.checks = reinterpret_cast<int32_t *>(p);
        return d;
    }
    d.q = reinterpret_cast<float *>(p);
    p += Arena::round(n * q->D * sizeof(float));
    if (q->r.valid_host) { d.valid = reinterpret_cast<uint8_t *>(p); p += Arena::round(n); }
    if (q->r.dist_host) { d.dist = reinterpret_cast<double *>(p); p += Arena::round(n * sizeof(double)); }
    if (q->r.profile_host) d.profile = reinterpret_cast<float *>(p);
    return d;
}

// Launch one batch on a reserved slot: copies in, the checks, copies out.
// Called by the worker without srv->mu (the batch and the slot are its own);
// takes ctx->mu for the enqueue.
// versions[k] receives the scene version batch[k] reads.
int launch_batch(rpm_server *srv, Slot &slot, const std::vector<Req *> &batch, std::vector<uint64_t> &versions) {
    rpm_ctx *ctx = srv->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    std::vector<SegReq> segs;
    std::vector<EdgeReq> edges;
    int64_t n_edges = 0;
    versions.assign(batch.size(), 0);
    for (size_t k = 0; k < batch.size(); ++k) {
        Req *q = batch[k];
        const DevBufs d = layout(srv, q);
        const size_t n = (size_t)q->r.count;
        SceneRec *s = find_scene(ctx, q->r.scene_id);
        if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", q->r.scene_id);
        versions[k] = s->version;   // the launch reads s->cur, made current with this version
        if (q->r.kind == RPM_REQ_EDGES) {
            CK(cudaMemcpyAsync(d.q1, q->r.q1_host, n * q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
            CK(cudaMemcpyAsync(d.q2, q->r.q2_host, n * q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
            edges.push_back(EdgeReq{s, d.q1, d.q2, (int64_t)n, q->r.step, q->r.num_checks, d.valid, d.checks});
            n_edges += (int64_t)n;
        } else {
            CK(cudaMemcpyAsync(d.q, q->r.q_host, n * q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
            segs.push_back(SegReq{s, d.q, (int64_t)n, d.valid, d.dist, d.profile});
        }
    }
    if (!segs.empty()) {
        const int rc = enqueue_segments(ctx, srv->cfg.precision, segs, slot.st);
        if (rc) return rc;
    }
    if (n_edges > 0) {
        // every edge request of the batch in one pipeline (up to kMaxSegs requests per launch)
        Scratch *sc = nullptr;
        int rc = get_scratch(ctx, slot.st, 0, &sc);
        if (!rc) rc = edge_scratch(ctx, sc, n_edges, slot.st);
        if (!rc) {
            auto it = ctx->edge_ctas.find({edges[0].scene->robot, srv->cfg.precision});
            rc = enqueue_edge_batch(ctx, sc, srv->cfg.precision, edges, it == ctx->edge_ctas.end() ? 4 : it->second,
                                    slot.st);
        }
        if (rc) return rc;
        std::vector<SceneBuf *> used;
        for (const EdgeReq &r : edges) {
            SceneBuf *b = &r.scene->bufs[r.scene->cur];
            if (std::find(used.begin(), used.end(), b) == used.end()) used.push_back(b);
        }
        for (SceneBuf *b : used) {
            prune_users(ctx, *b);
            cudaEvent_t e = get_event(ctx);
            CK(cudaEventRecord(e, slot.st));
            b->users.push_back(e);
        }
    }
    for (Req *q : batch) {
        const DevBufs d = layout(srv, q);
        const size_t n = (size_t)q->r.count;
        if (q->r.valid_host) CK(cudaMemcpyAsync(q->r.valid_host, d.valid, n, cudaMemcpyDeviceToHost, slot.st));
        if (q->r.kind == RPM_REQ_EDGES) {
            if (q->r.checks_host)
                CK(cudaMemcpyAsync(q->r.checks_host, d.checks, n * sizeof(int32_t), cudaMemcpyDeviceToHost, slot.st));
        } else {
            if (q->r.dist_host) CK(cudaMemcpyAsync(q->r.dist_host, d.dist, n * sizeof(double), cudaMemcpyDeviceToHost, slot.st));
            if (q->r.profile_host)
                CK(cudaMemcpyAsync(q->r.profile_host, d.profile, n * q->L * sizeof(float), cudaMemcpyDeviceToHost, slot.st));
        }
    }
    CK(cudaEventRecord(slot.done, slot.st));
    return RPM_OK;
}

void worker_loop(rpm_server *srv) {
    cudaSetDevice(srv->ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    while (!srv->stop) {
        bool progress = false;
        // ---- retire finished batches
        for (Slot &sl : srv->slots) {
            if (!sl.busy || cudaEventQuery(sl.done) != cudaSuccess) continue;
            const double t = now_s();
            for (Req *q : sl.reqs) {
                q->t.t_done = t;
                q->t.status = 0;
                srv->arena.release(q->off, q->bytes);
            }
            sl.reqs.clear();
            sl.busy = false;
            progress = true;
            srv->cv_done.notify_all();
        }
        // ---- admit in arrival order as memory frees up
        for (auto it = srv->incoming.begin(); it != srv->incoming.end();) {
            Req *q = *it;
            if (q->bytes > srv->arena.size) {
                q->t.status = RPM_ERR_ADMISSION;
                q->t.t_done = now_s();
                it = srv->incoming.erase(it);
                srv->cv_done.notify_all();
                continue;
            }
            size_t off;
            if (srv->arena.alloc(q->bytes, off)) {
                q->off = off;
                q->t.t_admit = now_s();
                srv->ready.push_back(q);
                it = srv->incoming.erase(it);
                progress = true;
            } else {
                ++it;
            }
        }
        // ---- launch batches on free slots: smallest requests first; the
        //      high-priority slots take batches of small (or long-waiting) requests
        if (!srv->ready.empty()) {
            std::stable_sort(srv->ready.begin(), srv->ready.end(),
                             [](const Req *a, const Req *b) { return work_of(a) < work_of(b); });
        }
        const double tnow = now_s();
        for (Slot &sl : srv->slots) {
            if (srv->ready.empty()) break;
            if (sl.busy) continue;
            // work cap of the batch: small on the high-priority slots so their
            // requests finish quickly; configuration and edge requests mix
            const int64_t cap = sl.small ? std::max<int64_t>(1, srv->cfg.max_batch_configs / 8) : srv->cfg.max_batch_configs;
            std::vector<Req *> batch;
            int64_t work = 0;
            int nseg = 0, nedge = 0;
            for (auto it = srv->ready.begin(); it != srv->ready.end();) {
                Req *q = *it;
                const bool edge = q->r.kind == RPM_REQ_EDGES;
                const bool small = work_of(q) <= kSmallRequest || tnow - q->t.t_submit > kAgeBoost;
                if (sl.small && !small) { ++it; continue; }
                if (!batch.empty() && (work + work_of(q) > cap || (edge ? nedge : nseg) >= srv->cfg.max_batch_segments)) {
                    ++it;
                    continue;
                }
                batch.push_back(q);
                work += work_of(q);
                (edge ? nedge : nseg) += 1;
                it = srv->ready.erase(it);
            }
            if (batch.empty()) continue;
            sl.busy = true;   // reserved: only this thread touches the slot
            const double t = now_s();
            lk.unlock();      // submissions and polls proceed while the batch is enqueued
            std::vector<uint64_t> versions;
            const int rc = launch_batch(srv, sl, batch, versions);
            lk.lock();
            for (size_t k = 0; k < batch.size(); ++k) {
                Req *q = batch[k];
                q->t.t_launch = t;
                q->t.batch_size = (int32_t)batch.size();
                q->t.scene_version = k < versions.size() ? versions[k] : 0;
            }
            if (rc) {
                // work already queued for the batch may still use its memory: let it finish first
                cudaStreamSynchronize(sl.st);
                cudaGetLastError();
                const double te = now_s();
                for (Req *q : batch) { q->t.status = rc; q->t.t_done = te; srv->arena.release(q->off, q->bytes); }
                sl.busy = false;
                srv->cv_done.notify_all();
            } else {
                sl.reqs = batch;
                srv->batches++;
            }
            progress = true;
        }
        if (!progress) {
            bool busy = false;
            for (Slot &sl : srv->slots) busy = busy || sl.busy;
            if (busy) {
                lk.unlock();
                std::this_thread::yield();
                lk.lock();
            } else {
                srv->cv_work.wait_for(lk, std::chrono::microseconds(200));
            }
        }
    }
}

}  // namespace

extern "C" {

int rpm_server_create(rpm_ctx *ctx, const rpm_server_config *cfg, rpm_server **out) {
    if (!ctx || !out) return fail(RPM_ERR_INVALID, "NULL argument");
    rpm_server_config c{4, RPM_PREC_FP32_RECHECK, (int64_t)8 << 30, kMaxSegs, kDefaultBatchWork};
    if (cfg) c = *cfg;
    if (c.num_slots < 1 || c.num_slots > 64) return fail(RPM_ERR_INVALID, "num_slots must be 1..64");
    if (c.precision < RPM_PREC_FP64 || c.precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision");
    if (c.max_batch_segments < 1 || c.max_batch_segments > kMaxSegs) c.max_batch_segments = kMaxSegs;
    if (c.max_batch_configs < 1) c.max_batch_configs = kDefaultBatchWork;
    if (c.memory_budget < (1 << 20)) return fail(RPM_ERR_INVALID, "memory budget below 1 MiB");
    rpm_server *srv = new rpm_server();
    srv->ctx = ctx;
    srv->cfg = c;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (set_device(ctx)) { delete srv; return RPM_ERR_CUDA; }
        if (cudaMalloc(&srv->arena_mem, (size_t)c.memory_budget) != cudaSuccess) {
            delete srv;
            return fail(RPM_ERR_NOMEM, "server arena of %lld bytes could not be allocated", (long long)c.memory_budget);
        }
        srv->arena.init((size_t)c.memory_budget);
        srv->slots.resize(c.num_slots);
        int lo_prio = 0, hi_prio = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
        const int n_small = std::max(1, c.num_slots / 2);
        for (int k = 0; k < c.num_slots; ++k) {
            Slot &sl = srv->slots[k];
            sl.small = k < n_small && c.num_slots > 1;
            CK(cudaStreamCreateWithPriority(&sl.st, cudaStreamNonBlocking, sl.small ? hi_prio : lo_prio));
            CK(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
            Scratch *sc = nullptr;   // pre-size scratch so the loop never allocates
            // sized for requests up to 262,144 configurations, which run as batches of their own
            const int64_t presize = std::max<int64_t>(c.max_batch_configs, 1 << 18);
            int rc = get_scratch(ctx, sl.st, presize, &sc);
            if (!rc) rc = edge_scratch(ctx, sc, presize / 4, sl.st);
            if (rc) return rc;
        }
    }
    srv->worker = std::thread(worker_loop, srv);
    *out = srv;
    return RPM_OK;
}

int rpm_server_submit(rpm_server *srv, const rpm_request *r, uint64_t *ticket) {
    if (!srv || !r || !ticket) return fail(RPM_ERR_INVALID, "NULL argument");
    if (r->count < 0) return fail(RPM_ERR_INVALID, "negative count");
    if (r->kind != RPM_REQ_CONFIGS && r->kind != RPM_REQ_EDGES) return fail(RPM_ERR_INVALID, "unknown request kind");
    if (r->count > 0 && (r->kind == RPM_REQ_CONFIGS ? !r->q_host : (!r->q1_host || !r->q2_host || !r->valid_host)))
        return fail(RPM_ERR_INVALID, "missing request buffers");
    const int dofs = scene_dofs(srv->ctx, r->scene_id);
    if (dofs < 0) return fail(RPM_ERR_INVALID, "unknown scene %d", r->scene_id);
    Req *q = new Req();
    q->r = *r;
    q->D = dofs;
    q->L = dofs;
    q->bytes = request_bytes(q->r, q->D, q->L);
    q->t.status = 1;
    q->t.t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        q->ticket = srv->next_ticket++;
        srv->reqs[q->ticket] = q;
        srv->incoming.push_back(q);
    }
    srv->cv_work.notify_one();
    *ticket = q->ticket;
    return RPM_OK;
}

int rpm_server_poll(rpm_server *srv, uint64_t ticket, rpm_request_timing *out) {
    if (!srv || !out) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return fail(RPM_ERR_INVALID, "unknown ticket");
    *out = it->second->t;
    return RPM_OK;
}

int rpm_server_wait(rpm_server *srv, uint64_t ticket, double timeout_s, rpm_request_timing *out) {
    if (!srv || !out) return fail(RPM_ERR_INVALID, "NULL argument");
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return fail(RPM_ERR_INVALID, "unknown ticket");
    Req *q = it->second;
    const bool ok = srv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return q->t.status != 1; });
    *out = q->t;
    if (!ok) return fail(RPM_ERR_TIMEOUT, "request %llu still pending", (unsigned long long)ticket);
    return RPM_OK;
}

int rpm_server_release(rpm_server *srv, uint64_t ticket) {
    if (!srv) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(ticket);
    if (it == srv->reqs.end()) return fail(RPM_ERR_INVALID, "unknown ticket");
    if (it->second->t.status == 1) return fail(RPM_ERR_INVALID, "request still pending");
    delete it->second;
    srv->reqs.erase(it);
    return RPM_OK;
}

int rpm_server_replay(rpm_server *srv, const rpm_request *reqs, const double *arrival_s, int64_t n,
                      const rpm_motion *motions, int32_t n_motions, double period_s, rpm_request_timing *out) {
    if (!srv || (n > 0 && (!reqs || !arrival_s || !out))) return fail(RPM_ERR_INVALID, "NULL argument");
    // moving obstacles: initial AABBs per (scene, obstacle)
    struct Mover { int32_t scene, idx; float v[3]; float a0[6]; };
    std::vector<Mover> movers;
    {
        std::lock_guard<std::mutex> lk(srv->ctx->mu);
        for (int k = 0; k < n_motions; ++k) {
            SceneRec *s = find_scene(srv->ctx, motions[k].scene_id);
            if (!s || motions[k].index < 0 || motions[k].index >= s->n) return fail(RPM_ERR_INVALID, "bad motion %d", k);
            Mover m{motions[k].scene_id, motions[k].index, {motions[k].velocity[0], motions[k].velocity[1], motions[k].velocity[2]}, {}};
            for (int c = 0; c < 6; ++c) m.a0[c] = s->aabb[6 * (size_t)m.idx + c];
            movers.push_back(m);
        }
    }
    std::vector<uint64_t> tickets((size_t)n, 0);
    const double t0 = now_s();
    std::atomic<bool> done_submitting(false);
    std::thread updater;
    std::atomic<int> upd_rc(RPM_OK);
    if (!movers.empty() && period_s > 0) {
        updater = std::thread([&] {
            cudaSetDevice(srv->ctx->device);
            std::map<int32_t, std::vector<const Mover *>> by_scene;
            for (const Mover &m : movers) by_scene[m.scene].push_back(&m);
            double next = t0 + period_s;
            std::vector<int32_t> idx;
            std::vector<float> ab;
            while (!done_submitting.load()) {
                while (now_s() < next && !done_submitting.load()) std::this_thread::sleep_for(std::chrono::microseconds(50));
                const float t = (float)(now_s() - t0);
                for (auto &kv : by_scene) {
                    idx.clear();
                    ab.clear();
                    for (const Mover *m : kv.second) {   // constant velocity (Environment::updateEnvironment, straight lines)
                        idx.push_back(m->idx);
                        for (int c = 0; c < 6; ++c) ab.push_back(m->a0[c] + m->v[c % 3] * t);
                    }
                    std::lock_guard<std::mutex> lk(srv->ctx->mu);
                    SceneRec *s = find_scene(srv->ctx, kv.first);
                    const int rc = s ? scene_update(srv->ctx, s, idx.data(), ab.data(), (int32_t)idx.size()) : RPM_ERR_INVALID;
                    if (rc) upd_rc.store(rc);
                }
                next += period_s;
            }
        });
    }
    int rc = RPM_OK;
    for (int64_t i = 0; i < n && !rc; ++i) {
        const double due = t0 + arrival_s[i];
        while (now_s() < due) {
            if (due - now_s() > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
        rc = rpm_server_submit(srv, &reqs[i], &tickets[i]);
    }
    for (int64_t i = 0; i < n; ++i) {
        if (!tickets[i]) continue;
        rpm_request_timing t{};
        const int w = rpm_server_wait(srv, tickets[i], 600.0, &t);
        if (w && !rc) rc = w;
        t.t_submit -= t0; t.t_admit -= t0; t.t_launch -= t0; t.t_done -= t0;
        out[i] = t;
        rpm_server_release(srv, tickets[i]);
    }
    done_submitting.store(true);
    if (updater.joinable()) updater.join();
    return rc ? rc : upd_rc.load();
}

int rpm_server_stats(rpm_server *srv, int64_t *batches, int64_t *pending) {
    if (!srv) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    if (batches) *batches = srv->batches;
    if (pending) *pending = (int64_t)(srv->incoming.size() + srv->ready.size());
    return RPM_OK;
}

int rpm_server_destroy(rpm_server *srv) {
    if (!srv) return RPM_OK;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    if (srv->worker.joinable()) srv->worker.join();
    cudaSetDevice(srv->ctx->device);
    for (Slot &sl : srv->slots) {
        if (sl.st) cudaStreamSynchronize(sl.st);
    }
    {
        std::lock_guard<std::mutex> lk(srv->ctx->mu);
        for (Slot &sl : srv->slots) {
            auto it = srv->ctx->scratch.find(sl.st);
            if (it != srv->ctx->scratch.end()) {
                free_scratch(it->second);
                srv->ctx->scratch.erase(it);
            }
            cudaStreamDestroy(sl.st);
            cudaEventDestroy(sl.done);
        }
    }
    cudaFree(srv->arena_mem);
    for (auto &kv : srv->reqs) delete kv.second;
    delete srv;
    return RPM_OK;
}

}  // extern "C"
