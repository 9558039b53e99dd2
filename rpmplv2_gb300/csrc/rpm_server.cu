// rpm_server.cu -- incremental scene updates and the continuous-batching
// serving loop.
//
// Serving model (DRGBT-style replanning, apps/test_drgbt_random_obstacles.cpp
// and DRGBT.cpp:79-176, as a service): planners submit isValid / distance
// batches and edge batches of any size against resident scenes while moving
// obstacles are updated every few milliseconds.  Two worker threads (one per
// class below)
//   * admits requests in arrival order as device memory of the budget frees up
//     (a request larger than the whole budget is rejected), skipping over
//     requests that do not fit yet so small ones are not held behind large ones;
//   * sorts them into two classes.  Express requests (at most express_work
//     units of work; an edge counts 8) run on high-priority streams, in
//     arrival order, each in a batch of its own unless it is below
//     kExpressShared units (those share batches up to that size); they carry
//     a small share of the work, so they find a stream and the SMs free.
//     Bulk requests run on low-priority streams, in arrival order, packed up
//     to max_batch_configs units per batch, and every batch runs as a chain
//     of launches of at most chunk_work units: short launches keep each CTA
//     short, so the block scheduler hands SMs to express kernels quickly.
//     Optionally the bulk streams live in an SM partition (a green context)
//     so some SMs only ever run express work;
//   * packs the requests of a batch -- from any scenes and robots,
//     configuration and edge requests alike -- into multi-segment launches
//     (configurations) and multi-segment edge pipelines (edges);
//   * completes a batch's requests in a host callback at the end of its
//     stream work, then retires the batch: frees its memory and time-stamps
//     every request (submit, admit, launch, done, and a device-side trace of
//     the batch's copies and checks).
// Each request's result is what the same check gives alone: configurations are
// evaluated independently, and a batch reads one consistent version of each
// scene (the version current when the batch was enqueued, kept for all its
// launches).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <limits>
#include <list>
#include <thread>
#include <unordered_map>

#include <cuda.h>   // driver types only: the green-context calls go through the runtime's entry points

#include "rpm_ctx_impl.cuh"

namespace rpm {
namespace impl {

// ------------------------------------------------------ incremental update --
// The next version of each listed scene: one kernel (k_scene_update_many)
// copies the current version, scatters the updated AABBs and rebuilds the
// sorted copy, one CTA per scene; 'ready' of each new version is recorded
// after it.  Checks issued afterwards wait on 'ready'; checks already issued
// keep reading the versions they started on, and the update stream first waits
// (on the device) for the checks still reading the buffers it overwrites.
// Descriptors and rows go through a pinned staging ring read by the kernel in
// place, so an update costs one launch plus an event per scene.  Caller holds
// ctx->mu.
int scene_update_many(rpm_ctx *ctx, const std::vector<SceneUpd> &ups) {
    if (ups.empty()) return RPM_OK;
    for (size_t a = 0; a < ups.size(); ++a)
        for (size_t b = a + 1; b < ups.size(); ++b)
            if (ups[a].s == ups[b].s) return fail(RPM_ERR_INVALID, "a scene appears twice in one update");
    if (!ctx->upd_stream) CK(cudaStreamCreateWithFlags(&ctx->upd_stream, cudaStreamNonBlocking));
    // staging: descriptors, then each scene's rows
    size_t bytes = ups.size() * sizeof(UpdDesc);
    for (const SceneUpd &u : ups) bytes += ((size_t)u.m * 7 * sizeof(float) + 15) & ~(size_t)15;
    const int slot = ctx->upd_next;
    ctx->upd_next = (slot + 1) % rpm_ctx::kUpdRing;
    if (!ctx->upd_done[slot]) CK(cudaEventCreateWithFlags(&ctx->upd_done[slot], cudaEventDisableTiming));
    else CK(cudaEventSynchronize(ctx->upd_done[slot]));   // its last kernel has read it (normally long done)
    if (ctx->upd_cap[slot] < bytes) {
        if (ctx->upd_stage[slot]) cudaFreeHost(ctx->upd_stage[slot]);
        ctx->upd_cap[slot] = std::max<size_t>(bytes * 2, 4096);
        if (cudaMallocHost(&ctx->upd_stage[slot], ctx->upd_cap[slot]) != cudaSuccess) {
            ctx->upd_stage[slot] = nullptr;
            ctx->upd_cap[slot] = 0;
            return fail(RPM_ERR_NOMEM, "update staging allocation failed");
        }
    }
    UpdDesc *descs = reinterpret_cast<UpdDesc *>(ctx->upd_stage[slot]);
    unsigned char *rows = ctx->upd_stage[slot] + ups.size() * sizeof(UpdDesc);
    for (size_t k = 0; k < ups.size(); ++k) {
        const SceneUpd &u = ups[k];
        SceneRec *s = u.s;
        for (int i = 0; i < u.m; ++i)
            for (int c = 0; c < 6; ++c) s->aabb[6 * (size_t)u.idx[i] + c] = u.aabb[6 * (size_t)i + c];
        const int nxt = (s->cur + 1) % kRing;
        SceneBuf &cur = s->bufs[s->cur];
        SceneBuf &b = s->bufs[nxt];
        // checks still reading the version about to be overwritten finish first
        stream_wait_users(ctx, b, ctx->upd_stream);
        if (!b.mem) {
            if (cudaMalloc(&b.mem, scene_bytes(*s)) != cudaSuccess) return fail(RPM_ERR_NOMEM, "scene version allocation failed");
            bind_scene_buf(*s, b);
        }
        if (!b.ready) CK(cudaEventCreateWithFlags(&b.ready, cudaEventDisableTiming));
        float *r = reinterpret_cast<float *>(rows);
        for (int i = 0; i < u.m; ++i) {
            const int32_t j = u.idx[i];
            std::memcpy(&r[7 * i], &j, sizeof j);
            for (int c = 0; c < 6; ++c) r[7 * i + 1 + c] = u.aabb[6 * (size_t)i + c];
        }
        descs[k] = UpdDesc{cur.f, cur.d, cur.perm, b.f, b.d, b.sf, b.sd, b.blk, b.perm, r, s->n_pad, s->ns, u.m, 0};
        rows += ((size_t)u.m * 7 * sizeof(float) + 15) & ~(size_t)15;
    }
    CK(launch_scene_update_many(descs, (int)ups.size(), ctx->upd_stream));
    CK(cudaEventRecord(ctx->upd_done[slot], ctx->upd_stream));
    for (const SceneUpd &u : ups) {
        SceneRec *s = u.s;
        const int nxt = (s->cur + 1) % kRing;
        SceneBuf &b = s->bufs[nxt];
        CK(cudaEventRecord(b.ready, ctx->upd_stream));
        b.pending = true;
        s->cur = nxt;
        s->version++;
    }
    return RPM_OK;
}

int scene_update(rpm_ctx *ctx, SceneRec *s, const int32_t *idx, const float *aabb, int32_t m) {
    return scene_update_many(ctx, {SceneUpd{s, idx, aabb, m}});
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
    uint64_t version = 0;           // the scene version its checks read (set before its launches)
    bool retired = false;           // its slot's worker has read the batch trace and freed its memory
    bool release_pending = false;   // released by the caller before that: the worker deletes it
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t trace[3] = {nullptr, nullptr, nullptr};   // batch start, copies in done, checks done
    std::vector<Req *> reqs;
    bool busy = false;
    bool express = false;   // high-priority stream for small requests
    bool finished = false;   // set (under srv->mu) by the stream's host callback at the end of the batch
    void *srv = nullptr;
};

// Defaults of rpm_server_config (a field of 0 takes its default).
// Chosen on the serving trace (64 scenes, Poisson 12k and 20k requests/s,
// sizes 1-65,536): 4 bulk streams in chunks of 65,536 units held capacity
// (16.1k req/s with the partition below) while 24 express streams kept express
// requests from queueing for a stream (queue p99 0.18 ms at 12k req/s).
constexpr int32_t kDefaultBulkSlots = 4;
constexpr int32_t kDefaultExpressSlots = 24;
constexpr int32_t kDefaultExpressWork = 8192;   // units: configurations, an edge counting 8
constexpr int32_t kDefaultBatchWork = 1 << 16;  // bulk batch
constexpr int32_t kDefaultChunkWork = 1 << 16;  // bulk launch
// Default bulk partition: all SMs but this many stay free of bulk work (p99 of
// 2k-8k requests at 12k req/s, two runs each: 1.05 / 0.97 ms with 32 free,
// 0.95 / 0.94 ms with 48, 1.26 / 0.98 ms with 64; capacity 24.1k, 23.0k and
// 21.7k req/s).
constexpr int32_t kDefaultExpressOnlySms = 48;
constexpr int64_t kExpressShared = 1024;        // express requests below this share batches

// Units of work: a configuration 1, an edge 8, a horizon state (spines,
// underestimations and a distance) 64, a motion one per validity point.
int64_t work_of(const Req *q) {
    switch (q->r.kind) {
    case RPM_REQ_EDGES: return 8 * q->r.count;
    case RPM_REQ_REACHED: return 64 * q->r.count;
    case RPM_REQ_MOTION: return (int64_t)std::max(1, q->r.num_points) * q->r.count;
    default: return q->r.count;
    }
}

// An SM partition for the bulk streams (a green context of the device's
// primary context).  Its driver calls are reached through the runtime's driver
// entry points, so the library needs no link against the driver.
struct GreenPartition {
    CUgreenCtx g = nullptr;
    unsigned sms = 0;
    CUresult (*stream_create)(CUstream *, CUgreenCtx, unsigned, int) = nullptr;
    CUresult (*stream_destroy)(CUstream) = nullptr;
    CUresult (*destroy)(CUgreenCtx) = nullptr;
};

template <typename F> bool driver_fn(const char *name, F &fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, CUDART_VERSION, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p)
        return false;
    fn = reinterpret_cast<F>(p);
    return true;
}

// A green context of at least 'want' SMs of 'device' (rounded as the driver
// requires).  Returns RPM_OK or an error with a message.
int make_partition(int device, unsigned want, GreenPartition &gp) {
    CUresult (*device_get)(CUdevice *, int) = nullptr;
    CUresult (*get_resource)(CUdevice, CUdevResource *, CUdevResourceType) = nullptr;
    CUresult (*split)(CUdevResource *, unsigned *, const CUdevResource *, CUdevResource *, unsigned, unsigned) = nullptr;
    CUresult (*gen_desc)(CUdevResourceDesc *, CUdevResource *, unsigned) = nullptr;
    CUresult (*create)(CUgreenCtx *, CUdevResourceDesc, CUdevice, unsigned) = nullptr;
    if (!driver_fn("cuDeviceGet", device_get) || !driver_fn("cuDeviceGetDevResource", get_resource) ||
        !driver_fn("cuDevSmResourceSplitByCount", split) || !driver_fn("cuDevResourceGenerateDesc", gen_desc) ||
        !driver_fn("cuGreenCtxCreate", create) || !driver_fn("cuGreenCtxStreamCreate", gp.stream_create) ||
        !driver_fn("cuStreamDestroy", gp.stream_destroy) || !driver_fn("cuGreenCtxDestroy", gp.destroy))
        return fail(RPM_ERR_CUDA, "green contexts are not available from this driver");
    CUdevice dev;
    CUdevResource all, part, rest;
    unsigned groups = 1;
    CUdevResourceDesc desc;
    if (device_get(&dev, device) != CUDA_SUCCESS || get_resource(dev, &all, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS)
        return fail(RPM_ERR_CUDA, "querying the device's SMs failed");
    if (want >= all.sm.smCount) return fail(RPM_ERR_INVALID, "bulk_sms %u leaves no SM of %u to express work", want, all.sm.smCount);
    if (split(&part, &groups, &all, &rest, 0, want) != CUDA_SUCCESS || groups != 1 ||
        gen_desc(&desc, &part, 1) != CUDA_SUCCESS || create(&gp.g, desc, dev, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS)
        return fail(RPM_ERR_CUDA, "creating an SM partition of %u SMs failed", want);
    gp.sms = part.sm.smCount;
    return RPM_OK;
}

}  // namespace

struct rpm_server {
    rpm_ctx *ctx = nullptr;
    rpm_server_config cfg{};
    char *arena_mem = nullptr;
    Arena arena;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> incoming;   // submitted, not yet admitted
    std::deque<Req *> express;    // admitted small requests, in arrival order
    std::deque<Req *> bulk;       // admitted large requests, in arrival order
    std::vector<Slot> slots;
    std::unordered_map<uint64_t, Req *> reqs;
    uint64_t next_ticket = 1;
    std::thread worker, bulk_worker;
    bool stop = false;
    int64_t batches = 0;
    GreenPartition bulk_part;   // bulk streams' SMs (when cfg.bulk_sms > 0)
};

namespace {

size_t request_bytes(const rpm_request &r, int D, int L) {
    const size_t n = (size_t)r.count;
    if (r.kind == RPM_REQ_EDGES || r.kind == RPM_REQ_MOTION)
        return Arena::round(2 * n * D * sizeof(float)) + Arena::round(n) + Arena::round(n * sizeof(int32_t));
    if (r.kind == RPM_REQ_REACHED)
        return Arena::round(D * sizeof(float)) + 2 * Arena::round(n * D * sizeof(float)) +
               Arena::round(n * sizeof(int32_t)) + (r.dist_host ? Arena::round(n * sizeof(double)) : 0);
    size_t b = Arena::round(n * D * sizeof(float));
    if (r.valid_host) b += Arena::round(n);
    if (r.dist_host) b += Arena::round(n * sizeof(double));
    if (r.profile_host) b += Arena::round(n * L * sizeof(float));
    return b;
}

// Device pointers of a request's buffers inside the arena.
struct DevBufs {
    float *q = nullptr, *q1 = nullptr, *q2 = nullptr, *q_out = nullptr;
    uint8_t *valid = nullptr;
    double *dist = nullptr;
    float *profile = nullptr;
    int32_t *checks = nullptr, *status = nullptr;
};

DevBufs layout(rpm_server *srv, const Req *q) {
    char *p = srv->arena_mem + q->off;
    const size_t n = (size_t)q->r.count;
    DevBufs d;
    if (q->r.kind == RPM_REQ_EDGES || q->r.kind == RPM_REQ_MOTION) {
        d.q1 = reinterpret_cast<float *>(p);
        d.q2 = d.q1 + n * q->D;
        p += Arena::round(2 * n * q->D * sizeof(float));
        d.valid = reinterpret_cast<uint8_t *>(p);
        p += Arena::round(n);
        d.checks = reinterpret_cast<int32_t *>(p);
        return d;
    }
    if (q->r.kind == RPM_REQ_REACHED) {
        d.q = reinterpret_cast<float *>(p);   // q_current
        p += Arena::round(q->D * sizeof(float));
        d.q1 = reinterpret_cast<float *>(p);  // horizon
        p += Arena::round(n * q->D * sizeof(float));
        d.q_out = reinterpret_cast<float *>(p);
        p += Arena::round(n * q->D * sizeof(float));
        d.status = reinterpret_cast<int32_t *>(p);
        p += Arena::round(n * sizeof(int32_t));
        if (q->r.dist_host) d.dist = reinterpret_cast<double *>(p);
        return d;
    }
    d.q = reinterpret_cast<float *>(p);
    p += Arena::round(n * q->D * sizeof(float));
    if (q->r.valid_host) { d.valid = reinterpret_cast<uint8_t *>(p); p += Arena::round(n); }
    if (q->r.dist_host) { d.dist = reinterpret_cast<double *>(p); p += Arena::round(n * sizeof(double)); }
    if (q->r.profile_host) d.profile = reinterpret_cast<float *>(p);
    return d;
}

// Host callback at the end of a batch's stream work.  Every result is in the
// callers' host buffers by then, so the batch's requests complete here
// (status, t_done, the scene version read) and their waiters wake; the slot is
// marked finished and the workers wake too (they sleep instead of polling
// events), and the slot's worker retires it later (trace, arena memory)
// without holding the requests up.  It calls no CUDA function.
void CUDART_CB batch_done(void *arg) {
    Slot *sl = static_cast<Slot *>(arg);
    rpm_server *srv = static_cast<rpm_server *>(sl->srv);
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        sl->finished = true;
        const double t = now_s();
        for (Req *q : sl->reqs) {
            q->t.t_done = t;
            q->t.scene_version = q->version;
            q->t.status = 0;
        }
    }
    srv->cv_work.notify_all();
    srv->cv_done.notify_all();
}

// Launch one batch on a reserved slot: copies in, the checks as launches of at
// most 'chunk' units of work each, copies out.  Every launch of the batch is
// enqueued here under ctx->mu, so all of them read the scene versions current
// now.  Called by the worker without srv->mu (the batch and the slot are its
// own).  versions[k] receives the scene version batch[k] reads.
int launch_batch(rpm_server *srv, Slot &slot, const std::vector<Req *> &batch, int64_t chunk,
                 std::vector<uint64_t> &versions) {
    rpm_ctx *ctx = srv->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    std::vector<SceneRec *> scene(batch.size(), nullptr);
    versions.assign(batch.size(), 0);
    CK(cudaEventRecord(slot.trace[0], slot.st));
    for (size_t k = 0; k < batch.size(); ++k) {
        Req *q = batch[k];
        const DevBufs d = layout(srv, q);
        const size_t n = (size_t)q->r.count;
        SceneRec *s = find_scene(ctx, q->r.scene_id);
        if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", q->r.scene_id);
        scene[k] = s;
        versions[k] = s->version;   // the launches read s->cur, made current with this version
        batch[k]->version = s->version;
        if (q->r.kind == RPM_REQ_EDGES || q->r.kind == RPM_REQ_MOTION) {
            CK(cudaMemcpyAsync(d.q1, q->r.q1_host, n * q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
            CK(cudaMemcpyAsync(d.q2, q->r.q2_host, n * q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
        } else if (q->r.kind == RPM_REQ_REACHED) {
            CK(cudaMemcpyAsync(d.q, q->r.q_host, q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
            CK(cudaMemcpyAsync(d.q1, q->r.q1_host, n * q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
        } else {
            CK(cudaMemcpyAsync(d.q, q->r.q_host, n * q->D * sizeof(float), cudaMemcpyHostToDevice, slot.st));
        }
    }
    CK(cudaEventRecord(slot.trace[1], slot.st));
    // configuration requests, cut into launches of at most 'chunk' configurations
    std::vector<SegReq> segs;
    int64_t segw = 0;
    auto flush_segs = [&]() -> int {
        if (segs.empty()) return RPM_OK;
        const int rc = enqueue_segments(ctx, srv->cfg.precision, segs, slot.st);
        segs.clear();
        segw = 0;
        return rc;
    };
    for (size_t k = 0; k < batch.size(); ++k) {
        const Req *q = batch[k];
        if (q->r.kind != RPM_REQ_CONFIGS) continue;
        const DevBufs d = layout(srv, q);
        for (int64_t first = 0; first < q->r.count;) {
            const int64_t cnt = std::min(q->r.count - first, chunk - segw);
            segs.push_back(SegReq{scene[k], d.q + first * q->D, cnt, d.valid ? d.valid + first : nullptr,
                                  d.dist ? d.dist + first : nullptr, d.profile ? d.profile + first * q->L : nullptr});
            segw += cnt;
            first += cnt;
            if (segw >= chunk || (int)segs.size() == kMaxSegs) {
                const int rc = flush_segs();
                if (rc) return rc;
            }
        }
    }
    int rc = flush_segs();
    if (rc) return rc;
    // edge requests, cut into pipelines of at most 'chunk' units (8 per edge)
    const int64_t echunk = std::max<int64_t>(1, chunk / 8);
    std::vector<std::vector<EdgeReq>> groups(1);
    int64_t ew = 0, emax = 0;
    for (size_t k = 0; k < batch.size(); ++k) {
        const Req *q = batch[k];
        if (q->r.kind != RPM_REQ_EDGES) continue;
        const DevBufs d = layout(srv, q);
        for (int64_t first = 0; first < q->r.count;) {
            const int64_t cnt = std::min(q->r.count - first, echunk - ew);
            groups.back().push_back(EdgeReq{scene[k], d.q1 + first * q->D, d.q2 + first * q->D, cnt, q->r.step,
                                            q->r.num_checks, d.valid + first, d.checks + first});
            ew += cnt;
            first += cnt;
            emax = std::max(emax, ew);
            if (ew >= echunk || (int)groups.back().size() == kMaxSegs) {
                groups.emplace_back();
                ew = 0;
            }
        }
    }
    if (emax > 0) {
        Scratch *sc = nullptr;
        rc = get_scratch(ctx, slot.st, 0, &sc);
        if (!rc) rc = edge_scratch(ctx, sc, emax, slot.st);
        if (rc) return rc;
        std::vector<SceneBuf *> used;
        for (const auto &g : groups) {
            if (g.empty()) continue;
            rc = enqueue_edge_batch(ctx, sc, srv->cfg.precision, g, 4, slot.st);
            if (rc) return rc;
            for (const EdgeReq &r : g) {
                SceneBuf *b = &r.scene->bufs[r.scene->cur];
                if (std::find(used.begin(), used.end(), b) == used.end()) used.push_back(b);
            }
        }
        for (SceneBuf *b : used) {
            prune_users(ctx, *b);
            cudaEvent_t e = get_event(ctx);
            CK(cudaEventRecord(e, slot.st));
            b->users.push_back(e);
        }
    }
    // the DRGBT steps, one call per request
    for (size_t k = 0; k < batch.size(); ++k) {
        const Req *q = batch[k];
        const DevBufs d = layout(srv, q);
        if (q->r.kind == RPM_REQ_REACHED) {
            rc = reached_states_locked(ctx, q->r.scene_id, srv->cfg.precision, d.q, d.q1, q->r.count, q->r.spine,
                                       d.q_out, d.status, d.dist, slot.st);
        } else if (q->r.kind == RPM_REQ_MOTION) {
            // the reference's own numerics unless the server runs the FP64 form
            const int32_t prec = srv->cfg.precision == RPM_PREC_FP64 ? RPM_PREC_FP64 : RPM_PREC_FP32_REF;
            rc = motion_validity_locked(ctx, q->r.scene_id, prec, d.q1, d.q2, q->r.count, q->r.boxes, q->r.num_boxes,
                                        q->r.max_iter_time, q->r.num_points, d.valid, d.checks, slot.st);
        }
        if (rc) return rc;
    }
    CK(cudaEventRecord(slot.trace[2], slot.st));
    for (Req *q : batch) {
        const DevBufs d = layout(srv, q);
        const size_t n = (size_t)q->r.count;
        if (q->r.kind == RPM_REQ_REACHED) {
            CK(cudaMemcpyAsync(q->r.q_out_host, d.q_out, n * q->D * sizeof(float), cudaMemcpyDeviceToHost, slot.st));
            CK(cudaMemcpyAsync(q->r.status_host, d.status, n * sizeof(int32_t), cudaMemcpyDeviceToHost, slot.st));
            if (q->r.dist_host) CK(cudaMemcpyAsync(q->r.dist_host, d.dist, n * sizeof(double), cudaMemcpyDeviceToHost, slot.st));
            continue;
        }
        if (q->r.valid_host) CK(cudaMemcpyAsync(q->r.valid_host, d.valid, n, cudaMemcpyDeviceToHost, slot.st));
        if (q->r.kind == RPM_REQ_EDGES || q->r.kind == RPM_REQ_MOTION) {
            if (q->r.checks_host)
                CK(cudaMemcpyAsync(q->r.checks_host, d.checks, n * sizeof(int32_t), cudaMemcpyDeviceToHost, slot.st));
        } else {
            if (q->r.dist_host) CK(cudaMemcpyAsync(q->r.dist_host, d.dist, n * sizeof(double), cudaMemcpyDeviceToHost, slot.st));
            if (q->r.profile_host)
                CK(cudaMemcpyAsync(q->r.profile_host, d.profile, n * q->L * sizeof(float), cudaMemcpyDeviceToHost, slot.st));
        }
    }
    CK(cudaEventRecord(slot.done, slot.st));
    CK(cudaLaunchHostFunc(slot.st, batch_done, &slot));
    return RPM_OK;
}

// One worker per class: the express worker retires and launches the express
// slots, the bulk worker the bulk slots, so enqueueing a bulk batch never holds
// up an express launch on the host.  Either admits new requests.
void worker_loop(rpm_server *srv, bool express) {
    cudaSetDevice(srv->ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    while (!srv->stop) {
        bool progress = false;
        // ---- retire finished batches
        for (Slot &sl : srv->slots) {
            if (sl.express != express) continue;
            if (!sl.busy || !sl.finished) continue;
            sl.finished = false;
            float ms[3] = {0.f, 0.f, 0.f};
            cudaEventElapsedTime(&ms[0], sl.trace[0], sl.trace[1]);
            cudaEventElapsedTime(&ms[1], sl.trace[1], sl.trace[2]);
            cudaEventElapsedTime(&ms[2], sl.trace[2], sl.done);
            const double t = now_s();
            for (Req *q : sl.reqs) {   // status and t_done normally set by the batch's callback
                if (q->t.status == 1) { q->t.t_done = t; q->t.status = 0; }
                q->t.h2d_ms = ms[0];
                q->t.kernel_ms = ms[1];
                q->t.d2h_ms = ms[2];
                srv->arena.release(q->off, q->bytes);
                q->retired = true;
                if (q->release_pending) delete q;
            }
            sl.reqs.clear();
            sl.busy = false;
            progress = true;
            srv->cv_done.notify_all();
        }
        // ---- admit in arrival order as memory frees up, into the two classes
        for (auto it = srv->incoming.begin(); it != srv->incoming.end();) {
            Req *q = *it;
            if (q->bytes > srv->arena.size) {
                q->t.status = RPM_ERR_ADMISSION;
                q->t.t_done = now_s();
                q->retired = true;
                it = srv->incoming.erase(it);
                srv->cv_done.notify_all();
                continue;
            }
            size_t off;
            if (srv->arena.alloc(q->bytes, off)) {
                q->off = off;
                q->t.t_admit = now_s();
                (work_of(q) <= srv->cfg.express_work ? srv->express : srv->bulk).push_back(q);
                it = srv->incoming.erase(it);
                progress = true;
            } else {
                ++it;
            }
        }
        // ---- launch: express slots take express requests, bulk slots bulk
        //      requests, each class in arrival order
        for (Slot &sl : srv->slots) {
            if (sl.express != express || sl.busy) continue;
            std::deque<Req *> &queue = sl.express ? srv->express : srv->bulk;
            if (queue.empty()) continue;
            // an express batch is one request, or several requests smaller than
            // kExpressShared units: a batch completes as a whole, so sharing one
            // would add the others' work to a request's latency
            const int64_t cap = sl.express ? kExpressShared : srv->cfg.max_batch_configs;
            std::vector<Req *> batch;
            int64_t work = 0;
            int nseg = 0, nedge = 0;
            while (!queue.empty()) {
                Req *q = queue.front();
                const bool edge = q->r.kind == RPM_REQ_EDGES;
                if (!batch.empty() && (work + work_of(q) > cap || (edge ? nedge : nseg) >= srv->cfg.max_batch_segments))
                    break;
                batch.push_back(q);
                work += work_of(q);
                (edge ? nedge : nseg) += 1;
                queue.pop_front();
            }
            sl.busy = true;   // reserved: only this thread touches the slot
            sl.reqs = batch;  // before the callback can run: it completes these requests
            const double t = now_s();
            for (Req *q : batch) {
                q->t.t_launch = t;
                q->t.batch_size = (int32_t)batch.size();
            }
            lk.unlock();      // submissions and polls proceed while the batch is enqueued
            std::vector<uint64_t> versions;
            const int64_t chunk = sl.express ? std::numeric_limits<int64_t>::max() / 16 : (int64_t)srv->cfg.chunk_work;
            const int rc = launch_batch(srv, sl, batch, chunk, versions);
            const float enq_ms = (float)((now_s() - t) * 1e3);
            lk.lock();
            for (size_t k = 0; k < batch.size(); ++k) {   // (the batch may have completed already)
                Req *q = batch[k];
                q->t.enqueue_ms = enq_ms;
            }
            if (rc) {
                // work already queued for the batch may still use its memory: let it finish first
                cudaStreamSynchronize(sl.st);
                cudaGetLastError();
                sl.finished = false;   // a callback enqueued before the failure may have run
                const double te = now_s();
                for (Req *q : batch) {
                    q->t.status = rc;
                    q->t.t_done = te;
                    srv->arena.release(q->off, q->bytes);
                    q->retired = true;
                }
                sl.reqs.clear();
                sl.busy = false;
                srv->cv_done.notify_all();
            } else {
                srv->batches++;
            }
            progress = true;
        }
        if (progress) srv->cv_work.notify_all();   // the other worker may have new work or memory
        else srv->cv_work.wait_for(lk, std::chrono::milliseconds(2));   // woken by submissions and batch ends
    }
}

}  // namespace

extern "C" {

int rpm_server_create(rpm_ctx *ctx, const rpm_server_config *cfg, rpm_server **out) {
    if (!ctx || !out) return fail(RPM_ERR_INVALID, "NULL argument");
    rpm_server_config c{kDefaultBulkSlots, RPM_PREC_FP32_RECHECK, (int64_t)8 << 30, kMaxSegs, kDefaultBatchWork,
                        kDefaultExpressSlots, kDefaultExpressWork, kDefaultChunkWork, 0, 0};
    if (cfg) c = *cfg;
    if (c.num_slots == 0) c.num_slots = kDefaultBulkSlots;
    if (c.express_slots == 0) c.express_slots = kDefaultExpressSlots;
    if (c.num_slots < 1 || c.num_slots > 64 || c.express_slots < 1 || c.express_slots > 64)
        return fail(RPM_ERR_INVALID, "num_slots and express_slots must be 1..64");
    if (c.precision < RPM_PREC_FP64 || c.precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision");
    if (c.max_batch_segments < 1 || c.max_batch_segments > kMaxSegs) c.max_batch_segments = kMaxSegs;
    if (c.max_batch_configs < 1) c.max_batch_configs = kDefaultBatchWork;
    if (c.express_work < 1) c.express_work = kDefaultExpressWork;
    if (c.chunk_work < 8) c.chunk_work = kDefaultChunkWork;
    if (c.memory_budget < (1 << 20)) return fail(RPM_ERR_INVALID, "memory budget below 1 MiB");
    if (c.bulk_sms < -1) return fail(RPM_ERR_INVALID, "bulk_sms below -1");
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
        if (c.bulk_sms > 0) {
            const int rc = make_partition(ctx->device, (unsigned)c.bulk_sms, srv->bulk_part);
            if (rc) { cudaFree(srv->arena_mem); delete srv; return rc; }
        } else if (c.bulk_sms == 0 && ctx->num_sms > 2 * kDefaultExpressOnlySms) {
            // the default partition where the driver offers green contexts; bulk
            // work uses every SM where it does not
            if (make_partition(ctx->device, (unsigned)(ctx->num_sms - kDefaultExpressOnlySms), srv->bulk_part) != RPM_OK)
                srv->bulk_part = GreenPartition{};
        }
        srv->slots.resize(c.express_slots + c.num_slots);
        int lo_prio = 0, hi_prio = 0;
        CK(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
        for (int k = 0; k < (int)srv->slots.size(); ++k) {
            Slot &sl = srv->slots[k];
            sl.express = k < c.express_slots;
            sl.srv = srv;
            if (!sl.express && srv->bulk_part.g) {
                CUstream cs = nullptr;
                if (srv->bulk_part.stream_create(&cs, srv->bulk_part.g, CU_STREAM_NON_BLOCKING, lo_prio) != CUDA_SUCCESS)
                    return fail(RPM_ERR_CUDA, "creating a stream in the bulk partition failed");
                sl.st = (cudaStream_t)cs;
            } else {
                CK(cudaStreamCreateWithPriority(&sl.st, cudaStreamNonBlocking, sl.express ? hi_prio : lo_prio));
            }
            CK(cudaEventCreate(&sl.done));   // timed: the batch trace ends on it
            for (cudaEvent_t &e : sl.trace) CK(cudaEventCreate(&e));
            Scratch *sc = nullptr;   // pre-size scratch so the loop never allocates
            // express batches hold up to express_work units; bulk launches chunk_work units
            const int64_t presize = sl.express ? c.express_work : c.chunk_work;
            int rc = get_scratch(ctx, sl.st, presize, &sc);
            if (!rc) rc = edge_scratch(ctx, sc, std::max<int64_t>(1, presize / 8), sl.st);
            if (rc) return rc;
        }
    }
    srv->worker = std::thread(worker_loop, srv, true);
    srv->bulk_worker = std::thread(worker_loop, srv, false);
    *out = srv;
    return RPM_OK;
}

int rpm_server_submit(rpm_server *srv, const rpm_request *r, uint64_t *ticket) {
    if (!srv || !r || !ticket) return fail(RPM_ERR_INVALID, "NULL argument");
    if (r->count < 0) return fail(RPM_ERR_INVALID, "negative count");
    if (r->kind < RPM_REQ_CONFIGS || r->kind > RPM_REQ_MOTION) return fail(RPM_ERR_INVALID, "unknown request kind");
    bool ok = true;
    if (r->count > 0) {
        switch (r->kind) {
        case RPM_REQ_CONFIGS: ok = r->q_host != nullptr; break;
        case RPM_REQ_EDGES: ok = r->q1_host && r->q2_host && r->valid_host; break;
        case RPM_REQ_REACHED: ok = r->q_host && r->q1_host && r->q_out_host && r->status_host && r->spine; break;
        default: ok = r->q1_host && r->q2_host && r->valid_host && r->num_points >= 1 && r->num_boxes >= 0 &&
                      (r->num_boxes == 0 || r->boxes);
        }
    }
    if (!ok) return fail(RPM_ERR_INVALID, "missing request buffers or parameters");
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
    srv->cv_work.notify_all();
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
    if (it->second->retired) delete it->second;
    else it->second->release_pending = true;   // complete but not yet retired: its worker deletes it
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
                // every moving scene of the period in one fused update
                idx.clear();
                ab.clear();
                std::vector<std::pair<int32_t, int32_t>> spans;   // (scene, movers)
                for (auto &kv : by_scene) {
                    for (const Mover *m : kv.second) {   // constant velocity (Environment::updateEnvironment, straight lines)
                        idx.push_back(m->idx);
                        for (int c = 0; c < 6; ++c) ab.push_back(m->a0[c] + m->v[c % 3] * t);
                    }
                    spans.push_back({kv.first, (int32_t)kv.second.size()});
                }
                {
                    std::lock_guard<std::mutex> lk(srv->ctx->mu);
                    std::vector<SceneUpd> ups;
                    size_t off = 0;
                    int rc = RPM_OK;
                    for (const auto &sp : spans) {
                        SceneRec *s = find_scene(srv->ctx, sp.first);
                        if (!s) { rc = RPM_ERR_INVALID; break; }
                        ups.push_back(SceneUpd{s, idx.data() + off, ab.data() + 6 * off, sp.second});
                        off += (size_t)sp.second;
                    }
                    if (!rc) rc = scene_update_many(srv->ctx, ups);
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
    }
    {   // the batch traces: wait until every request's slot has been retired
        std::unique_lock<std::mutex> lk(srv->mu);
        srv->cv_done.wait_for(lk, std::chrono::seconds(60), [&] {
            for (int64_t i = 0; i < n; ++i) {
                if (!tickets[i]) continue;
                auto it = srv->reqs.find(tickets[i]);
                if (it != srv->reqs.end() && !it->second->retired) return false;
            }
            return true;
        });
    }
    for (int64_t i = 0; i < n; ++i) {
        if (!tickets[i]) continue;
        rpm_request_timing t{};
        rpm_server_poll(srv, tickets[i], &t);
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
    if (pending) *pending = (int64_t)(srv->incoming.size() + srv->express.size() + srv->bulk.size());
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
    if (srv->bulk_worker.joinable()) srv->bulk_worker.join();
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
            if (!sl.express && srv->bulk_part.g) srv->bulk_part.stream_destroy((CUstream)sl.st);
            else cudaStreamDestroy(sl.st);
            cudaEventDestroy(sl.done);
            for (cudaEvent_t e : sl.trace) cudaEventDestroy(e);
        }
    }
    if (srv->bulk_part.g) srv->bulk_part.destroy(srv->bulk_part.g);
    cudaFree(srv->arena_mem);
    for (Slot &sl : srv->slots)   // released by their callers, never retired
        for (Req *q : sl.reqs)
            if (q->release_pending) delete q;
    for (auto &kv : srv->reqs) delete kv.second;
    delete srv;
    return RPM_OK;
}

}  // extern "C"
