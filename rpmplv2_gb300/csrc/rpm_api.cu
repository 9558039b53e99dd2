// rpm_api.cu -- the C ABI declared in include/rpm_gpu.h.
//
// Ownership: the context owns device robots (DevRobot), scenes (a small ring
// of versioned obstacle buffers per scene) and per-stream scratch (FP32 ->
// FP64 recheck list, counters, device status word).  Callers own every
// q / output pointer they pass.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rpm_ctx_impl.cuh"
#include "rpm_nearest.cuh"
#include "rpm_spine.cuh"

using namespace rpm;

namespace rpm {
namespace impl {

thread_local std::string g_err;

int set_device(rpm_ctx *ctx) {
    CK(cudaSetDevice(ctx->device));
    return RPM_OK;
}

cudaEvent_t get_event(rpm_ctx *ctx) {
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
}

// Drop completed user events of a buffer back into the pool.
void prune_users(rpm_ctx *ctx, SceneBuf &b) {
    std::vector<cudaEvent_t> keep;
    for (cudaEvent_t e : b.users) {
        if (cudaEventQuery(e) == cudaSuccess) ctx->event_pool.push_back(e);
        else keep.push_back(e);
    }
    b.users.swap(keep);
}

void stream_wait_users(rpm_ctx *ctx, SceneBuf &b, cudaStream_t st) {
    for (cudaEvent_t e : b.users) {
        // the wait binds to the event's current record, so the event can be reused at once
        cudaStreamWaitEvent(st, e, 0);
        ctx->event_pool.push_back(e);
    }
    b.users.clear();
}

int scene_dofs(rpm_ctx *ctx, int scene_id) {
    std::lock_guard<std::mutex> lk(ctx->dof_mu);
    auto it = ctx->scene_dofs.find(scene_id);
    return it == ctx->scene_dofs.end() ? -1 : it->second;
}

void wait_users(rpm_ctx *ctx, SceneBuf &b) {
    for (cudaEvent_t e : b.users) {
        cudaEventSynchronize(e);
        ctx->event_pool.push_back(e);
    }
    b.users.clear();
}

// Top-down median split of the obstacles in 'idx' (by centre, along the
// longest axis of their centres), left parts a multiple of kLeaf, appended to
// 'out' in depth-first order: every run of kLeaf consecutive entries is a
// compact leaf, and consecutive leaves are spatial neighbours.
static void kd_order(const SceneRec &s, std::vector<int> idx, std::vector<int> &out) {
    if ((int)idx.size() <= kLeaf) {
        out.insert(out.end(), idx.begin(), idx.end());
        return;
    }
    auto centre = [&](int j, int k) {
        const float c = 0.5f * (s.aabb[6 * (size_t)j + k] + s.aabb[6 * (size_t)j + 3 + k]);
        return std::isfinite(c) ? c : 0.f;
    };
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) lo[k] = hi[k] = centre(idx[0], k);
    for (int j : idx)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], centre(j, k));
            hi[k] = std::max(hi[k], centre(j, k));
        }
    int ax = 0;
    for (int k = 1; k < 3; ++k)
        if (hi[k] - lo[k] > hi[ax] - lo[ax]) ax = k;
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return centre(a, ax) < centre(b, ax); });
    const int n = (int)idx.size();
    int h = std::max(kLeaf, (int)std::lround((double)n / 2 / kLeaf) * kLeaf);
    h = std::min(h, n - 1);
    kd_order(s, std::vector<int>(idx.begin(), idx.begin() + h), out);
    kd_order(s, std::vector<int>(idx.begin() + h, idx.end()), out);
}

void sorted_layout(SceneRec &s) {
    // static, moving and ground obstacles in separate leaves, so moving ones
    // never widen a static leaf and ground leaves can be skipped whole
    std::vector<int> group[3];
    for (int j = 0; j < s.n; ++j)
        group[(s.flags[j] & RPM_OBS_GROUND) ? 2 : ((s.flags[j] & RPM_OBS_DYNAMIC) ? 1 : 0)].push_back(j);
    s.perm.clear();
    for (int g = 0; g < 3; ++g) {
        std::vector<int> ord;
        if (!group[g].empty()) kd_order(s, group[g], ord);
        for (int j : ord) s.perm.push_back(j);
        while (s.perm.size() % kLeaf) s.perm.push_back(-1);
    }
    if (s.perm.empty()) s.perm.assign(kLeaf, -1);
    s.ns = (int)s.perm.size();
    s.nb = s.ns / kLeaf;
}

size_t scene_bytes(const SceneRec &s) {
    const size_t np = (size_t)s.n_pad, ns = (size_t)s.ns;
    return kFRows * np * sizeof(float) + kDRows * np * sizeof(double) + 8 * ns * sizeof(float) +
           7 * ns * sizeof(double) + (size_t)s.nb * kBlkRec * sizeof(float) + ns * sizeof(int32_t);
}

void bind_scene_buf(const SceneRec &s, SceneBuf &b) {
    const size_t np = (size_t)s.n_pad, ns = (size_t)s.ns;
    char *p = reinterpret_cast<char *>(b.mem);
    b.f = reinterpret_cast<float *>(p);
    p += kFRows * np * sizeof(float);
    b.d = reinterpret_cast<double *>(p);
    p += kDRows * np * sizeof(double);
    b.sf = reinterpret_cast<float *>(p);
    p += 8 * ns * sizeof(float);
    b.sd = reinterpret_cast<double *>(p);
    p += 7 * ns * sizeof(double);
    b.blk = reinterpret_cast<float *>(p);
    p += (size_t)s.nb * kBlkRec * sizeof(float);
    b.perm = reinterpret_cast<int32_t *>(p);
}

// Gather the sorted copy of a version from its rows and bound each leaf of
// kLeaf slots (four leaves per warp).  Padding slots get bounds +inf / -inf so
// no gap test passes them; a leaf holding a NaN coordinate gets infinite
// bounds so it is never skipped.
__device__ __forceinline__ void sort_slots(const float *f, const double *d, int n_pad, const int32_t *perm, int ns,
                                           float *sf, double *sd, float *blk, int s) {
    const bool in = s < ns;
    const int j = in ? perm[s] : -1;
    const float inf = __int_as_float(0x7f800000);
    float lo[3], hi[3], tmax = -inf, tmin = inf;
    bool nan = false;
    uint32_t id = kPadIdx;
    if (j >= 0) {
        for (int c = 0; c < kDRows; ++c) {
            sf[c * ns + s] = f[c * n_pad + j];
            sd[c * ns + s] = d[c * n_pad + j];
        }
        for (int c = 0; c < 3; ++c) {
            lo[c] = f[c * n_pad + j];
            hi[c] = f[(3 + c) * n_pad + j];
            nan = nan || !(lo[c] == lo[c]) || !(hi[c] == hi[c]);
        }
        const float tol = f[kRowTol * n_pad + j];
        tmax = (tol == tol) ? tol : inf;
        tmin = (tol == tol) ? tol : inf;
        id = (uint32_t)j | (f[kRowGround * n_pad + j] != 0.f ? kGroundBit : 0u);
    } else {
        for (int c = 0; c < 3; ++c) {
            lo[c] = inf;
            hi[c] = -inf;
            if (in) {
                sf[c * ns + s] = inf;
                sf[(3 + c) * ns + s] = -inf;
                sd[c * ns + s] = (double)inf;
                sd[(3 + c) * ns + s] = -(double)inf;
            }
        }
        if (in) {
            sf[kRowTol * ns + s] = 0.f;
            sd[kRowTol * ns + s] = 0.0;
        }
    }
    if (in) sf[7 * ns + s] = __uint_as_float(id);
    const unsigned full = 0xffffffffu;
    // reductions within each group of kLeaf lanes
#pragma unroll
    for (int off = kLeaf / 2; off > 0; off >>= 1) {
        for (int c = 0; c < 3; ++c) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(full, lo[c], off));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(full, hi[c], off));
        }
        tmax = fmaxf(tmax, __shfl_xor_sync(full, tmax, off));
        tmin = fminf(tmin, __shfl_xor_sync(full, tmin, off));
        nan = nan || __shfl_xor_sync(full, (int)nan, off);
    }
    const int leaf = s / kLeaf;
    if ((s % kLeaf) == 0 && in) {
        float *r = blk + (size_t)leaf * kBlkRec;
        for (int c = 0; c < 3; ++c) {
            r[c] = nan ? -inf : lo[c];
            r[3 + c] = nan ? inf : hi[c];
        }
        r[6] = (tmax == -inf) ? 0.f : tmax;   // an all-padding leaf
        r[7] = (tmin == inf) ? 0.f : tmin;
    }
}

__global__ void k_scene_sort(const float *f, const double *d, int n_pad, const int32_t *perm, int ns, float *sf,
                             double *sd, float *blk) {
    sort_slots(f, d, n_pad, perm, ns, sf, sd, blk, blockIdx.x * 32 + threadIdx.x);
}

// The fused incremental update: one CTA per scene writes its next version
// (rows and permutation copied from the current version, the updated rows
// scattered in, then the sorted copy and leaf bounds rebuilt by its warps).
// Descriptors and rows are read from pinned host memory in place.
__global__ void __launch_bounds__(256) k_scene_update_many(const UpdDesc *descs) {
    const UpdDesc u = descs[blockIdx.x];
    const int np = u.n_pad;
    for (int i = threadIdx.x; i < kFRows * np; i += blockDim.x) u.f[i] = u.src_f[i];
    for (int i = threadIdx.x; i < kDRows * np; i += blockDim.x) u.d[i] = u.src_d[i];
    for (int i = threadIdx.x; i < u.ns; i += blockDim.x) u.perm[i] = u.src_perm[i];
    __syncthreads();
    for (int k = threadIdx.x; k < u.m; k += blockDim.x) {
        const int j = __float_as_int(u.rows[7 * k]);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const float v = u.rows[7 * k + 1 + c];
            u.f[c * np + j] = v;
            u.d[c * np + j] = (double)v;
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int s0 = warp * 32; s0 < u.ns; s0 += warps * 32)
        sort_slots(u.f, u.d, np, u.perm, u.ns, u.sf, u.sd, u.blk, s0 + lane);
}

cudaError_t launch_scene_update_many(const UpdDesc *descs, int count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    k_scene_update_many<<<count, 256, 0, st>>>(descs);
    return cudaGetLastError();
}

cudaError_t launch_scene_sort(const SceneRec &s, const SceneBuf &b, cudaStream_t st) {
    k_scene_sort<<<(s.ns + 31) / 32, 32, 0, st>>>(b.f, b.d, s.n_pad, b.perm, s.ns, b.sf, b.sd, b.blk);
    return cudaGetLastError();
}

int upload_scene(rpm_ctx *ctx, SceneRec &s, SceneBuf &b) {
    const int np = s.n_pad;
    if (!b.mem) {
        const size_t bytes = scene_bytes(s);
        if (cudaMalloc(&b.mem, bytes) != cudaSuccess) return fail(RPM_ERR_NOMEM, "scene allocation of %zu bytes failed", bytes);
        bind_scene_buf(s, b);
    }
    std::vector<float> f((size_t)kFRows * np, 0.f);
    std::vector<double> d((size_t)kDRows * np, 0.0);
    for (int j = 0; j < s.n; ++j) {
        for (int k = 0; k < 6; ++k) f[(size_t)k * np + j] = s.aabb[6 * (size_t)j + k];
        f[(size_t)kRowTol * np + j] = s.tol[j];
        f[(size_t)kRowGround * np + j] = (s.flags[j] & RPM_OBS_GROUND) ? 1.f : 0.f;
        for (int k = 0; k < 7; ++k) d[(size_t)k * np + j] = (double)f[(size_t)k * np + j];
    }
    (void)ctx;
    CK(cudaMemcpy(b.f, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.d, d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(b.perm, s.perm.data(), s.perm.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(launch_scene_sort(s, b, 0));
    CK(cudaStreamSynchronize(0));
    return RPM_OK;
}

void free_scratch(Scratch *sc) {
    for (auto &g : sc->graphs) cudaGraphExecDestroy(g.exec);
    cudaFree(sc->n_e); cudaFree(sc->local); cudaFree(sc->kmax); cudaFree(sc->bprefix); cudaFree(sc->full);
    cudaFree(sc->work); cudaFree(sc->erecheck); cudaFree(sc->recheck); cudaFree(sc->counters); cudaFree(sc->status);
    cudaFree(sc->pairs); cudaFree(sc->pcfgs); cudaFree(sc->pskel); cudaFree(sc->pacc);
    cudaFree(sc->pkey); cudaFree(sc->porder); cudaFree(sc->phist);
    cudaFree(sc->perm); cudaFree(sc->bins); cudaFree(sc->aux);
    for (int i = 0; i < 3; ++i) if (sc->ev[i]) cudaEventDestroy(sc->ev[i]);
    delete sc;
}

int get_scratch(rpm_ctx *ctx, cudaStream_t st, int64_t need, Scratch **out) {
    Scratch *s = ctx->scratch[st];
    if (!s) {
        s = new Scratch();
        ctx->scratch[st] = s;
        if (cudaMalloc(&s->counters, 64) != cudaSuccess || cudaMalloc(&s->status, 64) != cudaSuccess)
            return fail(RPM_ERR_NOMEM, "scratch allocation failed");
        CK(cudaMemset(s->counters, 0, 64));
        CK(cudaMemset(s->status, 0, 64));
    }
    if ((int64_t)s->cap < need) {
        if (s->recheck) {
            CK(cudaStreamSynchronize(st));
            // cached edge graphs hold the old lists' addresses: capture them again
            for (auto &g : s->graphs) cudaGraphExecDestroy(g.exec);
            s->graphs.clear();
            cudaFree(s->recheck);
            cudaFree(s->pairs); cudaFree(s->pcfgs); cudaFree(s->pskel); cudaFree(s->pacc); cudaFree(s->perm);
            cudaFree(s->pkey); cudaFree(s->porder);
            s->recheck = nullptr;
            s->perm = nullptr;
            s->pkey = s->porder = nullptr;
        }
        const size_t cap = std::max<size_t>((size_t)need, 1u << 16);
        // records for 1/8 of the configurations (at least 4096, at most 65536),
        // 16 listed pairs per record; what does not fit is rechecked whole
        const size_t pcfg = std::min<size_t>(cap, std::max<size_t>(4096, std::min<size_t>(cap / 8, 1u << 16)));
        const size_t ppair = 16 * pcfg;
        if (cudaMalloc(&s->recheck, 2 * cap * sizeof(uint64_t)) != cudaSuccess ||   // two launches per configuration
            cudaMalloc(&s->pairs, ppair * sizeof(uint64_t)) != cudaSuccess ||
            cudaMalloc(&s->pkey, ppair * sizeof(uint32_t)) != cudaSuccess ||
            cudaMalloc(&s->porder, ppair * sizeof(uint32_t)) != cudaSuccess ||
            (!s->phist && cudaMalloc(&s->phist, kPairHist * sizeof(uint32_t)) != cudaSuccess) ||
            cudaMalloc(&s->pcfgs, pcfg * sizeof(PairCfg)) != cudaSuccess ||
            cudaMalloc(&s->pskel, pcfg * (kMaxDof + 1) * 3 * sizeof(double)) != cudaSuccess ||
            cudaMalloc(&s->pacc, pcfg * sizeof(PairAcc)) != cudaSuccess ||
            cudaMalloc(&s->perm, cap * sizeof(int32_t)) != cudaSuccess ||
            (!s->bins && cudaMalloc(&s->bins, 2 * kConfigBins * sizeof(int32_t)) != cudaSuccess))
            return fail(RPM_ERR_NOMEM, "recheck list allocation failed");
        s->cap = cap;
        s->perm_cap = cap;
        s->pcfg_cap = pcfg;
        s->ppair_cap = ppair;
    }
    *out = s;
    return RPM_OK;
}

// The stream's planner working memory, at least `bytes`, reused in stream
// order: no allocation on a call's path once it is large enough.  It grows
// in stream order too (the old block is freed after the work already queued
// on the stream, the new one is ready for the work queued next), at least
// doubling, so a serving stream neither waits nor synchronises the device.
int get_aux(rpm_ctx *ctx, cudaStream_t st, size_t bytes, void **out) {
    Scratch *s = nullptr;
    int rc = get_scratch(ctx, st, 0, &s);
    if (rc) return rc;
    if (s->aux_cap < bytes) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(st, &cs));
        if (cs != cudaStreamCaptureStatusNone)
            return fail(RPM_ERR_INVALID, "the stream's planner scratch cannot grow during stream capture");
        const size_t cap = std::max<size_t>({bytes, 2 * s->aux_cap, (size_t)4 << 20});
        if (s->aux) {
            CK(cudaFreeAsync(s->aux, st));
            s->aux = nullptr;
            s->aux_cap = 0;
        }
        if (cudaMallocAsync(&s->aux, cap, st) != cudaSuccess) {
            cudaGetLastError();
            return fail(RPM_ERR_NOMEM, "planner scratch allocation failed");
        }
        s->aux_cap = cap;
    }
    *out = s->aux;
    return RPM_OK;
}

}  // namespace impl

using impl::fail;

int set_error(int code, const char *msg) { return fail(code, "%s", msg); }
int build_dev_robot(const rpm_robot_desc &d, DevRobot &r) {
    if (d.kind != RPM_ROBOT_CHAIN && d.kind != RPM_ROBOT_XARM6 && d.kind != RPM_ROBOT_SPATIAL) return fail(RPM_ERR_INVALID, "unknown robot kind %d", d.kind);
    if (d.num_dofs < 1 || d.num_dofs > RPM_MAX_DOF) return fail(RPM_ERR_INVALID, "num_dofs %d out of range", d.num_dofs);
    if (d.kind == RPM_ROBOT_XARM6 && d.num_dofs != 6) return fail(RPM_ERR_INVALID, "xArm6 needs num_dofs == 6");
    std::memset(&r, 0, sizeof r);
    r.kind = d.kind;
    r.D = d.num_dofs;
    r.ground_included = d.ground_included;
    for (int k = 0; k < d.num_dofs; ++k) {
        if (d.joint_axis[k] < 0 || d.joint_axis[k] > 2) return fail(RPM_ERR_INVALID, "joint %d axis must be 0, 1 or 2", k);
        const float rad = d.capsule_radius[k];
        if (!(rad >= 0.f) || !std::isfinite(rad)) return fail(RPM_ERR_INVALID, "capsule radius %d invalid", k);
        r.axis[k] = d.joint_axis[k];
        r.radius_f[k] = rad;
        r.radius_d[k] = (double)rad;
        r.rnew_d[k] = (double)rad * std::sqrt(3.0) / 3;
        r.rnew_f[k] = (float)r.rnew_d[k];
    }
    for (int k = 0; k <= d.num_dofs; ++k) {
        bool ident = true;
        for (int i = 0; i < 9; ++i) {
            double v = d.origin_rot[k][i];
            if (v != ((i % 4 == 0) ? 1.0 : 0.0)) ident = false;
            r.orot[k][i] = v;
            r.orot_f[k][i] = (float)v;
        }
        if (ident && k < 32) r.rot_identity_mask |= (1 << k);
        for (int i = 0; i < 3; ++i) {
            r.oxyz[k][i] = d.origin_xyz[k][i];
            r.oxyz_f[k][i] = (float)d.origin_xyz[k][i];
        }
    }
    r.gripper_d = (double)d.gripper_length;
    r.gripper_f = d.gripper_length;
    r.grip03_f = (float)(0.3 * (double)d.gripper_length);
    return RPM_OK;
}
}  // namespace rpm

namespace rpm {
namespace impl {

SceneRec *find_scene(rpm_ctx *ctx, int id) {
    auto it = ctx->scenes.find(id);
    return it == ctx->scenes.end() ? nullptr : it->second;
}

// Layout of one segment.  Lane-per-configuration walks a scene's obstacles in
// series per lane, which suits small scenes and large batches; warp-per-
// configuration culls whole leaves of the sorted copy and spreads the
// survivors over a warp, which suits large scenes and batches too small to
// fill the GPU with lanes.  Per-link distance profiles of large batches stay
// lane-per-configuration: every link needs its own nearest-first search
// there, which keeps the warp's drains half empty.  (Thresholds measured on
// GB300 over 10-22 links, 10-1000 obstacles and 256-65,536 configurations.)
constexpr int kDefaultEdgeCtas = 4;   // lane-layout edge pass, without a table entry

static int ceil_log2(int64_t x) {
    int l = 0;
    while (l < 62 && ((int64_t)1 << l) < x) ++l;
    return l;
}

static TuneKey tune_key(const rpm_ctx *ctx, const SceneRec *s, int64_t count, int prec, int outputs, int edges) {
    const rpm_robot_desc &d = ctx->robots[s->robot].desc;
    return TuneKey{d.kind, d.num_dofs, ceil_log2((int64_t)s->n + 1), ceil_log2(std::max<int64_t>(count, 1)), prec,
                   outputs, edges};
}

static const rpm_tile_shape *tuned(const rpm_ctx *ctx, const TuneKey &k) {
    if (ctx->layout != RPM_LAYOUT_AUTO) return nullptr;
    auto it = ctx->tune.find(k);
    return it == ctx->tune.end() ? nullptr : &it->second;
}

static int outputs_of(const SegReq &r) {
    return (r.valid ? RPM_OUT_VALID : 0) | (r.dist ? RPM_OUT_DIST : 0) | (r.profile ? RPM_OUT_PROFILE : 0);
}

// 'single': the request is the whole batch, so a lane-layout launch checks it
// in binned order (kBinMinConfigs and up).
static bool use_warp_layout(const rpm_ctx *ctx, const SegReq &r, int64_t total, int prec, bool single) {
    if (r.wide >= 0) return r.wide == 1;
    if (ctx->layout == RPM_LAYOUT_LANE) return false;
    if (ctx->layout == RPM_LAYOUT_WARP) return true;
    if (const rpm_tile_shape *t = tuned(ctx, tune_key(ctx, r.scene, total, prec, outputs_of(r), 0)))
        if (t->layout == RPM_LAYOUT_LANE || t->layout == RPM_LAYOUT_WARP) return t->layout == RPM_LAYOUT_WARP;
    const int n = r.scene->n;
    // binned and culled, the lane layout wins from 32,768 configurations for every
    // scene size measured (10-1000 obstacles; xarm6, spatial 10- and 22-DOF)
    if (prec == RPM_PREC_FP32_RECHECK && r.profile == nullptr && single && total >= kLaneBinnedBatch) return false;
    if (n >= kWideMinObstacles) return !(r.profile != nullptr && total > kWideMaxProfileBatch);
    if (prec == RPM_PREC_FP32_RECHECK && r.profile == nullptr && n >= 20) {
        if (n >= 80) return total <= kWide32Batch80;
        if (n >= 40) return total <= kWide32Batch40;
        return total <= kWide32Batch20;
    }
    if (n >= kWideMidObstacles) return total <= kWideMidBatch;
    const int64_t small = (prec == RPM_PREC_FP64) ? kWideSmallBatch : kWideSmallBatch32;
    return n >= kWideSmallObstacles && r.profile == nullptr && total <= small;
}

// Queue checks of up to kMaxSegs segments as one launch on 'st' (more
// segments, or segments of both layouts, become several launches).  The
// caller holds ctx->mu.
int enqueue_segments(rpm_ctx *ctx, int prec, const std::vector<SegReq> &reqs_in, cudaStream_t st) {
    int64_t total = 0;
    for (const SegReq &r : reqs_in) total += r.count;
    // In the FP32+recheck form a lane-layout segment that wants isValid and a
    // distance runs as two segments of the same launch, one per tree: a warp
    // then keeps to one of the two decision trees (measured 7.1 -> 6.0 ms per
    // 1M xarm6 configurations).  Each output is the reference's own function
    // of the configuration, so the outputs are the same.  The exact forms keep
    // one segment: their FP64 forward kinematics would run twice.
    std::vector<SegReq> reqs;
    reqs.reserve(2 * reqs_in.size());
    for (const SegReq &r : reqs_in) {
        const int wide = use_warp_layout(ctx, r, total, prec, reqs_in.size() == 1) ? 1 : 0;   // decided once per request
        if (prec == RPM_PREC_FP32_RECHECK && r.valid && (r.dist || r.profile) && !wide) {
            reqs.push_back(SegReq{r.scene, r.q, r.count, r.valid, nullptr, nullptr, 0});
            reqs.push_back(SegReq{r.scene, r.q, r.count, nullptr, r.dist, r.profile, 0});
        } else {
            SegReq c = r;
            c.wide = wide;
            reqs.push_back(c);
        }
    }
    Scratch *sc = nullptr;
    int rc = get_scratch(ctx, st, prec == RPM_PREC_FP32_RECHECK ? total : 0, &sc);
    if (rc) return rc;
    sc->last_configs = total;
    CK(cudaMemsetAsync(sc->counters, 0, 4 * sizeof(uint32_t), st));
    // Every FP32 lane-layout request of at least kBinMinConfigs configurations is
    // checked in binned order (launch_bin_configs), each with its own slice of the
    // order; the isValid and distance launches of a request share its slice.  The
    // order lives with the recheck lists, sized for the stream's largest batch
    // (get_scratch above), so a steady stream of requests allocates nothing.
    if (prec == RPM_PREC_FP32_RECHECK && sc->bins) {
        size_t used_perm = 0;
        for (size_t k = 0; k < reqs.size(); ++k) {
            SegReq &r = reqs[k];
            if (r.wide != 0 || r.count < kBinMinConfigs || r.count > INT32_MAX) continue;
            if (k > 0 && reqs[k - 1].perm && reqs[k - 1].q == r.q && reqs[k - 1].count == r.count &&
                reqs[k - 1].scene == r.scene) {
                r.perm = reqs[k - 1].perm;   // the other output of the same request
                continue;
            }
            if (used_perm + (size_t)r.count > sc->perm_cap) break;
            int32_t *slice = sc->perm + used_perm;
            CK(launch_bin_configs(r.q, r.count, ctx->robots[r.scene->robot].desc.num_dofs, sc->bins, slice, st));
            r.perm = slice;
            used_perm += (size_t)r.count;
        }
    }
    sc->timed = ctx->timing && total > 0;
    sc->had_recheck = prec == RPM_PREC_FP32_RECHECK;
    if (sc->timed && !sc->ev[0])
        for (int i = 0; i < 3; ++i) CK(cudaEventCreate(&sc->ev[i]));
    if (sc->timed) CK(cudaEventRecord(sc->ev[0], st));
    // chunks of at most kMaxSegs segments of one layout and, in the lane layout,
    // of one output kind (isValid only, distance only, distance with profile,
    // several), so a launch runs the kernel body compiled for its outputs
    auto kind_of = [](const SegReq &r) {
        if (!r.dist && !r.profile) return 1;
        if (r.valid) return 0;
        return r.profile ? 2 : 3;
    };
    std::vector<std::pair<bool, std::vector<const SegReq *>>> chunks;
    for (int wide = 0; wide < 2; ++wide) {
        for (int kind = 0; kind < 4; ++kind) {
            if (wide && kind > 0) break;   // the warp layout takes every kind in one launch
            std::vector<const SegReq *> cur;
            for (const SegReq &r : reqs) {
                if (r.count <= 0 || use_warp_layout(ctx, r, total, prec, reqs_in.size() == 1) != (wide == 1)) continue;
                if (!wide && kind_of(r) != kind) continue;
                cur.push_back(&r);
                if ((int)cur.size() == kMaxSegs) { chunks.push_back({wide == 1, cur}); cur.clear(); }
            }
            if (!cur.empty()) chunks.push_back({wide == 1, cur});
        }
    }
    const size_t tsz = prec == RPM_PREC_FP64 ? sizeof(double) : sizeof(float);
    std::vector<SceneBuf *> used;
    // FP32 + recheck: the FP64 recheck of a group of launches (as many as fit
    // kMaxSegs segments together) runs once, after the group's last launch.
    // Their records carry the segment's index in the group (PairSink::seg_base),
    // so the isValid and distance launches of a request share one round of the
    // latency-bound recheck instead of two.  Each configuration is listed once
    // per launch it is in: the whole-configuration list holds twice the
    // configurations (get_scratch).
    const bool recheck = prec == RPM_PREC_FP32_RECHECK;
    KParams group, last_p;
    int32_t group_segs = 0;
    auto flush_group = [&]() -> int {
        if (group_segs == 0) return RPM_OK;
        KParams rp = last_p;
        std::memcpy(rp.segs, group.segs, sizeof(Seg) * (size_t)group_segs);
        rp.nseg = group_segs;
        rp.ps.seg_base = 0;
        group_segs = 0;
        CK(launch_pair_recheck(rp, ctx->num_sms * 2, st));
        CK(launch_recheck(rp, ctx->num_sms * 4, st));
        return RPM_OK;
    };
    for (size_t ci = 0; ci < chunks.size(); ++ci) {
        const bool wide = chunks[ci].first;
        const std::vector<const SegReq *> &segs = chunks[ci].second;
        const bool last = ci + 1 == chunks.size();
        KParams p;
        std::memset(&p, 0, sizeof p);
        int64_t chunk_total = 0;
        int gmax = 32;
        for (const SegReq *r : segs) {
            chunk_total += r->count;
            const int D = ctx->robots[r->scene->robot].desc.num_dofs;
            gmax = std::min(gmax, kWidePtsBytes / ((D + 1) * 3 * (int)tsz));
            p.skel_pts = std::max(p.skel_pts, D + 1);
        }
        // configurations per warp: enough warps for two waves of two CTAs per SM,
        // unless the tile-shape table holds a count for every segment's bucket
        // (at least 2 from 2,048 configurations: the autotuner chose 2 for every
        // 4,096-configuration bucket it tuned in the warp layout)
        int64_t want = (chunk_total + (int64_t)ctx->num_sms * 32 - 1) / ((int64_t)ctx->num_sms * 32);
        if (chunk_total >= 2048) want = std::max<int64_t>(want, 2);
        p.wide_g = (int32_t)std::max<int64_t>(1, std::min<int64_t>(gmax, want));
        if (wide) {
            int tg = 0;
            for (const SegReq *r : segs) {
                const rpm_tile_shape *t = tuned(ctx, tune_key(ctx, r->scene, total, prec, outputs_of(*r), 0));
                if (!t || t->configs_per_warp <= 0) { tg = 0; break; }
                tg = tg ? std::min(tg, t->configs_per_warp) : t->configs_per_warp;
            }
            if (tg > 0) p.wide_g = std::max(1, std::min(gmax, tg));
        }
        sc->last_shape = rpm_tile_shape{wide ? RPM_LAYOUT_WARP : RPM_LAYOUT_LANE, wide ? p.wide_g : 0, 0, 0.f};
        const int64_t per_cta = wide ? (int64_t)kWideWarps * p.wide_g : kThreads;
        int64_t blocks = 0;
        size_t smem = 0;
        for (const SegReq *rp : segs) {
            const SegReq &r = *rp;
            SceneBuf &buf = r.scene->bufs[r.scene->cur];
            if (buf.pending) {   // an incremental update still writing this version
                if (cudaEventQuery(buf.ready) == cudaSuccess) buf.pending = false;
                else CK(cudaStreamWaitEvent(st, buf.ready, 0));
            }
            used.push_back(&buf);
            Seg &g = p.segs[p.nseg++];
            g.robot = ctx->robots[r.scene->robot].dev;
            g.obs_f = buf.f;
            g.obs_d = buf.d;
            g.q = r.q;
            g.valid = r.valid;
            g.dist = r.dist;
            g.profile = r.profile;
            g.count = r.count;
            g.first_block = blocks;
            g.n = r.scene->n;
            g.n_pad = r.scene->n_pad;
            g.srt_f = buf.sf;
            g.srt_d = buf.sd;
            g.blk = buf.blk;
            g.ns = r.scene->ns;
            g.nb = r.scene->nb;
            g.perm = wide ? nullptr : r.perm;
            blocks += (r.count + per_cta - 1) / per_cta;
            smem = std::max(smem, wide ? wide_smem_bytes(prec, r.scene->ns, r.scene->nb)
                                       : smem_bytes(prec == RPM_PREC_FP32_RECHECK ? RPM_PREC_FP32_REF : prec, r.scene->n_pad));
        }
        p.nmd.eq = ctx->params.equality_threshold;
        p.nmd.maxd = ctx->params.max_distance;
        p.nmf.eq = (float)ctx->params.equality_threshold;
        p.nmf.maxd = (float)ctx->params.max_distance;
        p.recheck = sc->recheck;
        p.recheck_count = sc->counters;
        p.status = sc->status;
        p.ps.pairs = sc->pairs;
        p.ps.pair_count = sc->counters + 3;
        p.ps.pair_cap = (uint32_t)sc->ppair_cap;
        p.ps.cfg_cap = (uint32_t)sc->pcfg_cap;
        p.ps.cfgs = sc->pcfgs;
        p.ps.cfg_count = sc->counters + 2;
        p.ps.skel = sc->pskel;
        p.ps.acc = sc->pacc;
        if (total >= kSortPairsMinConfigs) {   // small batches list few pairs: list order, two launches fewer
            p.ps.key = sc->pkey;
            p.ps.order = sc->porder;
            p.ps.hist = sc->phist;
        }
        if (recheck) {
            if (group_segs + p.nseg > kMaxSegs) {   // the group is full: its recheck, then fresh lists
                rc = flush_group();
                if (rc) return rc;
                CK(cudaMemsetAsync(sc->counters, 0, 4 * sizeof(uint32_t), st));
            }
            p.ps.seg_base = group_segs;
            std::memcpy(group.segs + group_segs, p.segs, sizeof(Seg) * (size_t)p.nseg);
            group_segs += p.nseg;
        } else if (ci > 0) {
            CK(cudaMemsetAsync(sc->counters, 0, 4 * sizeof(uint32_t), st));
        }
        if (wide) CK(launch_check_wide(prec, p, blocks, smem, st));
        else if (recheck) CK(launch_check_fp32(p, blocks, smem, st));
        else CK(launch_check_exact(prec, p, blocks, smem, st));
        if (sc->timed && last) CK(cudaEventRecord(sc->ev[1], st));
        if (recheck) last_p = p;
    }
    if (recheck) {
        rc = flush_group();
        if (rc) return rc;
    }
    if (sc->timed) {
        if (chunks.empty()) CK(cudaEventRecord(sc->ev[1], st));
        CK(cudaEventRecord(sc->ev[2], st));
    }
    for (SceneBuf *b : used) {
        prune_users(ctx, *b);
        cudaEvent_t e = get_event(ctx);
        CK(cudaEventRecord(e, st));
        b->users.push_back(e);
    }
    return RPM_OK;
}

// Layout of an edge batch: the checks of one edge are neighbours in space,
// so the lane-per-check warps of the lane layout already share most of their
// obstacle walk; the warp layout pays off once culling whole leaves beats
// walking every obstacle.
// Shape of an edge request in a batch of 'total' edges: the layout from the
// tile-shape table or the obstacle-count rule, and the table's counts.
static rpm_tile_shape edge_shape(const rpm_ctx *ctx, const SceneRec *s, int64_t total, int prec) {
    rpm_tile_shape sh{0, 0, 0, 0.f};
    if (ctx->layout == RPM_LAYOUT_LANE || ctx->layout == RPM_LAYOUT_WARP) {
        sh.layout = ctx->layout;
        return sh;
    }
    if (const rpm_tile_shape *t = tuned(ctx, tune_key(ctx, s, total, prec, RPM_OUT_VALID, 1))) sh = *t;
    if (sh.layout != RPM_LAYOUT_LANE && sh.layout != RPM_LAYOUT_WARP) {
        // the FP32 lane pass culls obstacles per warp (a warp's checks are neighbours on
        // one or a few edges), which beats the warp pass except on very large scenes and batches
        const bool wide = prec == RPM_PREC_FP32_RECHECK
                              ? (s->n >= kWideEdgeObstacles32 && total > kWideEdgeBatch32)
                              : s->n >= kWideEdgeObstacles;
        sh.layout = wide ? RPM_LAYOUT_WARP : RPM_LAYOUT_LANE;
    }
    return sh;
}

int edge_scratch(rpm_ctx *ctx, Scratch *sc, int64_t E, cudaStream_t st) {
    if ((int64_t)sc->ecap >= E && sc->work) return RPM_OK;
    CK(cudaStreamSynchronize(st));
    for (auto &g : sc->graphs) cudaGraphExecDestroy(g.exec);
    sc->graphs.clear();
    cudaFree(sc->n_e); cudaFree(sc->local); cudaFree(sc->kmax); cudaFree(sc->bprefix); cudaFree(sc->full);
    cudaFree(sc->work); cudaFree(sc->erecheck);
    const size_t cap = std::max<size_t>((size_t)E, 1u << 12);
    const size_t nb = cap / kEdgeScanBlock + 2;
    sc->erecheck_cap = 4 * cap + (1u << 16);
    if (cudaMalloc(&sc->n_e, cap * 4) || cudaMalloc(&sc->local, cap * 4) || cudaMalloc(&sc->kmax, cap * 4) ||
        cudaMalloc(&sc->bprefix, nb * 8) || cudaMalloc(&sc->full, cap) || cudaMalloc(&sc->work, 64) ||
        cudaMalloc(&sc->erecheck, sc->erecheck_cap * 8))
        return fail(RPM_ERR_NOMEM, "edge scratch allocation failed");
    sc->ecap = cap;
    (void)ctx;
    return RPM_OK;
}

// Queue the edge pipeline (counts + scan, the lane- and warp-layout passes,
// recheck, final) for a batch of edge requests, kMaxSegs requests per launch.
// The scratch must hold the batch's edges (edge_scratch).
int enqueue_edge_batch(rpm_ctx *ctx, Scratch *sc, int prec, const std::vector<EdgeReq> &reqs, int ctas_per_sm,
                       cudaStream_t st) {
    int64_t batch_total = 0;
    for (const EdgeReq &r : reqs) batch_total += r.E;
    std::vector<rpm_tile_shape> shape(reqs.size());
    for (size_t k = 0; k < reqs.size(); ++k) shape[k] = edge_shape(ctx, reqs[k].scene, batch_total, prec);
    auto is_wide = [&](const EdgeReq *r) { return shape[(size_t)(r - reqs.data())].layout == RPM_LAYOUT_WARP; };
    std::vector<const EdgeReq *> order;   // lane-layout requests first
    for (int wide = 0; wide < 2; ++wide)
        for (const EdgeReq &r : reqs)
            if (r.E > 0 && is_wide(&r) == (wide == 1)) order.push_back(&r);
    const size_t tsz = prec == RPM_PREC_FP64 ? sizeof(double) : sizeof(float);
    for (size_t first = 0; first < order.size(); first += kMaxSegs) {
        const size_t last = std::min(order.size(), first + (size_t)kMaxSegs);
        EdgeParams p;
        std::memset(&p, 0, sizeof p);
        int64_t E = 0, E_wide = 0;
        int gmax = 32;
        for (size_t i = first; i < last; ++i) {
            const EdgeReq &r = *order[i];
            SceneRec *s = r.scene;
            SceneBuf &buf = s->bufs[s->cur];
            if (buf.pending) {   // an incremental update still writing this version
                if (cudaEventQuery(buf.ready) == cudaSuccess) buf.pending = false;
                else CK(cudaStreamWaitEvent(st, buf.ready, 0));
            }
            const bool wide = is_wide(&r);
            EdgeSeg &es = p.segs[p.nseg];
            if (!wide) p.nseg_lane = p.nseg + 1;
            p.nseg++;
            const int D = ctx->robots[s->robot].desc.num_dofs;
            es.seg.robot = ctx->robots[s->robot].dev;
            es.seg.obs_f = buf.f;
            es.seg.obs_d = buf.d;
            es.seg.n = s->n;
            es.seg.n_pad = s->n_pad;
            es.seg.srt_f = buf.sf;
            es.seg.srt_d = buf.sd;
            es.seg.blk = buf.blk;
            es.seg.ns = s->ns;
            es.seg.nb = s->nb;
            es.seg.q = r.q1;
            es.seg.count = r.E;
            es.seg.valid = r.valid;
            es.q2 = r.q2;
            es.checks_out = r.checks;
            es.e0 = E;
            es.step = r.step;
            es.num_checks = r.num_checks;
            es.D = D;
            E += r.E;
            if (wide) {
                E_wide += r.E;
                gmax = std::min(gmax, kWidePtsBytes / ((D + 1) * 3 * (int)tsz));
            }
        }
        if ((int64_t)sc->ecap < E) return fail(RPM_ERR_INVALID, "edge scratch below the batch's %lld edges", (long long)E);
        p.E = E;
        p.n_e = sc->n_e; p.local = sc->local; p.bprefix = sc->bprefix; p.kmax = sc->kmax; p.work = sc->work;
        p.full = sc->full;
        p.recheck = sc->erecheck;
        p.recheck_cap = (uint32_t)std::min<size_t>(sc->erecheck_cap, 0xffffffffu);
        p.recheck_count = sc->counters;
        p.overflow = sc->counters + 1;
        p.counters = sc->counters;
        p.status = sc->status;
        p.nmd.eq = ctx->params.equality_threshold; p.nmd.maxd = ctx->params.max_distance;
        p.nmf.eq = (float)ctx->params.equality_threshold; p.nmf.maxd = (float)ctx->params.max_distance;
        p.ps.pairs = sc->pairs;
        p.ps.pair_count = sc->counters + 3;
        p.ps.pair_cap = (uint32_t)sc->ppair_cap;
        p.ps.cfg_cap = (uint32_t)sc->pcfg_cap;
        p.ps.cfgs = sc->pcfgs;
        p.ps.cfg_count = sc->counters + 2;
        p.ps.skel = sc->pskel;
        p.ps.acc = sc->pacc;
        p.wide_g = std::max(1, gmax);
        // the table's counts of the launch's first request of each layout
        int lane_ctas = ctas_per_sm, wide_g = 0;
        for (size_t i = first; i < last; ++i) {
            const rpm_tile_shape &sh = shape[(size_t)(order[i] - reqs.data())];
            if (sh.layout == RPM_LAYOUT_LANE && sh.ctas_per_sm > 0 && lane_ctas == ctas_per_sm) lane_ctas = sh.ctas_per_sm;
            if (sh.layout == RPM_LAYOUT_WARP && sh.configs_per_warp > 0 && !wide_g) wide_g = sh.configs_per_warp;
        }
        if (wide_g > 0) p.wide_g = std::max(1, std::min(gmax, wide_g));
        sc->last_shape = p.nseg_lane < p.nseg ? rpm_tile_shape{RPM_LAYOUT_WARP, p.wide_g, 0, 0.f}
                                              : rpm_tile_shape{RPM_LAYOUT_LANE, 0, std::max(1, lane_ctas), 0.f};
        CK(launch_edge_prep(p, st));   // also zeroes the counters
        if (p.nseg_lane > 0) {
            const int grid = ctx->num_sms * std::max(1, lane_ctas);
            const size_t smem = p.nseg_lane == 1
                ? smem_bytes(prec == RPM_PREC_FP32_RECHECK ? RPM_PREC_FP32_REF : prec, p.segs[0].seg.n_pad) : 0;
            if (prec == RPM_PREC_FP32_RECHECK) CK(launch_edges_fp32(p, grid, smem, st));
            else CK(launch_edges(prec, p, grid, smem, st));
        }
        if (p.nseg_lane < p.nseg) {
            // persistent: as many CTAs as fit (two per SM for the FP32 forms)
            const int grid = ctx->num_sms * (prec == RPM_PREC_FP64 ? 1 : 2);
            // edge streams pay off once every stream has a couple of edges to walk
            p.streams = E_wide >= 2 * (int64_t)grid * kWideWarps * p.wide_g ? 1 : 0;
            const Seg &sg = p.segs[p.nseg_lane].seg;
            const size_t smem = p.nseg - p.nseg_lane == 1 ? wide_smem_bytes(prec, sg.ns, sg.nb)
                                                          : (size_t)kWideWarps * kWidePtsBytes;
            CK(launch_edges_wide(prec, p, grid, smem, st));
        }
        CK(launch_edge_recheck_final(p, ctx->num_sms * 4, prec == RPM_PREC_FP32_RECHECK, st));
    }
    return RPM_OK;
}

int enqueue_edges(rpm_ctx *ctx, Scratch *sc, SceneRec *s, int prec, const float *q1, const float *q2, int64_t E,
                  float step, int32_t num_checks, uint8_t *valid, int32_t *checks, int ctas_per_sm, cudaStream_t st) {
    return enqueue_edge_batch(ctx, sc, prec, {EdgeReq{s, q1, q2, E, step, num_checks, valid, checks}}, ctas_per_sm, st);
}

int enqueue_check(rpm_ctx *ctx, SceneRec *s, int prec, const float *q, int64_t C, uint8_t *valid, double *dist,
                  float *profile, cudaStream_t st) {
    return enqueue_segments(ctx, prec, {SegReq{s, q, C, valid, dist, profile}}, st);
}

}  // namespace impl
}  // namespace rpm

using namespace rpm::impl;

// Stream-ordered scratch of one call, freed on the stream however the call returns.
struct AsyncScratch {
    void *p = nullptr;
    cudaStream_t st = nullptr;
    ~AsyncScratch() {
        if (p) cudaFreeAsync(p, st);
    }
};

// Device address of a page-locked host buffer (cudaHostAlloc / cudaHostRegister,
// mapped), or null for any other pointer.
template <typename P> static P *mapped_ptr(P *host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, (const void *)host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return reinterpret_cast<P *>(a.devicePointer);
}

// The status word of a stream's scratch after its work: a bounded device-side
// wait that gave up is reported (and the word reset).
static int host_status(rpm_ctx *ctx, cudaStream_t st) {
    if (!st) return RPM_OK;
    auto it = ctx->scratch.find(st);
    if (it == ctx->scratch.end()) return RPM_OK;
    int32_t v = 0;
    CK(cudaMemcpy(&v, it->second->status, sizeof v, cudaMemcpyDeviceToHost));
    if (v) {
        cudaMemset(it->second->status, 0, sizeof(int32_t));
        return fail(RPM_ERR_TIMEOUT, "a bounded device-side wait gave up (status %d)", v);
    }
    return RPM_OK;
}

extern "C" {

const char *rpm_last_error_string(void) { return g_err.c_str(); }
int rpm_version(void) { return 1; }

int rpm_ctx_create(int device, rpm_ctx **out) {
    if (!out) return fail(RPM_ERR_INVALID, "out is NULL");
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(RPM_ERR_INVALID, "device %d not present (%d devices)", device, n);
    rpm_ctx *ctx = new rpm_ctx();
    ctx->device = device;
    CK(cudaSetDevice(device));
    CK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
    // a tile-shape table named by the environment (rpm_tuning_save's format)
    if (const char *tf = std::getenv("RPM_TUNING_FILE")) {
        if (*tf) {
            const int rc = rpm_tuning_load(ctx, tf);
            if (rc) { delete ctx; return rc; }
        }
    }
    *out = ctx;
    return RPM_OK;
}

int rpm_ctx_destroy(rpm_ctx *ctx) {
    if (!ctx) return RPM_OK;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    for (auto &kv : ctx->scenes) {
        for (auto &b : kv.second->bufs) {
            for (cudaEvent_t e : b.users) cudaEventDestroy(e);
            if (b.mem) cudaFree(b.mem);
        }
        delete kv.second;
    }
    for (auto &r : ctx->robots) cudaFree(r.dev);
    for (auto &kv : ctx->scratch) {
        free_scratch(kv.second);
    }
    for (int i = 0; i < 2; ++i) {
        if (ctx->hs[i]) cudaStreamDestroy(ctx->hs[i]);
        cudaFree(ctx->hq[i]); cudaFree(ctx->hv[i]); cudaFree(ctx->hd[i]); cudaFree(ctx->hp[i]);
    }
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    for (int i = 0; i < rpm_ctx::kUpdRing; ++i) {
        if (ctx->upd_stage[i]) cudaFreeHost(ctx->upd_stage[i]);
        if (ctx->upd_done[i]) cudaEventDestroy(ctx->upd_done[i]);
    }
    if (ctx->upd_stream) cudaStreamDestroy(ctx->upd_stream);
    delete ctx;
    return RPM_OK;
}

int rpm_ctx_set_params(rpm_ctx *ctx, const rpm_params *params) {
    if (!ctx || !params) return fail(RPM_ERR_INVALID, "NULL argument");
    if (!(params->max_distance > 0) || !(params->equality_threshold >= 0))
        return fail(RPM_ERR_INVALID, "invalid RealVectorSpaceConfig constants");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->params = *params;
    return RPM_OK;
}

int rpm_robot_upload(rpm_ctx *ctx, const rpm_robot_desc *desc, int32_t *robot_id) {
    if (!ctx || !desc || !robot_id) return fail(RPM_ERR_INVALID, "NULL argument");
    DevRobot r;
    int rc = build_dev_robot(*desc, r);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    RobotRec rec;
    rec.desc = *desc;
    if (cudaMalloc(&rec.dev, sizeof(DevRobot)) != cudaSuccess) return fail(RPM_ERR_NOMEM, "robot allocation failed");
    CK(cudaMemcpy(rec.dev, &r, sizeof r, cudaMemcpyHostToDevice));
    ctx->robots.push_back(rec);
    *robot_id = (int32_t)ctx->robots.size() - 1;
    return RPM_OK;
}

int rpm_scene_create(rpm_ctx *ctx, int32_t robot_id, const float *aabb_host, const float *min_dist_tol_host,
                     const uint8_t *flags_host, int32_t n, int32_t *scene_id) {
    if (!ctx || !scene_id || (n > 0 && !aabb_host)) return fail(RPM_ERR_INVALID, "NULL argument");
    if (n < 0) return fail(RPM_ERR_INVALID, "negative obstacle count");
    if (n > kMaxObstacles) return fail(RPM_ERR_RANGE, "%d obstacles exceed the maximum of %d per scene", n, kMaxObstacles);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (robot_id < 0 || robot_id >= (int)ctx->robots.size()) return fail(RPM_ERR_INVALID, "unknown robot %d", robot_id);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    SceneRec *s = new SceneRec();
    s->robot = robot_id;
    s->n = n;
    s->n_pad = std::max(16, (n + 15) / 16 * 16);
    s->aabb.assign(aabb_host, aabb_host + 6 * (size_t)n);
    s->tol.resize(n);
    s->flags.resize(n);
    for (int j = 0; j < n; ++j) {
        s->tol[j] = min_dist_tol_host ? min_dist_tol_host[j] : (float)ctx->params.max_distance;
        s->flags[j] = flags_host ? flags_host[j] : 0;
    }
    sorted_layout(*s);
    int rc = upload_scene(ctx, *s, s->bufs[0]);
    if (rc) { delete s; return rc; }
    s->cur = 0;
    s->version = 1;
    *scene_id = ctx->next_scene++;
    ctx->scenes[*scene_id] = s;
    {
        std::lock_guard<std::mutex> dl(ctx->dof_mu);
        ctx->scene_dofs[*scene_id] = ctx->robots[robot_id].desc.num_dofs;
    }
    return RPM_OK;
}

int rpm_scene_update(rpm_ctx *ctx, int32_t scene_id, const int32_t *idx_host, const float *aabb_host, int32_t m,
                     uint64_t *version_out) {
    if (!ctx || m < 0 || (m > 0 && (!idx_host || !aabb_host))) return fail(RPM_ERR_INVALID, "bad update arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    for (int k = 0; k < m; ++k)
        if (idx_host[k] < 0 || idx_host[k] >= s->n) return fail(RPM_ERR_INVALID, "obstacle index %d out of range", idx_host[k]);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    const int rc = scene_update(ctx, s, idx_host, aabb_host, m);
    if (rc) return rc;
    if (version_out) *version_out = s->version;
    return RPM_OK;
}

int rpm_scene_update_many(rpm_ctx *ctx, int32_t n_scenes, const int32_t *scene_ids, const int32_t *counts,
                          const int32_t *idx_host, const float *aabb_host, uint64_t *versions_out) {
    if (!ctx || n_scenes < 0 || (n_scenes > 0 && (!scene_ids || !counts))) return fail(RPM_ERR_INVALID, "bad update arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    std::vector<SceneUpd> ups;
    size_t off = 0;
    for (int k = 0; k < n_scenes; ++k) {
        SceneRec *s = find_scene(ctx, scene_ids[k]);
        if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_ids[k]);
        const int32_t m = counts[k];
        if (m < 0 || (m > 0 && (!idx_host || !aabb_host))) return fail(RPM_ERR_INVALID, "bad update count %d", m);
        for (int i = 0; i < m; ++i)
            if (idx_host[off + i] < 0 || idx_host[off + i] >= s->n)
                return fail(RPM_ERR_INVALID, "obstacle index %d out of range", idx_host[off + i]);
        ups.push_back(SceneUpd{s, m ? idx_host + off : nullptr, m ? aabb_host + 6 * off : nullptr, m});
        off += (size_t)m;
    }
    if (set_device(ctx)) return RPM_ERR_CUDA;
    const int rc = scene_update_many(ctx, ups);
    if (rc) return rc;
    if (versions_out)
        for (int k = 0; k < n_scenes; ++k) versions_out[k] = ups[k].s->version;
    return RPM_OK;
}

int rpm_scene_destroy(rpm_ctx *ctx, int32_t scene_id) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    for (auto &b : s->bufs) {
        wait_users(ctx, b);
        if (b.ready) { cudaEventSynchronize(b.ready); cudaEventDestroy(b.ready); }
        if (b.mem) cudaFree(b.mem);
    }
    ctx->scenes.erase(scene_id);
    {
        std::lock_guard<std::mutex> dl(ctx->dof_mu);
        ctx->scene_dofs.erase(scene_id);
    }
    delete s;
    return RPM_OK;
}

int rpm_scene_info(rpm_ctx *ctx, int32_t scene_id, int32_t *robot_id, int32_t *num_obstacles, uint64_t *version) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    if (robot_id) *robot_id = s->robot;
    if (num_obstacles) *num_obstacles = s->n;
    if (version) *version = s->version;
    return RPM_OK;
}

int rpm_box_aabb(const float dim[3], const float pos[3], const float quat_xyzw[4], float aabb_out[6]) {
    if (!dim || !pos || !quat_xyzw || !aabb_out) return fail(RPM_ERR_INVALID, "NULL argument");
    const float x = quat_xyzw[0], y = quat_xyzw[1], z = quat_xyzw[2], w = quat_xyzw[3];
    const bool ident = x == 0.f && y == 0.f && z == 0.f && (w == 1.f || w == -1.f);
    const float h[3] = {0.5f * dim[0], 0.5f * dim[1], 0.5f * dim[2]};
    if (ident) {
        for (int k = 0; k < 3; ++k) { aabb_out[k] = (-h[k]) + pos[k]; aabb_out[3 + k] = h[k] + pos[k]; }
    } else {
        const float rad = std::sqrt(h[0] * h[0] + (h[1] * h[1] + h[2] * h[2]));
        for (int k = 0; k < 3; ++k) { aabb_out[k] = pos[k] - rad; aabb_out[3 + k] = pos[k] + rad; }
    }
    return RPM_OK;
}

int rpm_check_configs(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev, int64_t num_configs,
                      uint8_t *valid_dev, double *dist_dev, float *profile_dev, void *stream) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    if (num_configs < 0) return fail(RPM_ERR_INVALID, "negative configuration count");
    if (num_configs > 0 && !q_dev) return fail(RPM_ERR_INVALID, "q is NULL");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    if (num_configs >= (int64_t)1 << 40) return fail(RPM_ERR_RANGE, "too many configurations in one call");
    std::lock_guard<std::mutex> lk(ctx->mu);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    return enqueue_check(ctx, s, precision, q_dev, num_configs, valid_dev, dist_dev, profile_dev, (cudaStream_t)stream);
}

int rpm_check_batch(rpm_ctx *ctx, int32_t precision, const rpm_batch_item *items, int32_t n_items, void *stream) {
    if (!ctx || (n_items > 0 && !items) || n_items < 0) return fail(RPM_ERR_INVALID, "bad batch");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    std::vector<SegReq> reqs;
    int64_t total = 0;
    for (int k = 0; k < n_items; ++k) {
        const rpm_batch_item &it = items[k];
        SceneRec *s = find_scene(ctx, it.scene_id);
        if (!s) return fail(RPM_ERR_INVALID, "batch item %d: unknown scene %d", k, it.scene_id);
        if (it.num_configs < 0 || (it.num_configs > 0 && !it.q_dev)) return fail(RPM_ERR_INVALID, "batch item %d: bad configurations", k);
        total += it.num_configs;
        reqs.push_back(SegReq{s, it.q_dev, it.num_configs, it.valid_dev, it.dist_dev, it.profile_dev});
    }
    if (total >= (int64_t)1 << 40) return fail(RPM_ERR_RANGE, "too many configurations in one batch");
    return enqueue_segments(ctx, precision, reqs, (cudaStream_t)stream);
}

int rpm_check_edges_batch(rpm_ctx *ctx, int32_t precision, const rpm_edge_batch_item *items, int32_t n_items,
                          void *stream) {
    if (!ctx || (n_items > 0 && !items) || n_items < 0) return fail(RPM_ERR_INVALID, "bad edge batch");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    std::vector<EdgeReq> reqs;
    int64_t total = 0;
    for (int k = 0; k < n_items; ++k) {
        const rpm_edge_batch_item &it = items[k];
        SceneRec *s = find_scene(ctx, it.scene_id);
        if (!s) return fail(RPM_ERR_INVALID, "edge batch item %d: unknown scene %d", k, it.scene_id);
        if (it.num_edges < 0 || (it.num_edges > 0 && (!it.q1_dev || !it.q2_dev || !it.valid_dev)))
            return fail(RPM_ERR_INVALID, "edge batch item %d: bad edge buffers", k);
        if (!(it.step > 0.f) && it.num_checks < 1)
            return fail(RPM_ERR_INVALID, "edge batch item %d: need step > 0 or num_checks >= 1", k);
        total += it.num_edges;
        reqs.push_back(EdgeReq{s, it.q1_dev, it.q2_dev, it.num_edges, it.step, it.num_checks, it.valid_dev, it.checks_dev});
    }
    if (total >= (int64_t)1 << 40) return fail(RPM_ERR_RANGE, "too many edges in one batch");
    if (total == 0) return RPM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch *sc = nullptr;
    int rc = get_scratch(ctx, st, total, &sc);
    if (!rc) rc = edge_scratch(ctx, sc, total, st);
    if (rc) return rc;
    sc->last_configs = total;
    sc->timed = false;
    rc = enqueue_edge_batch(ctx, sc, precision, reqs, kDefaultEdgeCtas, st);
    if (rc) return rc;
    std::vector<SceneBuf *> used;
    for (const EdgeReq &r : reqs) {
        SceneBuf *b = &r.scene->bufs[r.scene->cur];
        if (std::find(used.begin(), used.end(), b) == used.end()) used.push_back(b);
    }
    for (SceneBuf *b : used) {
        prune_users(ctx, *b);
        cudaEvent_t e = get_event(ctx);
        CK(cudaEventRecord(e, st));
        b->users.push_back(e);
    }
    return RPM_OK;
}

int rpm_check_edges(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q1_dev, const float *q2_dev,
                    int64_t num_edges, float step, int32_t num_checks, uint8_t *valid_dev, int32_t *checks_dev,
                    void *stream) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    if (num_edges < 0 || (num_edges > 0 && (!q1_dev || !q2_dev || !valid_dev))) return fail(RPM_ERR_INVALID, "bad edge buffers");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    if (!(step > 0.f) && num_checks < 1) return fail(RPM_ERR_INVALID, "need step > 0 or num_checks >= 1");
    if (num_edges >= (int64_t)1 << 40) return fail(RPM_ERR_RANGE, "too many edges in one call");
    std::lock_guard<std::mutex> lk(ctx->mu);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch *sc = nullptr;
    int rc = get_scratch(ctx, st, std::max<int64_t>(1, num_edges), &sc);   // pair-recheck lists sized by the batch
    if (rc) return rc;
    rc = edge_scratch(ctx, sc, num_edges, st);
    if (rc) return rc;
    sc->last_configs = num_edges;
    sc->timed = false;
    const int ctas = kDefaultEdgeCtas;
    SceneBuf &buf = s->bufs[s->cur];
    if (ctx->use_graphs) {
        // replay a captured graph of the whole pipeline when the arguments repeat
        uint32_t step_bits;
        std::memcpy(&step_bits, &step, sizeof step_bits);
        std::vector<uint64_t> key = {(uint64_t)(uintptr_t)&buf, (uint64_t)(uintptr_t)buf.f, (uint64_t)precision,
                                     (uint64_t)(uintptr_t)q1_dev, (uint64_t)(uintptr_t)q2_dev, (uint64_t)num_edges,
                                     (uint64_t)step_bits, (uint64_t)num_checks, (uint64_t)(uintptr_t)valid_dev,
                                     (uint64_t)(uintptr_t)checks_dev, (uint64_t)ctx->tune_epoch, (uint64_t)ctx->layout};
        cudaGraphExec_t exec = nullptr;
        for (auto &g : sc->graphs) if (g.key == key) { exec = g.exec; break; }
        if (!exec) {
            cudaStream_t cap;
            CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_edges(ctx, sc, s, precision, q1_dev, q2_dev, num_edges, step, num_checks, valid_dev, checks_dev,
                               ctas, cap);
            cudaGraph_t graph = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(cap, &graph);
            cudaStreamDestroy(cap);
            if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
            CK(ce);
            CK(cudaGraphInstantiate(&exec, graph, 0));
            cudaGraphDestroy(graph);
            if (sc->graphs.size() >= 16) { cudaGraphExecDestroy(sc->graphs.front().exec); sc->graphs.erase(sc->graphs.begin()); }
            sc->graphs.push_back({key, exec});
        }
        CK(cudaGraphLaunch(exec, st));
    } else {
        rc = enqueue_edges(ctx, sc, s, precision, q1_dev, q2_dev, num_edges, step, num_checks, valid_dev, checks_dev, ctas, st);
        if (rc) return rc;
    }
    prune_users(ctx, buf);
    cudaEvent_t e = get_event(ctx);
    CK(cudaEventRecord(e, st));
    buf.users.push_back(e);
    return RPM_OK;
}

// Shared set-up of the nearest-point and underestimation calls (caller holds ctx->mu).
static int near_setup(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q, int64_t C, cudaStream_t st,
                      NearParams &p, SceneBuf **used) {
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    SceneBuf &buf = s->bufs[s->cur];
    if (buf.pending) {
        if (cudaEventQuery(buf.ready) == cudaSuccess) buf.pending = false;
        else CK(cudaStreamWaitEvent(st, buf.ready, 0));
    }
    std::memset(&p, 0, sizeof p);
    p.robot = ctx->robots[s->robot].dev;
    p.obs_f = buf.f;
    p.obs_d = buf.d;
    p.n = s->n;
    p.n_pad = s->n_pad;
    p.q = q;
    p.C = C;
    p.nmd.eq = ctx->params.equality_threshold;
    p.nmd.maxd = ctx->params.max_distance;
    p.nmf.eq = (float)ctx->params.equality_threshold;
    p.nmf.maxd = (float)ctx->params.max_distance;
    *used = &buf;
    return RPM_OK;
}

static int near_done(rpm_ctx *ctx, SceneBuf *buf, cudaStream_t st) {
    prune_users(ctx, *buf);
    cudaEvent_t e = get_event(ctx);
    CK(cudaEventRecord(e, st));
    buf->users.push_back(e);
    return RPM_OK;
}

int rpm_distance_nearest(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev, int64_t num_configs,
                         double *dist_dev, float *profile_dev, float *nearest_dev, uint8_t *nearest_valid_dev,
                         void *stream) {
    if (!ctx || num_configs < 0 || (num_configs > 0 && (!q_dev || !dist_dev || !profile_dev || !nearest_valid_dev)))
        return fail(RPM_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t st = (cudaStream_t)stream;
    NearParams p;
    SceneBuf *buf = nullptr;
    int rc = near_setup(ctx, scene_id, precision, q_dev, num_configs, st, p, &buf);
    if (rc) return rc;
    if (num_configs > 0 && p.n > 0 && !nearest_dev) return fail(RPM_ERR_INVALID, "NULL nearest-point buffer");
    p.dist = dist_dev;
    p.profile = profile_dev;
    p.nearest = nearest_dev;
    p.flag = nearest_valid_dev;
    CK(launch_distance_nearest(precision == RPM_PREC_FP32_REF ? RPM_PREC_FP32_REF : RPM_PREC_FP64, p, st));
    return near_done(ctx, buf, st);
}

int rpm_decision_margins(rpm_ctx *ctx, int32_t scene_id, const float *q_dev, int64_t num_configs,
                         double *margin_valid_dev, double *margin_dist_dev, void *stream) {
    if (!ctx || num_configs < 0 || (num_configs > 0 && (!q_dev || !margin_valid_dev || !margin_dist_dev)))
        return fail(RPM_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t st = (cudaStream_t)stream;
    NearParams p;
    SceneBuf *buf = nullptr;
    int rc = near_setup(ctx, scene_id, RPM_PREC_FP64, q_dev, num_configs, st, p, &buf);
    if (rc) return rc;
    p.margin_valid = margin_valid_dev;
    p.margin_dist = margin_dist_dev;
    CK(launch_decision_margins(p, st));
    return near_done(ctx, buf, st);
}

static int spine_robot(rpm_ctx *ctx, int32_t robot_id, SpineParams &p) {
    if (robot_id < 0 || robot_id >= (int32_t)ctx->robots.size() || !ctx->robots[robot_id].dev)
        return fail(RPM_ERR_INVALID, "unknown robot %d", robot_id);
    std::memset(&p, 0, sizeof p);
    p.robot = ctx->robots[robot_id].dev;
    p.maxd = (float)ctx->params.max_distance;
    return RPM_OK;
}

int rpm_enclosing_radii(rpm_ctx *ctx, int32_t robot_id, const float *q_dev, int64_t num_configs, float *radii_dev,
                        void *stream) {
    if (!ctx || num_configs < 0 || (num_configs > 0 && (!q_dev || !radii_dev))) return fail(RPM_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    SpineParams p;
    const int rc = spine_robot(ctx, robot_id, p);
    if (rc) return rc;
    p.q = q_dev;
    p.C = num_configs;
    p.radii = radii_dev;
    CK(launch_enclosing_radii(p, (cudaStream_t)stream));
    return RPM_OK;
}

int rpm_extend_spines(rpm_ctx *ctx, int32_t robot_id, const float *q_dev, const float *q_e_dev, const float *dist_dev,
                      const float *profile_dev, int64_t num_spines, int32_t num_iter, int32_t expanded, float *q_new_dev,
                      int32_t *status_dev, void *stream) {
    if (!ctx || num_spines < 0 ||
        (num_spines > 0 && (!q_dev || !q_e_dev || !dist_dev || !profile_dev || !q_new_dev || !status_dev)))
        return fail(RPM_ERR_INVALID, "bad arguments");
    if (num_iter < 1) return fail(RPM_ERR_INVALID, "num_iter must be >= 1");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    SpineParams p;
    const int rc = spine_robot(ctx, robot_id, p);
    if (rc) return rc;
    p.q = q_dev;
    p.qe = q_e_dev;
    p.dist = dist_dev;
    p.profile = profile_dev;
    p.C = num_spines;
    p.num_iter = num_iter;
    p.expanded = expanded;
    p.q_new = q_new_dev;
    p.status = status_dev;
    CK(launch_extend_spines(p, (cudaStream_t)stream));
    return RPM_OK;
}

}  // extern "C"

namespace rpm {
namespace impl {
// rpm_reached_states with ctx->mu held (the C entry point and the server's
// DRGBT requests).
int reached_states_locked(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_current_dev,
                          const float *horizon_dev, int64_t horizon_size, const rpm_spine_params *params,
                          float *q_reached_dev, int32_t *status_dev, double *dist_dev, cudaStream_t st) {
    if (!ctx || !params || horizon_size < 0 || !q_current_dev ||
        (horizon_size > 0 && (!horizon_dev || !q_reached_dev || !status_dev)))
        return fail(RPM_ERR_INVALID, "bad arguments");
    if (params->num_iter < 1 || params->num_layers < 0) return fail(RPM_ERR_INVALID, "num_iter >= 1 and num_layers >= 0");
    NearParams np;
    SceneBuf *buf = nullptr;
    int rc = near_setup(ctx, scene_id, RPM_PREC_FP32_REF, q_current_dev, 1, st, np, &buf);
    if (rc) return rc;
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    SceneRec *s = find_scene(ctx, scene_id);
    const int L = ctx->robots[s->robot].desc.num_dofs;
    // computeDistance of the current state with nearest points (the stream's
    // planner scratch).  A short horizon's final computeDistance runs on the same
    // CTA-per-state kernel (its points land in the scratch too), when they fit
    // in a few megabytes; otherwise it is an ordinary check.
    const size_t near_floats = (size_t)std::max(1, np.n) * 6 * L;
    const bool short_h = dist_dev && horizon_size > 0 && horizon_size <= 64 &&
                         (size_t)horizon_size * near_floats * 4 <= ((size_t)8 << 20);
    const size_t h_bytes = short_h ? (size_t)horizon_size * (8 + 4 * (size_t)L + 4 * near_floats) + 64 : 0;
    const size_t skel_off = (16 + 4 * (size_t)L + 4 * near_floats + 16 + h_bytes + 15) & ~(size_t)15;
    const size_t bytes = skel_off + 4 * 3 * ((size_t)L + 1);
    void *aux = nullptr;
    rc = get_aux(ctx, st, bytes, &aux);
    if (rc) return rc;
    char *tmp = static_cast<char *>(aux);
    np.dist = reinterpret_cast<double *>(tmp);
    np.flag = reinterpret_cast<uint8_t *>(tmp + 8);
    np.profile = reinterpret_cast<float *>(tmp + 16);
    np.nearest = reinterpret_cast<float *>(tmp + 16 + 4 * (size_t)L);
    np.skel_out = reinterpret_cast<float *>(tmp + skel_off);   // q_cur's float skeleton, for the spines
    CK(launch_distance_nearest(RPM_PREC_FP32_REF, np, st));
    SpineParams p;
    std::memset(&p, 0, sizeof p);
    p.robot = np.robot;
    p.qe = horizon_dev;
    p.C = horizon_size;
    p.num_iter = params->num_iter;
    p.expanded = params->expanded;
    p.num_layers = params->num_layers;
    p.d_crit = params->d_crit;
    p.q_new = q_reached_dev;
    p.status = status_dev;
    p.q_cur = q_current_dev;
    p.cur_dist = np.dist;
    p.cur_prof = np.profile;
    p.cur_near = np.nearest;
    p.cur_skel = np.skel_out;
    p.n = np.n;
    p.maxd = np.nmf.maxd;
    p.L = L;
    CK(launch_reached_states(p, st));
    if (short_h) {
        // computeDistance(q_reached, true): the exact FP64 value for the FP64 and
        // FP32 + recheck forms, the reference's numerics for RPM_PREC_FP32_REF
        char *h = tmp + 16 + 4 * (size_t)L + 4 * near_floats + 16;
        NearParams hp = np;
        hp.skel_out = nullptr;
        hp.q = q_reached_dev;
        hp.C = horizon_size;
        hp.dist = dist_dev;
        hp.nearest = reinterpret_cast<float *>(h);
        hp.profile = reinterpret_cast<float *>(h + 4 * (size_t)horizon_size * near_floats);
        hp.flag = reinterpret_cast<uint8_t *>(h + 4 * (size_t)horizon_size * (near_floats + L));
        CK(launch_distance_nearest(precision == RPM_PREC_FP32_REF ? RPM_PREC_FP32_REF : RPM_PREC_FP64, hp, st));
    }
    rc = near_done(ctx, buf, st);
    if (rc) return rc;
    // computeDistance(q_reached, true) in the requested form
    if (dist_dev && horizon_size > 0 && !short_h)
        return enqueue_check(ctx, s, precision, q_reached_dev, horizon_size, nullptr, dist_dev, nullptr, st);
    return RPM_OK;
}
}  // namespace impl
}  // namespace rpm

extern "C" {

int rpm_reached_states(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_current_dev,
                       const float *horizon_dev, int64_t horizon_size, const rpm_spine_params *params,
                       float *q_reached_dev, int32_t *status_dev, double *dist_dev, void *stream) {
    if (!ctx) return fail(RPM_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return reached_states_locked(ctx, scene_id, precision, q_current_dev, horizon_dev, horizon_size, params,
                                 q_reached_dev, status_dev, dist_dev, (cudaStream_t)stream);
}

}  // extern "C"

namespace rpm {
namespace impl {
// rpm_motion_validity with ctx->mu held (the C entry point and the server's
// DRGBT requests).
int motion_validity_locked(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_prev_dev,
                           const float *q_cur_dev, int64_t num_motions, const rpm_moving_box *boxes, int32_t num_boxes,
                           float max_iter_time, int32_t num_points, uint8_t *valid_dev, int32_t *checks_dev,
                           cudaStream_t st) {
    if (!ctx || num_motions < 0 || num_boxes < 0 || (num_boxes > 0 && !boxes) ||
        (num_motions > 0 && (!q_prev_dev || !q_cur_dev || !valid_dev)))
        return fail(RPM_ERR_INVALID, "bad arguments");
    if (precision != RPM_PREC_FP64 && precision != RPM_PREC_FP32_REF)
        return fail(RPM_ERR_INVALID, "motion validity runs RPM_PREC_FP64 or RPM_PREC_FP32_REF");
    if (num_points < 1) return fail(RPM_ERR_INVALID, "num_points must be >= 1");
    NearParams np;
    SceneBuf *buf = nullptr;
    int rc = near_setup(ctx, scene_id, precision, q_prev_dev, num_motions, st, np, &buf);
    if (rc) return rc;
    if (num_motions == 0) return RPM_OK;
    const int n = np.n;
    for (int b = 0; b < num_boxes; ++b)
        if (boxes[b].index < 0 || boxes[b].index >= n) return fail(RPM_ERR_INVALID, "moving box %d: bad index", b);
    if ((int64_t)num_points * num_boxes > (int64_t)1 << 24) return fail(RPM_ERR_RANGE, "too many moving-box steps");
    // the moving boxes' AABBs before each check, on the host in float as the
    // reference's Environment::moveStraight and fcl compute them
    const float dt = max_iter_time / (float)num_points;
    const size_t moving_bytes = ((size_t)std::max(n, 1) + 15) & ~(size_t)15;
    const size_t idx_bytes = (((size_t)num_boxes * 4) + 15) & ~(size_t)15;
    std::vector<unsigned char> host(moving_bytes + idx_bytes + (size_t)num_points * num_boxes * 24, 0);
    int32_t *hidx = reinterpret_cast<int32_t *>(host.data() + moving_bytes);
    float *haabb = reinterpret_cast<float *>(host.data() + moving_bytes + idx_bytes);
    for (int b = 0; b < num_boxes; ++b) {
        host[boxes[b].index] = 1;
        hidx[b] = boxes[b].index;
        float pos[3] = {boxes[b].pos[0], boxes[b].pos[1], boxes[b].pos[2]};
        for (int k = 0; k < num_points; ++k) {
            pos[0] = pos[0] - dt * boxes[b].max_vel;
            rpm_box_aabb(boxes[b].dim, pos, boxes[b].quat_xyzw, haabb + ((size_t)k * num_boxes + b) * 6);
        }
    }
    AsyncScratch scratch;
    scratch.st = st;
    CK(cudaMallocAsync(&scratch.p, host.size(), st));
    unsigned char *dev = static_cast<unsigned char *>(scratch.p);
    CK(cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, st));
    MotionParams p;
    std::memset(&p, 0, sizeof p);
    p.robot = np.robot;
    p.obs_f = np.obs_f;
    p.obs_d = np.obs_d;
    p.n = n;
    p.n_pad = np.n_pad;
    p.q_prev = q_prev_dev;
    p.q_cur = q_cur_dev;
    p.M = num_motions;
    p.N = num_points;
    p.n_mov = num_boxes;
    p.max_iter_time = max_iter_time;
    p.moving = dev;
    p.mov_idx = reinterpret_cast<const int32_t *>(dev + moving_bytes);
    p.mov_aabb = reinterpret_cast<const float *>(dev + moving_bytes + idx_bytes);
    p.nmd = np.nmd;
    p.nmf = np.nmf;
    p.valid = valid_dev;
    p.checks = checks_dev;
    CK(launch_motion_validity(precision, p, st));
    return near_done(ctx, buf, st);
}
}  // namespace impl
}  // namespace rpm

extern "C" {

int rpm_motion_validity(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_prev_dev,
                        const float *q_cur_dev, int64_t num_motions, const rpm_moving_box *boxes, int32_t num_boxes,
                        float max_iter_time, int32_t num_points, uint8_t *valid_dev, int32_t *checks_dev, void *stream) {
    if (!ctx) return fail(RPM_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return motion_validity_locked(ctx, scene_id, precision, q_prev_dev, q_cur_dev, num_motions, boxes, num_boxes,
                                  max_iter_time, num_points, valid_dev, checks_dev, (cudaStream_t)stream);
}

int rpm_scene_move_straight(rpm_ctx *ctx, int32_t scene_id, rpm_moving_box *boxes, int32_t num_boxes, float delta_time,
                            int32_t steps, uint64_t *version_out) {
    if (!ctx || num_boxes < 0 || (num_boxes > 0 && !boxes) || steps < 0) return fail(RPM_ERR_INVALID, "bad arguments");
    std::vector<int32_t> idx((size_t)num_boxes);
    std::vector<float> aabb((size_t)num_boxes * 6);
    for (int b = 0; b < num_boxes; ++b) {
        for (int k = 0; k < steps; ++k) boxes[b].pos[0] = boxes[b].pos[0] - delta_time * boxes[b].max_vel;
        rpm_box_aabb(boxes[b].dim, boxes[b].pos, boxes[b].quat_xyzw, aabb.data() + 6 * (size_t)b);
        idx[b] = boxes[b].index;
    }
    return rpm_scene_update(ctx, scene_id, idx.data(), aabb.data(), num_boxes, version_out);
}

int rpm_distance_underestimation(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev,
                                 int64_t num_configs, const float *nearest_dev, double *dist_dev, float *profile_dev,
                                 uint8_t *complete_dev, void *stream) {
    if (!ctx || num_configs < 0 || (num_configs > 0 && (!q_dev || !dist_dev || !profile_dev || !complete_dev)))
        return fail(RPM_ERR_INVALID, "bad arguments");
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaStream_t st = (cudaStream_t)stream;
    NearParams p;
    SceneBuf *buf = nullptr;
    int rc = near_setup(ctx, scene_id, precision, q_dev, num_configs, st, p, &buf);
    if (rc) return rc;
    if (num_configs > 0 && p.n > 0 && !nearest_dev) return fail(RPM_ERR_INVALID, "NULL nearest-point buffer");
    p.dist = dist_dev;
    p.profile = profile_dev;
    p.nearest = const_cast<float *>(nearest_dev);
    p.flag = complete_dev;
    CK(launch_distance_underest(precision == RPM_PREC_FP32_REF ? RPM_PREC_FP32_REF : RPM_PREC_FP64, p, st));
    return near_done(ctx, buf, st);
}

int rpm_ctx_set_layout(rpm_ctx *ctx, int32_t layout) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    if (layout < RPM_LAYOUT_AUTO || layout > RPM_LAYOUT_WARP) return fail(RPM_ERR_INVALID, "unknown layout %d", layout);
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->layout = layout;
    return RPM_OK;
}

int rpm_ctx_set_graphs(rpm_ctx *ctx, int enable) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->use_graphs = enable != 0;
    return RPM_OK;
}

}  // extern "C"

// ---- tile shapes and the autotuner ------------------------------------------
// Times 'call' (one check on 'st') with each candidate shape in the bucket's
// table entry: a warm-up call, then 'reps' timed calls, median; keeps the
// fastest.  The candidates go through the same table lookups the launches use.
template <typename F>
static int tune_bucket(rpm_ctx *ctx, const TuneKey &key, const std::vector<rpm_tile_shape> &cands, int reps, F call,
                       rpm_tile_shape *best) {
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    rpm_tile_shape win{0, 0, 0, 1e30f};
    int rc = RPM_OK;
    for (const rpm_tile_shape &c : cands) {
        {
            std::lock_guard<std::mutex> lk(ctx->mu);
            ctx->tune[key] = c;
            ctx->tune_epoch++;
        }
        std::vector<float> ms;
        for (int r = 0; r <= reps && !rc; ++r) {
            if (cudaEventRecord(a, st) != cudaSuccess) { rc = fail(RPM_ERR_CUDA, "event record failed"); break; }
            rc = call(st);
            if (rc) break;
            if (cudaEventRecord(b, st) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) {
                rc = fail(RPM_ERR_CUDA, "timing the candidate failed");
                break;
            }
            float t = 0.f;
            cudaEventElapsedTime(&t, a, b);
            if (r > 0) ms.push_back(t);   // the first call is the warm-up
        }
        if (rc) break;
        std::sort(ms.begin(), ms.end());
        const float med = ms[ms.size() / 2];
        if (med < win.ms) { win = c; win.ms = med; }
    }
    cudaStreamSynchronize(st);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamDestroy(st);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (rc) {
        ctx->tune.erase(key);
    } else {
        ctx->tune[key] = win;
        *best = win;
    }
    ctx->tune_epoch++;
    return rc;
}

extern "C" {

int rpm_autotune_configs(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_dev, int64_t num_configs,
                         uint8_t *valid_dev, double *dist_dev, float *profile_dev, int32_t reps, rpm_tile_shape *best) {
    if (!ctx || !best || num_configs < 1 || !q_dev || reps < 1 || (!valid_dev && !dist_dev && !profile_dev))
        return fail(RPM_ERR_INVALID, "bad arguments");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    TuneKey key;
    int gmax = 32;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (ctx->layout != RPM_LAYOUT_AUTO) return fail(RPM_ERR_INVALID, "the autotuner needs RPM_LAYOUT_AUTO");
        SceneRec *s = find_scene(ctx, scene_id);
        if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
        const int outputs = (valid_dev ? RPM_OUT_VALID : 0) | (dist_dev ? RPM_OUT_DIST : 0) | (profile_dev ? RPM_OUT_PROFILE : 0);
        key = tune_key(ctx, s, num_configs, precision, outputs, 0);
        const int D = ctx->robots[s->robot].desc.num_dofs;   // the warp's skeleton buffer bounds its configurations
        gmax = std::max(1, kWidePtsBytes / ((D + 1) * 3 * (int)(precision == RPM_PREC_FP64 ? sizeof(double) : sizeof(float))));
    }
    std::vector<rpm_tile_shape> cands = {{RPM_LAYOUT_LANE, 0, 0, 0.f}, {RPM_LAYOUT_WARP, 0, 0, 0.f}};
    for (int g : {1, 2, 4, 8, 16, 32})
        if (g <= gmax) cands.push_back(rpm_tile_shape{RPM_LAYOUT_WARP, g, 0, 0.f});
    if (gmax < 32 && gmax != 1 && gmax != 2 && gmax != 4 && gmax != 8 && gmax != 16)
        cands.push_back(rpm_tile_shape{RPM_LAYOUT_WARP, gmax, 0, 0.f});
    return tune_bucket(ctx, key, cands, reps, [&](cudaStream_t st) {
        return rpm_check_configs(ctx, scene_id, precision, q_dev, num_configs, valid_dev, dist_dev, profile_dev, st);
    }, best);
}

int rpm_autotune_edges(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q1_dev, const float *q2_dev,
                       int64_t num_edges, float step, int32_t num_checks, uint8_t *valid_dev, int32_t reps,
                       rpm_tile_shape *best) {
    if (!ctx || !best || num_edges < 1 || !q1_dev || !q2_dev || !valid_dev || reps < 1)
        return fail(RPM_ERR_INVALID, "bad arguments");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    TuneKey key;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (ctx->layout != RPM_LAYOUT_AUTO) return fail(RPM_ERR_INVALID, "the autotuner needs RPM_LAYOUT_AUTO");
        SceneRec *s = find_scene(ctx, scene_id);
        if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
        key = tune_key(ctx, s, num_edges, precision, RPM_OUT_VALID, 1);
    }
    std::vector<rpm_tile_shape> cands;
    for (int c : {1, 2, 3, 4, 6, 8}) cands.push_back(rpm_tile_shape{RPM_LAYOUT_LANE, 0, c, 0.f});
    for (int g : {0, 1, 2, 4, 8}) cands.push_back(rpm_tile_shape{RPM_LAYOUT_WARP, g, 0, 0.f});
    return tune_bucket(ctx, key, cands, reps, [&](cudaStream_t st) {
        return rpm_check_edges(ctx, scene_id, precision, q1_dev, q2_dev, num_edges, step, num_checks, valid_dev, nullptr, st);
    }, best);
}

int rpm_set_tile_shape(rpm_ctx *ctx, int32_t scene_id, int32_t precision, int32_t edges, int64_t count,
                       int32_t outputs, const rpm_tile_shape *shape) {
    if (!ctx || count < 1 || outputs < 1 || outputs > 7) return fail(RPM_ERR_INVALID, "bad arguments");
    if (shape && ((shape->layout != RPM_LAYOUT_LANE && shape->layout != RPM_LAYOUT_WARP) || shape->configs_per_warp < 0 ||
                  shape->configs_per_warp > 32 || shape->ctas_per_sm < 0 || shape->ctas_per_sm > 32))
        return fail(RPM_ERR_INVALID, "bad tile shape");
    std::lock_guard<std::mutex> lk(ctx->mu);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    const TuneKey key = tune_key(ctx, s, count, precision, edges ? RPM_OUT_VALID : outputs, edges ? 1 : 0);
    if (shape) ctx->tune[key] = *shape;
    else ctx->tune.erase(key);
    ctx->tune_epoch++;
    return RPM_OK;
}

int rpm_tuning_save(rpm_ctx *ctx, const char *path) {
    if (!ctx || !path) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    FILE *f = std::fopen(path, "w");
    if (!f) return fail(RPM_ERR_INVALID, "cannot write %s", path);
    cudaDeviceProp prop;
    const char *name = cudaGetDeviceProperties(&prop, ctx->device) == cudaSuccess ? prop.name : "unknown";
    std::fprintf(f, "{\n \"format\": \"rpmplv2_gb300 tile shapes 1\",\n \"device\": \"%s\",\n \"entries\": [\n", name);
    size_t k = 0;
    for (const auto &kv : ctx->tune) {
        const TuneKey &t = kv.first;
        const rpm_tile_shape &v = kv.second;
        std::fprintf(f,
                     "  {\"robot_kind\": %d, \"dofs\": %d, \"obstacles_log2\": %d, \"count_log2\": %d, "
                     "\"precision\": %d, \"outputs\": %d, \"edges\": %d, \"layout\": %d, \"configs_per_warp\": %d, "
                     "\"ctas_per_sm\": %d, \"ms\": %.4f}%s\n",
                     t.robot_kind, t.dofs, t.obstacles_log2, t.count_log2, t.prec, t.outputs, t.edges, v.layout,
                     v.configs_per_warp, v.ctas_per_sm, (double)v.ms, ++k < ctx->tune.size() ? "," : "");
    }
    std::fprintf(f, " ]\n}\n");
    const bool ok = std::fclose(f) == 0;
    return ok ? RPM_OK : fail(RPM_ERR_INVALID, "writing %s failed", path);
}

// The value after "\"name\":" in one entry line.
static bool json_num(const std::string &line, const char *name, double &v) {
    const std::string key = std::string("\"") + name + "\":";
    const size_t at = line.find(key);
    if (at == std::string::npos) return false;
    char *end = nullptr;
    v = std::strtod(line.c_str() + at + key.size(), &end);
    return end != line.c_str() + at + key.size();
}

int rpm_tuning_load(rpm_ctx *ctx, const char *path) {
    if (!ctx || !path) return fail(RPM_ERR_INVALID, "NULL argument");
    FILE *f = std::fopen(path, "r");
    if (!f) return fail(RPM_ERR_INVALID, "cannot read %s", path);
    std::vector<std::pair<TuneKey, rpm_tile_shape>> got;
    char buf[1024];
    int lineno = 0, rc = RPM_OK;
    while (std::fgets(buf, sizeof buf, f)) {
        ++lineno;
        const std::string line(buf);
        if (line.find("\"robot_kind\"") == std::string::npos) continue;
        static const char *names[11] = {"robot_kind", "dofs", "obstacles_log2", "count_log2", "precision", "outputs",
                                        "edges", "layout", "configs_per_warp", "ctas_per_sm", "ms"};
        double v[11];
        for (int i = 0; i < 11 && !rc; ++i)
            if (!json_num(line, names[i], v[i])) rc = fail(RPM_ERR_INVALID, "%s:%d: no \"%s\"", path, lineno, names[i]);
        if (rc) break;
        const rpm_tile_shape sh{(int32_t)v[7], (int32_t)v[8], (int32_t)v[9], (float)v[10]};
        if ((sh.layout != RPM_LAYOUT_LANE && sh.layout != RPM_LAYOUT_WARP) || sh.configs_per_warp < 0 ||
            sh.configs_per_warp > 32 || sh.ctas_per_sm < 0 || sh.ctas_per_sm > 32) {
            rc = fail(RPM_ERR_INVALID, "%s:%d: bad tile shape", path, lineno);
            break;
        }
        got.push_back({TuneKey{(int32_t)v[0], (int32_t)v[1], (int32_t)v[2], (int32_t)v[3], (int32_t)v[4], (int32_t)v[5],
                               (int32_t)v[6]}, sh});
    }
    std::fclose(f);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    for (const auto &e : got) ctx->tune[e.first] = e.second;
    ctx->tune_epoch++;
    return RPM_OK;
}

int rpm_last_shape(rpm_ctx *ctx, void *stream, rpm_tile_shape *out) {
    if (!ctx || !out) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scratch.find((cudaStream_t)stream);
    if (it == ctx->scratch.end()) return fail(RPM_ERR_INVALID, "no launch on this stream yet");
    *out = it->second->last_shape;
    return RPM_OK;
}

int rpm_check_configs_host(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_host, int64_t num_configs,
                           uint8_t *valid_host, double *dist_host, float *profile_host) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    if (num_configs < 0 || (num_configs > 0 && !q_host)) return fail(RPM_ERR_INVALID, "bad configuration buffer");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    std::lock_guard<std::mutex> lk(ctx->mu);
    SceneRec *s = find_scene(ctx, scene_id);
    if (!s) return fail(RPM_ERR_INVALID, "unknown scene %d", scene_id);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    const int D = ctx->robots[s->robot].desc.num_dofs;
    // Pinned (page-locked, mapped) host buffers: the kernels read q and write
    // the outputs in host memory directly, over NVLink-C2C on GB300, in one
    // launch.  Any other buffer takes the staged path below, and so does a
    // batch that the FP32 lane kernel checks in binned order: its scattered
    // row reads and output writes would cross the link line by line, while the
    // staged path moves whole buffers by DMA.
    const float *zq = mapped_ptr(q_host);
    uint8_t *zv = valid_host ? mapped_ptr(valid_host) : nullptr;
    double *zd = dist_host ? mapped_ptr(dist_host) : nullptr;
    float *zp = profile_host ? mapped_ptr(profile_host) : nullptr;
    const bool binned = precision == RPM_PREC_FP32_RECHECK && num_configs >= kBinMinConfigs &&
                        !use_warp_layout(ctx, SegReq{s, q_host, num_configs, valid_host, dist_host, profile_host},
                                         num_configs, precision, true);
    if (!binned && num_configs > 0 && zq && (!valid_host || zv) && (!dist_host || zd) && (!profile_host || zp)) {
        if (!ctx->hs[0]) CK(cudaStreamCreateWithFlags(&ctx->hs[0], cudaStreamNonBlocking));
        cudaStream_t st = ctx->hs[0];
        int rc = enqueue_check(ctx, s, precision, zq, num_configs, zv, zd, zp, st);
        if (rc) return rc;
        CK(cudaStreamSynchronize(st));
        return host_status(ctx, st);
    }
    // Pinned buffers move by DMA in chunks of up to 1,048,576 configurations
    // (the copies are short next to the checks); other buffers in chunks of
    // 262,144, two streams overlapping the copies of one chunk with the checks
    // of the other.
    const bool pinned = zq && (!valid_host || zv) && (!dist_host || zd) && (!profile_host || zp);
    const int64_t chunk = pinned ? std::max<int64_t>(1 << 18, std::min<int64_t>(num_configs, 1 << 20)) : 1 << 18;
    if (ctx->hcap_cfg < (size_t)chunk || ctx->hcap_qf < (size_t)(chunk * D)) {
        for (int i = 0; i < 2; ++i) {
            if (!ctx->hs[i]) CK(cudaStreamCreateWithFlags(&ctx->hs[i], cudaStreamNonBlocking));
            cudaFree(ctx->hq[i]); cudaFree(ctx->hv[i]); cudaFree(ctx->hd[i]);
            ctx->hq[i] = nullptr; ctx->hv[i] = nullptr; ctx->hd[i] = nullptr;
        }
        ctx->hcap_cfg = ctx->hcap_qf = 0;
        const size_t cfg = (size_t)chunk;
        for (int i = 0; i < 2; ++i)
            if (cudaMalloc(&ctx->hq[i], cfg * D * sizeof(float)) != cudaSuccess ||
                cudaMalloc(&ctx->hv[i], cfg) != cudaSuccess || cudaMalloc(&ctx->hd[i], cfg * sizeof(double)) != cudaSuccess)
                return fail(RPM_ERR_NOMEM, "staging allocation failed");
        ctx->hcap_cfg = cfg;
        ctx->hcap_qf = cfg * D;
    }
    if (profile_host && ctx->hcap_prof < (size_t)(chunk * D)) {
        for (int i = 0; i < 2; ++i) {
            cudaFree(ctx->hp[i]);
            ctx->hp[i] = nullptr;
            if (cudaMalloc(&ctx->hp[i], chunk * D * sizeof(float)) != cudaSuccess)
                return fail(RPM_ERR_NOMEM, "staging allocation failed");
        }
        ctx->hcap_prof = chunk * D;
    }
    int k = 0;
    for (int64_t off = 0; off < num_configs; off += chunk, ++k) {
        const int i = k & 1;
        cudaStream_t st = ctx->hs[i];
        const int64_t n = std::min(chunk, num_configs - off);
        CK(cudaMemcpyAsync(ctx->hq[i], q_host + off * D, n * D * sizeof(float), cudaMemcpyHostToDevice, st));
        int rc = enqueue_check(ctx, s, precision, ctx->hq[i], n, valid_host ? ctx->hv[i] : nullptr,
                               dist_host ? ctx->hd[i] : nullptr, profile_host ? ctx->hp[i] : nullptr, st);
        if (rc) return rc;
        if (valid_host) CK(cudaMemcpyAsync(valid_host + off, ctx->hv[i], n, cudaMemcpyDeviceToHost, st));
        if (dist_host) CK(cudaMemcpyAsync(dist_host + off, ctx->hd[i], n * sizeof(double), cudaMemcpyDeviceToHost, st));
        if (profile_host)
            CK(cudaMemcpyAsync(profile_host + off * D, ctx->hp[i], n * D * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    for (int i = 0; i < 2; ++i)
        if (ctx->hs[i]) CK(cudaStreamSynchronize(ctx->hs[i]));
    for (int i = 0; i < 2; ++i) {
        const int rc = host_status(ctx, ctx->hs[i]);
        if (rc) return rc;
    }
    return RPM_OK;
}

int rpm_skeleton(rpm_ctx *ctx, int32_t robot_id, int32_t precision, const float *q_dev, int64_t num_configs,
                 double *points_dev, void *stream) {
    if (!ctx || (num_configs > 0 && (!q_dev || !points_dev))) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (robot_id < 0 || robot_id >= (int)ctx->robots.size()) return fail(RPM_ERR_INVALID, "unknown robot %d", robot_id);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    const RobotRec &r = ctx->robots[robot_id];
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    CK(launch_skeleton(precision, r.dev, r.desc.num_dofs, q_dev, num_configs, points_dev, (cudaStream_t)stream));
    return RPM_OK;
}

int rpm_last_stats(rpm_ctx *ctx, void *stream, rpm_check_stats *out) {
    if (!ctx || !out) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    std::memset(out, 0, sizeof *out);
    auto it = ctx->scratch.find(st);
    if (it == ctx->scratch.end()) return RPM_OK;
    CK(cudaStreamSynchronize(st));
    uint32_t cnt[4] = {0, 0, 0, 0};
    int32_t status = 0;
    CK(cudaMemcpy(cnt, it->second->counters, sizeof cnt, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&status, it->second->status, sizeof status, cudaMemcpyDeviceToHost));
    out->configs = it->second->last_configs;
    // configurations that used FP64: whole, or through their listed pairs
    out->rechecked = (int64_t)cnt[0] + std::min<int64_t>(cnt[2], (int64_t)it->second->pcfg_cap);
    out->overflow = cnt[1];
    out->device_status = status;
    return RPM_OK;
}

int rpm_ctx_set_timing(rpm_ctx *ctx, int enable) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    ctx->timing = enable != 0;
    return RPM_OK;
}

int rpm_last_timing(rpm_ctx *ctx, void *stream, float *bulk_ms, float *recheck_ms) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;
    auto it = ctx->scratch.find(st);
    if (it == ctx->scratch.end() || !it->second->timed) return fail(RPM_ERR_INVALID, "no timed check on this stream");
    Scratch *sc = it->second;
    CK(cudaEventSynchronize(sc->ev[2]));
    float a = 0.f, b = 0.f;
    CK(cudaEventElapsedTime(&a, sc->ev[0], sc->ev[1]));
    CK(cudaEventElapsedTime(&b, sc->ev[1], sc->ev[2]));
    if (bulk_ms) *bulk_ms = a;
    if (recheck_ms) *recheck_ms = b;
    return RPM_OK;
}

int rpm_probe_bounded_wait(rpm_ctx *ctx, uint32_t polls) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    if (polls < 1 || polls > kWaitLimit) return fail(RPM_ERR_INVALID, "polls must be 1 .. %u", kWaitLimit);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    int32_t *status = nullptr;
    CK(cudaMalloc(&status, sizeof(int32_t)));
    int32_t v = 0;
    cudaError_t e = cudaMemset(status, 0, sizeof(int32_t));
    if (e == cudaSuccess) e = launch_wait_probe(status, polls, 0);
    if (e == cudaSuccess) e = cudaMemcpy(&v, status, sizeof v, cudaMemcpyDeviceToHost);
    cudaFree(status);
    CK(e);
    if (v == kStatusTimeout) return fail(RPM_ERR_TIMEOUT, "a bounded device-side wait gave up after %u polls", polls);
    return fail(RPM_ERR_CUDA, "the wait probe did not report its timeout (status %d)", v);
}

int rpm_probe_fp32_peak(rpm_ctx *ctx, double *tflops) {
    if (!ctx || !tflops) return fail(RPM_ERR_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    float *buf = nullptr;
    const int blocks = ctx->num_sms * 8, threads = 256, iters = 4096;
    CK(cudaMalloc(&buf, (size_t)blocks * threads * sizeof(float)));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    double best = 0.0;
    for (int rep = 0; rep < 5; ++rep) {
        CK(cudaEventRecord(a, 0));
        CK(launch_ffma_probe(buf, blocks, threads, iters, 0));
        CK(cudaEventRecord(b, 0));
        CK(cudaEventSynchronize(b));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, a, b));
        const double flops = 2.0 * kProbeChains * (double)iters * blocks * threads;
        if (rep > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    *tflops = best;
    return RPM_OK;
}

int rpm_probe_primitives(rpm_ctx *ctx, int32_t precision, const int32_t *kind_dev, const float *a_dev,
                         const float *b_dev, const float *x_dev, const float *r_dev, int64_t n, double *value_dev,
                         uint8_t *settled_dev, void *stream) {
    if (!ctx || n < 0 || (n > 0 && (!kind_dev || !a_dev || !b_dev || !x_dev || !r_dev || !value_dev)))
        return fail(RPM_ERR_INVALID, "NULL argument");
    if (precision < RPM_PREC_FP64 || precision > RPM_PREC_FP32_REF) return fail(RPM_ERR_INVALID, "unknown precision %d", precision);
    if (precision == RPM_PREC_FP32_RECHECK && n > 0 && !settled_dev)
        return fail(RPM_ERR_INVALID, "the FP32 + recheck form needs settled_dev");
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (set_device(ctx)) return RPM_ERR_CUDA;
    ProbeParams p{};
    p.kind = kind_dev; p.a = a_dev; p.b = b_dev; p.x = x_dev; p.r = r_dev; p.n = n;
    p.nmd.eq = ctx->params.equality_threshold; p.nmd.maxd = ctx->params.max_distance;
    p.nmf.eq = (float)ctx->params.equality_threshold; p.nmf.maxd = (float)ctx->params.max_distance;
    p.value = value_dev;
    p.settled = settled_dev;
    cudaStream_t st = (cudaStream_t)stream;
    if (precision == RPM_PREC_FP32_RECHECK) {
        CK(launch_probe_fp32(p, st));
        CK(launch_probe_exact(0, p, true, st));   // the FP64 recheck of what the FP32 pass left open
    } else {
        CK(launch_probe_exact(precision == RPM_PREC_FP64 ? 0 : 1, p, false, st));
    }
    return RPM_OK;
}

int rpm_sync(rpm_ctx *ctx, void *stream) {
    if (!ctx) return fail(RPM_ERR_INVALID, "NULL context");
    cudaStream_t st = (cudaStream_t)stream;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if (set_device(ctx)) return RPM_ERR_CUDA;
    }
    CK(cudaStreamSynchronize(st));
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scratch.find(st);
    if (it != ctx->scratch.end()) {
        int32_t status = 0;
        CK(cudaMemcpy(&status, it->second->status, sizeof status, cudaMemcpyDeviceToHost));
        if (status) {
            cudaMemset(it->second->status, 0, sizeof(int32_t));
            return fail(RPM_ERR_TIMEOUT, "a bounded device-side wait gave up (status %d)", status);
        }
    }
    return RPM_OK;
}

}  // extern "C"
