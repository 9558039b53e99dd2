// rpm_ctx_impl.cuh -- internal state of a context (robots, versioned scenes,
// per-stream scratch) shared by the C ABI translation units.  Not part of the
// public interface.
#pragma once
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rpm_edges.cuh"
#include "rpm_launch.cuh"
#include "rpm_wide.cuh"

namespace rpm {
namespace impl {

extern thread_local std::string g_err;

inline int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(x)                                                                                                \
    do {                                                                                                     \
        cudaError_t e_ = (x);                                                                                \
        if (e_ != cudaSuccess) return ::rpm::impl::fail(RPM_ERR_CUDA, "%s: %s", #x, cudaGetErrorString(e_)); \
    } while (0)

constexpr int kRing = 8;   // versions kept per scene

struct RobotRec {
    rpm_robot_desc desc;
    DevRobot *dev = nullptr;
};

// One version of a scene's obstacles in device memory (one allocation):
//   f [8][n_pad], d [7][n_pad]  rows in the caller's order
//   sf [8][ns], sd [7][ns]      spatially sorted copy (row 7 of sf: original index | ground bit)
//   blk [nb][8]                 bounds and tolerance range of each block of 32 sorted slots
//   perm [ns]                   original index of each sorted slot (-1 = padding)
struct SceneBuf {
    void *mem = nullptr;
    float *f = nullptr;
    double *d = nullptr;
    float *sf = nullptr;
    double *sd = nullptr;
    float *blk = nullptr;
    int32_t *perm = nullptr;
    std::vector<cudaEvent_t> users;   // checks that may still read this buffer
    cudaEvent_t ready = nullptr;      // end of the incremental update that wrote this version
    bool pending = false;             // 'ready' must be waited on before reading
};

// One scene version written by the fused update kernel: the current
// version's rows and permutation copied, m updated rows ([m][7]: index as
// bits, six AABB values) scattered in, the sorted copy and leaf bounds rebuilt.
struct UpdDesc {
    const float *src_f;
    const double *src_d;
    const int32_t *src_perm;
    float *f;
    double *d;
    float *sf;
    double *sd;
    float *blk;
    int32_t *perm;
    const float *rows;   // pinned host memory, read in place by the kernel
    int32_t n_pad, ns, m, pad;
};

struct SceneRec {
    int robot = 0;
    int n = 0, n_pad = 16;
    int ns = 32, nb = 1;            // sorted slots and blocks
    std::vector<int32_t> perm;      // [ns] original index per sorted slot, -1 = padding
    std::vector<float> aabb, tol;
    std::vector<uint8_t> flags;
    int cur = 0;
    SceneBuf bufs[kRing];
    uint64_t version = 0;
};

struct Scratch {
    uint64_t *recheck = nullptr;
    size_t cap = 0;
    // pair-level recheck lists (see PairSink)
    size_t pcfg_cap = 0, ppair_cap = 0;
    uint64_t *pairs = nullptr;
    uint32_t *pkey = nullptr, *porder = nullptr;   // evaluation order of the pairs (ppair_cap each)
    uint32_t *phist = nullptr;                     // kPairHist
    PairCfg *pcfgs = nullptr;
    double *pskel = nullptr;
    PairAcc *pacc = nullptr;
    // [0] whole-configuration recheck count, [1] edge recheck overflow,
    // [2] pair-recheck records, [3] listed pairs
    uint32_t *counters = nullptr;
    int32_t *status = nullptr;
    int64_t last_configs = 0;
    rpm_tile_shape last_shape{0, 0, 0, 0.f};   // shape of the last main launch on this stream
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};   // bulk start, bulk end / recheck start, recheck end
    bool timed = false, had_recheck = false;
    // edge checks
    size_t ecap = 0;
    int32_t *n_e = nullptr, *local = nullptr, *kmax = nullptr;
    int64_t *bprefix = nullptr;
    uint8_t *full = nullptr;
    unsigned long long *work = nullptr;
    uint64_t *erecheck = nullptr;
    size_t erecheck_cap = 0;
    // check order of a large FP32 lane-layout batch (binned configurations),
    // allocated with the recheck lists (cap entries)
    int32_t *perm = nullptr;
    size_t perm_cap = 0;
    int32_t *bins = nullptr;   // [2][kConfigBins]: counts, then running offsets
    // the planner calls' working memory (a DRGBT step's nearest points and
    // distances), reused in stream order; grown only between calls
    void *aux = nullptr;
    size_t aux_cap = 0;
    // cached CUDA graphs of edge calls, keyed by their arguments
    struct Graph { std::vector<uint64_t> key; cudaGraphExec_t exec; };
    std::vector<Graph> graphs;
};

// One segment of a launch: a scene and its configurations / outputs.
struct SegReq {
    SceneRec *scene;
    const float *q;
    int64_t count;
    uint8_t *valid;
    double *dist;
    float *profile;
    int32_t wide = -1;   // layout decided for the segment (-1: not yet)
    const int32_t *perm = nullptr;   // check order (FP32 lane layout), nullable
};

// Tile-shape table of the autotuner: the launch shape to use for a (robot,
// scene size, batch size, arithmetic form, outputs, configurations or edges)
// bucket.  Sizes are bucketed by ceil(log2).
struct TuneKey {
    int32_t robot_kind, dofs, obstacles_log2, count_log2, prec, outputs, edges;
    bool operator<(const TuneKey &o) const {
        const int32_t a[7] = {robot_kind, dofs, obstacles_log2, count_log2, prec, outputs, edges};
        const int32_t b[7] = {o.robot_kind, o.dofs, o.obstacles_log2, o.count_log2, o.prec, o.outputs, o.edges};
        for (int i = 0; i < 7; ++i)
            if (a[i] != b[i]) return a[i] < b[i];
        return false;
    }
};

}  // namespace impl
}  // namespace rpm

struct rpm_ctx {
    int device = 0;
    int num_sms = 0;
    rpm_params params{1e-4, 1000.0};
    std::mutex mu;
    std::vector<rpm::impl::RobotRec> robots;
    std::map<int, rpm::impl::SceneRec *> scenes;
    int next_scene = 0;
    std::map<cudaStream_t, rpm::impl::Scratch *> scratch;
    std::vector<cudaEvent_t> event_pool;
    cudaStream_t upd_stream = nullptr;    // incremental scene updates
    // pinned staging ring of incremental updates (descriptors and rows, read in
    // place by the update kernel); a slot is reused once its kernel has run
    static constexpr int kUpdRing = 4;
    unsigned char *upd_stage[kUpdRing] = {};
    size_t upd_cap[kUpdRing] = {};
    cudaEvent_t upd_done[kUpdRing] = {};
    int upd_next = 0;
    // host-buffer pipeline
    cudaStream_t hs[2] = {nullptr, nullptr};
    float *hq[2] = {nullptr, nullptr};
    uint8_t *hv[2] = {nullptr, nullptr};
    double *hd[2] = {nullptr, nullptr};
    float *hp[2] = {nullptr, nullptr};
    size_t hcap_cfg = 0, hcap_qf = 0, hcap_prof = 0;   // staging capacity: configurations, q floats, profile floats
    bool timing = false;
    bool use_graphs = false;
    int layout = RPM_LAYOUT_AUTO;    // lane- or warp-per-configuration checks
    std::map<rpm::impl::TuneKey, rpm_tile_shape> tune;   // autotuned tile shapes
    uint64_t tune_epoch = 0;                              // bumped on every change (graph cache key)
    // degrees of freedom per scene, readable without 'mu' (the server's submit path)
    std::mutex dof_mu;
    std::map<int, int> scene_dofs;
};

namespace rpm {
namespace impl {
// helpers defined in rpm_api.cu; callers hold ctx->mu
int set_device(rpm_ctx *ctx);
cudaEvent_t get_event(rpm_ctx *ctx);
void prune_users(rpm_ctx *ctx, SceneBuf &b);
void wait_users(rpm_ctx *ctx, SceneBuf &b);
// Make stream 'st' wait (on the device) for every check still reading 'b'.
void stream_wait_users(rpm_ctx *ctx, SceneBuf &b, cudaStream_t st);
int scene_dofs(rpm_ctx *ctx, int scene_id);   // -1: unknown scene
int get_scratch(rpm_ctx *ctx, cudaStream_t st, int64_t need, Scratch **out);
void free_scratch(Scratch *sc);   // stream work using it must be complete
SceneRec *find_scene(rpm_ctx *ctx, int id);
int enqueue_segments(rpm_ctx *ctx, int prec, const std::vector<SegReq> &reqs, cudaStream_t st);
int edge_scratch(rpm_ctx *ctx, Scratch *sc, int64_t E, cudaStream_t st);
// One edge request of a batched edge launch.
struct EdgeReq {
    SceneRec *scene;
    const float *q1, *q2;
    int64_t E;
    float step;
    int32_t num_checks;
    uint8_t *valid;
    int32_t *checks;
};
int enqueue_edge_batch(rpm_ctx *ctx, Scratch *sc, int prec, const std::vector<EdgeReq> &reqs, int ctas_per_sm,
                       cudaStream_t st);
int enqueue_edges(rpm_ctx *ctx, Scratch *sc, SceneRec *s, int prec, const float *q1, const float *q2, int64_t E,
                  float step, int32_t num_checks, uint8_t *valid, int32_t *checks, int ctas_per_sm, cudaStream_t st);
// Incremental updates of several scenes at once: one kernel launch writes the
// next version of every scene (UpdDesc).  Caller holds ctx->mu.
struct SceneUpd {
    SceneRec *s;
    const int32_t *idx;
    const float *aabb;   // m x 6
    int32_t m;
};
int scene_update_many(rpm_ctx *ctx, const std::vector<SceneUpd> &u);
int scene_update(rpm_ctx *ctx, SceneRec *s, const int32_t *idx, const float *aabb, int32_t m);
cudaError_t launch_scene_update_many(const UpdDesc *descs, int count, cudaStream_t st);
// The DRGBT steps with ctx->mu held (rpm_reached_states, rpm_motion_validity).
int reached_states_locked(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_current_dev,
                          const float *horizon_dev, int64_t horizon_size, const rpm_spine_params *params,
                          float *q_reached_dev, int32_t *status_dev, double *dist_dev, cudaStream_t st);
int motion_validity_locked(rpm_ctx *ctx, int32_t scene_id, int32_t precision, const float *q_prev_dev,
                           const float *q_cur_dev, int64_t num_motions, const rpm_moving_box *boxes, int32_t num_boxes,
                           float max_iter_time, int32_t num_points, uint8_t *valid_dev, int32_t *checks_dev,
                           cudaStream_t st);
// Spatially sorted copy: Morton order of the obstacle centres (fixed for the
// scene's lifetime), its size, and the kernel that rebuilds it in a version.
void sorted_layout(SceneRec &s);
size_t scene_bytes(const SceneRec &s);
void bind_scene_buf(const SceneRec &s, SceneBuf &b);
cudaError_t launch_scene_sort(const SceneRec &s, const SceneBuf &b, cudaStream_t st);
}  // namespace impl
}  // namespace rpm
