// rpm_edges.cuh -- RealVectorSpace::isValid(q1, q2) (RealVectorSpace.cpp:261-275)
// for batches of edges with uneven discretisation.
//
// Edge e has n_e checks at q1 + (q2 - q1) * ((k / n_e * dist) / dist),
// k = n_e .. 1 (q2 first, q1 never), with dist = |q1 - q2| summed in index
// order and n_e = max(1, ceil(dist / step)) (step > 0) or the fixed
// NUM_INTERPOLATION_VALIDITY_CHECKS (step <= 0).  Every operation of the
// interpolation is an explicit round-to-nearest float op, so all arithmetic
// forms check exactly the same configurations as the CPU restatement.
//
// A launch takes the edges of up to kMaxSegs requests (segments), each with
// its own robot and scene; edges are numbered globally, segment-major, the
// lane-layout segments first.
//
// Work: the checks of all edges are flattened (edge-major, k descending) and
// taken 32 at a time by persistent warps from a global atomic counter.  Early
// exit: each edge keeps kmax, the largest colliding k found so far; a check
// with k <= kmax is skipped.  Every check with k above the final kmax still
// runs, so kmax ends as the first collision in the reference's order and the
// number of checks the reference evaluates is n_e - kmax + 1.
#pragma once
#include "rpm_check.cuh"
#include "rpm_launch.cuh"

namespace rpm {

constexpr int kEdgeScanBlock = 1024;   // edges per block of the count/scan pass

// One edge request of a launch: its robot and scene, its edges and outputs.
// Edges of all segments are numbered globally (segment-major); segment s
// holds the global edges [e0, e0 + seg.count).
struct EdgeSeg {
    Seg seg;                 // robot, scene rows; seg.q = q1 [E][D], seg.count = E, seg.valid = output
    const float *q2;         // [E][D]
    int32_t *checks_out;     // [E] checks in the reference's order (nullable)
    int64_t e0;              // first global edge
    float step;              // > 0: n_e = max(1, ceil(dist / step))
    int32_t num_checks;      // step <= 0: fixed count per edge
    int32_t D;
    int32_t pad;
};

struct EdgeParams {
    EdgeSeg segs[kMaxSegs];
    int32_t nseg;
    int32_t nseg_lane;       // segments [0, nseg_lane) run the lane layout, the rest the warp layout
    int64_t E;               // edges of all segments
    int32_t *n_e;            // [E] checks per edge
    int32_t *local;          // [E] exclusive offset within its block of kEdgeScanBlock edges
    int64_t *bprefix;        // [blocks + 1] exclusive prefix of block totals; [blocks] = total
    int32_t *kmax;           // [E] largest colliding k (0 = none)
    unsigned long long *work;    // [2] work counters of the lane- and warp-layout passes
    uint64_t *recheck;       // unsettled checks (FP32 form): edge << 20 | k
    uint32_t *recheck_count;
    uint32_t recheck_cap;
    uint32_t *overflow;
    uint32_t *counters;      // [4] zeroed by the count pass
    uint8_t *full;           // [E] edges whose unsettled checks did not fit the list: all rechecked in FP64
    int32_t *status;
    Num<double> nmd;
    Num<float> nmf;
    PairSink ps;             // FP32 pass -> pair-level FP64 recheck (records: seg = k, config = edge)
    int32_t wide_g;          // warp-per-check kernels: checks taken per warp
    int32_t streams;         // warp-per-check kernels: 1 = edge streams, 0 = flat checks
};

// Segment of global edge g (segments are few: a binary search over e0).
RPM_HD int edge_seg(const EdgeParams &P, int64_t g) {
    int lo = 0, hi = P.nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.segs[mid].e0 <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// First global edge of the warp-layout segments.
RPM_HD int64_t edge_split(const EdgeParams &P) {
    return P.nseg_lane < P.nseg ? P.segs[P.nseg_lane].e0 : P.E;
}

RPM_HD void edge_point(const float *a, const float *b, int D, float ratio, float *out) {
    for (int i = 0; i < D; ++i) out[i] = fadd(a[i], fmul(fadd(b[i], -a[i]), ratio));
}

// getNorm (RealVectorSpace.cpp:48-52) summed in index order, and the number
// of checks of the edge.
RPM_HD int edge_count(const float *a, const float *b, int D, float step, int fixed, float &dist) {
    float ss = 0.f;
    for (int i = 0; i < D; ++i) {
        const float df = fadd(a[i], -b[i]);
        ss = fadd(ss, fmul(df, df));
    }
    dist = sqrtf(ss);
    if (step > 0.f) {
        const float n = ceilf(dist / step);
        return n < 1.f ? 1 : (int)n;
    }
    return fixed;
}

// Interpolated configuration of check k (k = N..1) of an edge
// (RealVectorSpace.cpp:267-269 and interpolateEdge :75-88).
RPM_HD void edge_config(const float *a, const float *b, int D, int N, int k, float dist, float *out) {
    if (dist > 0.f) {
        const float stp = fmul((float)k / (float)N, dist);
        edge_point(a, b, D, stp / dist, out);
    } else {
        for (int i = 0; i < D; ++i) out[i] = b[i];
    }
}

// Endpoints and check count of global edge g of segment s.
struct EdgeGeom {
    const float *a, *b;
    int D, n;
    float dist;
};
RPM_HD EdgeGeom edge_geom(const EdgeParams &P, int s, int64_t g) {
    const EdgeSeg &es = P.segs[s];
    EdgeGeom r;
    r.D = es.D;
    r.a = es.seg.q + (g - es.e0) * es.D;
    r.b = es.q2 + (g - es.e0) * es.D;
    r.n = edge_count(r.a, r.b, r.D, es.step, es.num_checks, r.dist);
    return r;
}

// Views of a segment's robot and scene in global memory (launches of several
// segments read them through L1 instead of staging one scene per CTA).
template <typename T> RPM_HD ObsView<T> global_obs(const Seg &sg);
template <> RPM_HD ObsView<double> global_obs<double>(const Seg &sg) {
    return ObsView<double>{sg.obs_d, sg.obs_f + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
}
template <> RPM_HD ObsView<float> global_obs<float>(const Seg &sg) {
    return ObsView<float>{sg.obs_f, sg.obs_f + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
}

#ifdef __CUDACC__
// A check the FP32 pass could not settle through the pair recheck: recheck it
// whole in FP64, or, when that list is full, every check of its edge.
__device__ __forceinline__ void edge_recheck_whole(const EdgeParams &P, int64_t e, int k) {
    const uint32_t slot = atomicAdd(P.recheck_count, 1u);
    if (slot < P.recheck_cap) P.recheck[slot] = ((uint64_t)e << 20) | (uint64_t)k;
    else { atomicAdd(P.overflow, 1u); P.full[e] = 1; }
}

// Record the outcome of check k of edge e.
template <int MODE>
__device__ __forceinline__ void edge_outcome(const EdgeParams &P, int64_t e, int k, int st, int slot, uint8_t v) {
    if (MODE == 2) complete_record(&P.ps, slot, st, k, e, -1, 0x7fffffff);
    if (st == kFull) edge_recheck_whole(P, e, k);
    else if (st == kSettled && v == 0) atomicMax(&P.kmax[e], k);
}

// Flat offset of global edge e's first check (e = E: the total).
__device__ __forceinline__ int64_t flat_off(const EdgeParams &P, int64_t e) {
    if (e >= P.E) return P.bprefix[(P.E + kEdgeScanBlock - 1) / kEdgeScanBlock];
    return P.bprefix[e / kEdgeScanBlock] + P.local[e];
}

// Edge index of flat check 'idx': the last edge in [lo, hi] whose offset <= idx.
__device__ __forceinline__ int64_t edge_of_flat(const EdgeParams &P, int64_t idx, int64_t lo, int64_t hi) {
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (flat_off(P, mid) <= idx) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The persistent lane-per-check pass over the lane-layout segments.  rb_st /
// ob_st: the robot and scene staged in shared memory when the pass has one
// segment, else null (each segment read from global memory).  A warp's 32
// checks may span segments: they are checked one segment at a time.  The FP32
// pass (MODE 2) runs the order-free isValid driver (warp_check_any): a warp's
// checks are consecutive checks of one or a few edges, so its skeletons lie
// close together and its obstacle culling skips most obstacles; skel is the
// CTA's skeleton buffer (kThreads x 3 x (D + 1) floats for the largest D).
template <int MODE, typename T>
__device__ void edge_warps(const EdgeParams &P, const DevRobot *rb_st, const ObsView<T> *ob_st, const Num<T> &nm,
                           WarpShared<T> &sh, float *qbuf /* 32 x kMaxDof */, float *skel = nullptr) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t split = edge_split(P);
    const int64_t total = flat_off(P, split);
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(&P.work[0], 32ull);
        base = __shfl_sync(full, base, 0);
        if ((int64_t)base >= total) break;
        const int64_t idx = (int64_t)base + lane;
        bool active = idx < total;
        int64_t e = 0;
        int k = 0, s = 0;
        if (active) {
            e = edge_of_flat(P, idx, 0, split - 1);
            s = edge_seg(P, e);
            const int n = P.n_e[e];
            k = n - (int)(idx - flat_off(P, e));
            if (k <= *(volatile int32_t *)&P.kmax[e]) active = false;   // a check nearer q2 already collides
            if (active) {
                const EdgeGeom gm = edge_geom(P, s, e);
                edge_config(gm.a, gm.b, gm.D, n, k, gm.dist, qbuf + lane * kMaxDof);
            }
        }
        __syncwarp();
        unsigned todo = __ballot_sync(full, active);
        while (todo) {
            const int cur = __shfl_sync(full, s, __ffs(todo) - 1);
            const bool mine = active && s == cur;
            const unsigned m = __ballot_sync(full, mine);
            const DevRobot &rb = rb_st ? *rb_st : *P.segs[cur].seg.robot;
            const ObsView<T> ob = ob_st ? *ob_st : global_obs<T>(P.segs[cur].seg);
            const Want w{true, false, false};
            uint8_t v = 1;
            int slot = -1;
            int st;
            if constexpr (MODE == 2)
                st = warp_check_any<1, kThreads>(sh, skel, rb, ob, qbuf + lane * kMaxDof, mine, nm, &v, nullptr, &P.ps,
                                                 &slot);
            else
                st = warp_check<MODE, T, 1>(sh, rb, ob, qbuf + lane * kMaxDof, mine, nm, w, &v, nullptr, nullptr,
                                            nullptr, &slot);
            if (mine) edge_outcome<MODE>(P, e, k, st, slot, v);
            todo &= ~m;
            __syncwarp();
        }
    }
}
#endif

// Host-side launchers (rpm_exact.cu / rpm_fast.cu).
cudaError_t launch_edge_prep(const EdgeParams &p, cudaStream_t st);
cudaError_t launch_edges(int mode, const EdgeParams &p, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_edges_fp32(const EdgeParams &p, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_edge_recheck_final(const EdgeParams &p, int grid, bool pairs, cudaStream_t st);
cudaError_t launch_edges_wide(int mode, const EdgeParams &p, int grid, size_t smem, cudaStream_t st);
cudaError_t launch_edges_wide_fp32(const EdgeParams &p, int grid, size_t smem, cudaStream_t st);

}  // namespace rpm
