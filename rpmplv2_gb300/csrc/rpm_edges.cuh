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
// Work: the checks of all edges are flattened (edge-major, k descending) and
// taken 32 at a time by persistent warps from a global atomic counter.  Early
// exit: each edge keeps kmax, the largest colliding k found so far; a check
// with k <= kmax is skipped.  Every check with k above the final kmax still
// runs, so kmax ends as the first collision in the reference's order and the
// number of checks the reference evaluates is n_e - kmax + 1.
#pragma once
#include "rpm_check.cuh"

namespace rpm {

constexpr int kEdgeScanBlock = 1024;   // edges per block of the count/scan pass

struct EdgeParams {
    Seg seg;                 // robot, scene rows, n, n_pad (q/count/outputs unused)
    const float *q1, *q2;    // [E][D]
    int64_t E;
    float step;              // > 0: n_e = max(1, ceil(dist / step))
    int32_t num_checks;      // step <= 0: fixed count per edge
    int32_t *n_e;            // [E] checks per edge
    int32_t *local;          // [E] exclusive offset within its block of kEdgeScanBlock edges
    int64_t *bprefix;        // [blocks + 1] exclusive prefix of block totals; [blocks] = total
    int32_t *kmax;           // [E] largest colliding k (0 = none)
    unsigned long long *work;    // flat-check work counter
    uint64_t *recheck;       // unsettled checks (FP32 form): edge << 20 | k
    uint32_t *recheck_count;
    uint32_t recheck_cap;
    uint32_t *overflow;
    uint8_t *full;           // [E] edges whose unsettled checks did not fit the list: all rechecked in FP64
    uint8_t *valid;          // [E] output
    int32_t *checks_out;     // [E] checks in the reference's order (nullable)
    int32_t *status;
    Num<double> nmd;
    Num<float> nmf;
    PairSink ps;             // FP32 pass -> pair-level FP64 recheck (records: seg = k, config = edge)
    int32_t wide_g;          // warp-per-check kernels: checks taken per warp
    int32_t streams;         // warp-per-check kernels: 1 = edge streams, 0 = flat checks
};

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

// Edge index of flat check 'idx': the last edge whose global offset <= idx.
__device__ __forceinline__ int64_t edge_of_flat(const EdgeParams &P, int64_t idx) {
    int64_t lo = 0, hi = P.E - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        const int64_t off = P.bprefix[mid / kEdgeScanBlock] + P.local[mid];
        if (off <= idx) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The persistent edge kernel body for one arithmetic form.
template <int MODE, typename T>
__device__ void edge_warps(const EdgeParams &P, const DevRobot &rb, const ObsView<T> &ob, const Num<T> &nm,
                           WarpShared<T> &sh, float *qbuf /* 32 x kMaxDof */) {
    const int lane = threadIdx.x & 31;
    const int D = rb.D;
    const int64_t total = P.bprefix[(P.E + kEdgeScanBlock - 1) / kEdgeScanBlock];
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(P.work, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((int64_t)base >= total) break;
        const int64_t idx = (int64_t)base + lane;
        bool active = idx < total;
        int64_t e = 0;
        int k = 0;
        if (active) {
            e = edge_of_flat(P, idx);
            const int64_t first = P.bprefix[e / kEdgeScanBlock] + P.local[e];
            const int n = P.n_e[e];
            k = n - (int)(idx - first);
            if (k <= *(volatile int32_t *)&P.kmax[e]) active = false;   // a check nearer q2 already collides
            if (active) {
                float dist;
                edge_count(P.q1 + e * D, P.q2 + e * D, D, P.step, P.num_checks, dist);
                edge_config(P.q1 + e * D, P.q2 + e * D, D, n, k, dist, qbuf + lane * kMaxDof);
            }
        }
        __syncwarp();
        const Want w{true, false, false};
        uint8_t v = 1;
        int slot = -1;
        const int st = warp_check<MODE, T>(sh, rb, ob, qbuf + lane * kMaxDof, active, nm, w, &v, nullptr, nullptr,
                                           MODE == 2 ? &P.ps : nullptr, &slot);
        if (active) edge_outcome<MODE>(P, e, k, st, slot, v);
        __syncwarp();
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
