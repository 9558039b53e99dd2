// rpm_exact.cu -- exact forms: FP64 ("plain form"), the reference's own FP32
// numerics, and the FP64 recheck of configurations the FP32 pass could not
// settle.  Built with --fmad=false: no multiply-add is contracted, so every
// operation rounds as the CPU restatement's does.
#include <type_traits>

#include "rpm_check.cuh"
#include "rpm_edges.cuh"
#include "rpm_launch.cuh"
#include "rpm_nearest.cuh"
#include "rpm_spine.cuh"
#include "rpm_wide.cuh"

namespace rpm {

size_t smem_bytes(int mode, int n_pad) {
    size_t rb = sizeof(DevRobot);
    if (mode == RPM_PREC_FP64) return rb + (size_t)kDRows * n_pad * sizeof(double) + (size_t)kFRows * n_pad * sizeof(float);
    return rb + (size_t)kFRows * n_pad * sizeof(float);
}

// Stage the segment's robot and obstacle rows in shared memory (bulk async
// copies on one mbarrier).  Returns false if the bounded wait gave up.
template <int MODE>
__device__ __forceinline__ bool stage(const Seg &sg, unsigned char *smem, uint64_t *bar, int32_t *status) {
    if (threadIdx.x == 0) {
        const uint32_t rb = (uint32_t)sizeof(DevRobot);
        if (MODE == 0) {   // FP64 rows, then the float rows (ground row, float pre-test)
            const uint32_t rows = (uint32_t)(kDRows * sg.n_pad * sizeof(double));
            const uint32_t frows = (uint32_t)(kFRows * sg.n_pad * sizeof(float));
            bulk_expect(bar, rb + rows + frows);
            bulk_copy(bar, smem, sg.robot, rb);
            bulk_copy(bar, smem + rb, sg.obs_d, rows);
            bulk_copy(bar, smem + rb + rows, sg.obs_f, frows);
        } else {
            const uint32_t rows = (uint32_t)(kFRows * sg.n_pad * sizeof(float));
            bulk_expect(bar, rb + rows);
            bulk_copy(bar, smem, sg.robot, rb);
            bulk_copy(bar, smem + rb, sg.obs_f, rows);
        }
    }
    return bulk_wait(bar, 0, status);
}

__device__ __forceinline__ int find_seg(const KParams &P) {
    int k = 0;
    while (k + 1 < P.nseg && P.segs[k + 1].first_block <= (int64_t)blockIdx.x) ++k;
    return k;
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_check_exact(const __grid_constant__ KParams P) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ WarpShared<T> wsh[kThreads / 32];
    const int s = find_seg(P);
    const Seg &sg = P.segs[s];
    bulk_init(&bar);
    if (!stage<MODE>(sg, smem, &bar, P.status)) return;
    const DevRobot &rb = *reinterpret_cast<const DevRobot *>(smem);
    const T *rows = reinterpret_cast<const T *>(smem + sizeof(DevRobot));
    const float *frows = (MODE == 0) ? reinterpret_cast<const float *>(smem + sizeof(DevRobot) + kDRows * sg.n_pad * sizeof(double))
                                     : reinterpret_cast<const float *>(rows);
    const float *ground = frows + (size_t)kRowGround * sg.n_pad;
    const int64_t c = (int64_t)(blockIdx.x - sg.first_block) * kThreads + threadIdx.x;
    const int64_t warp0 = c - (threadIdx.x & 31);
    if (warp0 >= sg.count) return;   // whole warp idle
    const bool active = c < sg.count;
    ObsView<T> ob{rows, ground, sg.n, sg.n_pad, MODE == 0 ? frows : nullptr};
    const Want w{sg.valid != nullptr, sg.dist != nullptr, sg.profile != nullptr};
    const int D = rb.D;
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    warp_check<MODE, T>(wsh[threadIdx.x >> 5], rb, ob, sg.q + c * D, active, nm, w,
                        (w.valid && active) ? sg.valid + c : nullptr, (w.dist && active) ? sg.dist + c : nullptr,
                        (w.profile && active) ? sg.profile + c * D : nullptr);
}

// Warp-per-configuration form (rpm_wide.cuh): G configurations per warp.
template <int MODE>
__global__ void __launch_bounds__(kWideThreads, MODE == 0 ? 1 : 2) k_check_wide(const __grid_constant__ KParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ MultiState<typename std::conditional<MODE == 0, double, float>::type> ms[kWideWarps];
    const int s = find_seg(P);
    bulk_init(&bar);
    wide_kernel_body<MODE>(P, smem, &bar, ms, s);
}

// FP64 recomputation of the configurations listed by the FP32 pass, one warp
// per configuration.  Reads robot and obstacles from global memory (the list
// mixes segments).
__global__ void __launch_bounds__(kThreads) k_recheck(const __grid_constant__ KParams P) {
    const uint32_t n = *P.recheck_count;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t k = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); k < n; k += warps) {
        const uint64_t e = P.recheck[k];
        const int s = (int)(e >> 40);
        const int64_t c = (int64_t)(e & ((1ull << 40) - 1));
        if (s >= P.nseg) continue;
        const Seg &sg = P.segs[s];
        if (c >= sg.count) continue;
        ObsView<double> ob{sg.obs_d, sg.obs_f + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
        const Want w{sg.valid != nullptr, sg.dist != nullptr, sg.profile != nullptr};
        const int D = sg.robot->D;
        config_exact_warp<0, double>(*sg.robot, ob, sg.q + c * D, P.nmd, w, w.valid ? sg.valid + c : nullptr,
                                     w.dist ? sg.dist + c : nullptr, w.profile ? sg.profile + c * D : nullptr);
    }
}

// ---------------------------------------------------------- pair recheck --
// FP64 skeleton of one configuration; its accumulators reset.
__device__ __forceinline__ void pair_skel_one(const DevRobot &rb, const float *q, double *out, PairAcc &a) {
    SkelWalker<0> sw;
    sw.begin();
    for (int i = 0; i <= rb.D; ++i) sw.point(rb, q, i, out + 3 * i);
    for (int i = 0; i < kMaxDof; ++i) {
        a.lkey[i] = 0x7fffffff;
        a.hkey[i] = ~0ull;
    }
    a.dkey = 0x7fffffffffffffffLL;
    a.coll = 0;
}

// The reference's FP64 tree for one listed pair, folded into the record's
// accumulators.
__device__ __forceinline__ void pair_eval_one(const DevRobot &rb, const ObsView<double> &ob, const Num<double> &nmd,
                                              const double *skel, int link, int j, int kind, PairAcc &a) {
    const double *A = skel + 3 * link;
    const double *B = A + 3;
    double o[6];
    ob.box(j, o);
    if (kind == 0) {
        if (coll_box_call<double, ExactPol>(nmd, A, B, rb.radius_d[link], rb.rnew_d[link], o).v) atomicOr(&a.coll, 1);
    } else {
        double d = capsule_box_call<double, ExactPol>(nmd, A, B, rb.radius_d[link], o).v;
        if (d > ob.tol(j)) d = nmd.maxd;   // :367-368
        if (d == d) {
            const float f = (float)d;
            atomicMin(&a.lkey[link], Key<float>::of(f));
            atomicMin(&a.dkey, Key<double>::of(d));
            if (d <= 0.0) atomicMin(&a.hkey[link], ((unsigned long long)j << 32) | __float_as_uint(f));
        }
    }
}

__device__ __forceinline__ bool decode_pair(const PairSink &ps, uint32_t k, uint32_t ncfg, uint32_t &slot, int &link,
                                            int &j, int &kind) {
    const uint64_t e = ps.pairs[k];
    slot = (uint32_t)(e >> 17);
    link = (int)((e >> 12) & 31u);
    j = (int)((e >> 1) & 2047u);
    kind = (int)(e & 1u);
    return slot < ncfg && ps.cfgs[slot].status == kPairs;
}

// FP64 skeleton with the whole warp: the joints' sines and cosines in
// parallel (warp_sincos: the taylor_sincos values), then the chain spread
// over the warp (skel_coop).
__device__ __forceinline__ void pair_skel_warp(const DevRobot &rb, const float *q, double *out, PairAcc &a,
                                               double *sc) {
    const int lane = threadIdx.x & 31;
    warp_sincos(q, rb.D, sc);
    a.lkey[lane] = 0x7fffffff;
    a.hkey[lane] = ~0ull;
    if (lane == 0) {
        a.dkey = 0x7fffffffffffffffLL;
        a.coll = 0;
    }
    __syncwarp();
    skel_coop<0, double>(rb, sc, out);
    __syncwarp();
}

// Records up to this many times the warps are skeletonised a warp each, in
// rounds, consecutive records on different CTAs so that they run on different
// SMs (a warp's FP64 chain is latency-bound); beyond, one thread each.
constexpr uint32_t kSkelWarpRounds = 2;

// 1. FP64 skeleton of each recorded configuration.
__global__ void k_pair_skel(const __grid_constant__ KParams P) {
    __shared__ double sc[kThreads / 32][2 * kMaxDof];
    if (P.ps.hist && blockIdx.x == 0)   // for k_pair_key, which runs next
        for (uint32_t i = threadIdx.x; i < kPairHist; i += blockDim.x) P.ps.hist[i] = 0;
    const uint32_t n = min(*P.ps.cfg_count, P.ps.cfg_cap);
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    if (n <= kSkelWarpRounds * warps) {   // a warp each, consecutive records on different SMs
        for (uint32_t k = (threadIdx.x / 32) * gridDim.x + blockIdx.x; k < n; k += warps) {
            const PairCfg c = P.ps.cfgs[k];
            if (c.status != kPairs) continue;
            const Seg &sg = P.segs[c.seg];
            const DevRobot &rb = *sg.robot;
            pair_skel_warp(rb, sg.q + c.config * rb.D, P.ps.skel + (size_t)k * (kMaxDof + 1) * 3, P.ps.acc[k],
                           sc[threadIdx.x / 32]);
        }
        return;
    }
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const PairCfg c = P.ps.cfgs[k];
        if (c.status != kPairs) continue;
        const Seg &sg = P.segs[c.seg];
        const DevRobot &rb = *sg.robot;
        pair_skel_one(rb, sg.q + c.config * rb.D, P.ps.skel + (size_t)k * (kMaxDof + 1) * 3, P.ps.acc[k]);
    }
}

// Listed pair k of run r: each warp takes runs of `per` consecutive pairs,
// one per lane, the runs dealt to the warps so that consecutive runs land on
// different CTAs.  `per` is the fewest pairs per warp that covers the list
// (at most 32), so every SM gets work and a warp diverges over a few pairs
// only: each divergent path of an FP64 tree issues its own FP64
// instructions, and a lone warp's FP64 chain is latency-bound.
struct PairRuns {
    uint32_t per, lane, first, stride;
    __device__ PairRuns(uint32_t n) {
        const uint32_t warps = gridDim.x * (blockDim.x / 32);
        per = min(32u, max(1u, (n + warps - 1) / warps));
        lane = threadIdx.x & 31;
        first = ((threadIdx.x / 32) * gridDim.x + blockIdx.x) * per + lane;
        stride = warps * per;
    }
    __device__ bool active() const { return lane < per; }
};

// 2a. Sort key of each listed pair (kPairKeys), counted per key; the last CTA
// to finish turns the counts into bucket offsets.  The pairs of a warp then
// mostly take one path through the FP64 trees, where the list order mixes
// the two kinds and every region of both.
__global__ void k_pair_key(const __grid_constant__ KParams P) {
    __shared__ bool last;
    __shared__ uint32_t wsum[kThreads / 32];
    const uint32_t n = min(*P.ps.pair_count, P.ps.pair_cap);
    const uint32_t ncfg = min(*P.ps.cfg_count, P.ps.cfg_cap);
    uint32_t *hist = P.ps.hist;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        uint32_t slot, key = kPairKeys - 1;
        int link, j, kind;
        if (decode_pair(P.ps, k, ncfg, slot, link, j, kind)) {
            const Seg &sg = P.segs[P.ps.cfgs[slot].seg];
            const double *A = P.ps.skel + (size_t)slot * (kMaxDof + 1) * 3 + 3 * link, *B = A + 3;
            uint32_t ra = 0, rb = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const double lo = sg.obs_d[a * sg.n_pad + j], hi = sg.obs_d[(a + 3) * sg.n_pad + j];
                ra = ra * 3 + (A[a] < lo ? 0u : (A[a] > hi ? 2u : 1u));
                rb = rb * 3 + (B[a] < lo ? 0u : (B[a] > hi ? 2u : 1u));
            }
            key = (uint32_t)kind * 729u + ra * 27u + rb;
        }
        P.ps.key[k] = key;
        atomicAdd(&hist[key], 1u);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&hist[2 * kPairKeys], 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // exclusive scan of the counts: kPer consecutive keys per thread, then
    // the threads' sums across the CTA
    constexpr int kPer = (int)((kPairKeys + kThreads - 1) / kThreads);
    uint32_t c[kPer], sum = 0;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const uint32_t b = threadIdx.x * kPer + i;
        c[i] = b < kPairKeys ? __ldcg(&hist[b]) : 0u;
        sum += c[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    uint32_t run = x - sum;
    for (int w = 0; w < warp; ++w) run += wsum[w];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const uint32_t b = threadIdx.x * kPer + i;
        if (b < kPairKeys) hist[kPairKeys + b] = run;
        run += c[i];
    }
}

// 2b. The pairs in key order.
__global__ void k_pair_scatter(const __grid_constant__ KParams P) {
    const uint32_t n = min(*P.ps.pair_count, P.ps.pair_cap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        P.ps.order[atomicAdd(&P.ps.hist[kPairKeys + P.ps.key[k]], 1u)] = k;
}

// 2. The reference's FP64 tree for each listed pair on the FP64 skeleton
// (pairs of configurations that ended settled, or that were routed to the
// whole-configuration recheck, belong to records not completed with kPairs
// and are skipped).
// Four CTAs per SM (128 registers, a few spilled), so its grid of four per SM
// is one resident wave (measured: the recheck round 0.179 -> 0.177 ms).
__global__ void __launch_bounds__(kThreads, 4) k_pair_eval(const __grid_constant__ KParams P) {
    const uint32_t n = min(*P.ps.pair_count, P.ps.pair_cap);
    const uint32_t ncfg = min(*P.ps.cfg_count, P.ps.cfg_cap);
    const PairRuns run(n);
    if (!run.active()) return;
    for (uint32_t k = run.first; k < n; k += run.stride) {
        uint32_t slot;
        int link, j, kind;
        if (!decode_pair(P.ps, P.ps.order ? P.ps.order[k] : k, ncfg, slot, link, j, kind)) continue;
        const Seg &sg = P.segs[P.ps.cfgs[slot].seg];
        ObsView<double> ob{sg.obs_d, sg.obs_f + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
        pair_eval_one(*sg.robot, ob, P.nmd, P.ps.skel + (size_t)slot * (kMaxDof + 1) * 3, link, j, kind, P.ps.acc[slot]);
    }
}

// Edge checks: the same three steps; a record is check k (seg) of an edge
// (config), and an FP64 collision raises the edge's largest colliding k.
__global__ void k_edge_pair_skel(const __grid_constant__ EdgeParams P) {
    __shared__ double sc[kThreads / 32][2 * kMaxDof];
    __shared__ float qs[kThreads / 32][kMaxDof];
    const uint32_t n = min(*P.ps.cfg_count, P.ps.cfg_cap);
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    if (n <= kSkelWarpRounds * warps) {   // a warp each, consecutive records on different SMs
        const int w = threadIdx.x / 32;
        for (uint32_t k = (threadIdx.x / 32) * gridDim.x + blockIdx.x; k < n; k += warps) {
            const PairCfg c = P.ps.cfgs[k];
            if (c.status != kPairs) continue;
            const int s = edge_seg(P, c.config);
            __syncwarp();
            if ((threadIdx.x & 31) == 0) {
                const EdgeGeom gm = edge_geom(P, s, c.config);
                edge_config(gm.a, gm.b, gm.D, gm.n, c.seg, gm.dist, qs[w]);
            }
            __syncwarp();
            pair_skel_warp(*P.segs[s].seg.robot, qs[w], P.ps.skel + (size_t)k * (kMaxDof + 1) * 3, P.ps.acc[k],
                           sc[w]);
        }
        return;
    }
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const PairCfg c = P.ps.cfgs[k];
        if (c.status != kPairs) continue;
        const int s = edge_seg(P, c.config);
        const EdgeGeom gm = edge_geom(P, s, c.config);
        float q[kMaxDof];
        edge_config(gm.a, gm.b, gm.D, gm.n, c.seg, gm.dist, q);
        pair_skel_one(*P.segs[s].seg.robot, q, P.ps.skel + (size_t)k * (kMaxDof + 1) * 3, P.ps.acc[k]);
    }
}

__global__ void k_edge_pair_eval(const __grid_constant__ EdgeParams P) {
    const uint32_t n = min(*P.ps.pair_count, P.ps.pair_cap);
    const uint32_t ncfg = min(*P.ps.cfg_count, P.ps.cfg_cap);
    const PairRuns run(n);
    if (!run.active()) return;
    for (uint32_t k = run.first; k < n; k += run.stride) {
        uint32_t slot;
        int link, j, kind;
        if (!decode_pair(P.ps, k, ncfg, slot, link, j, kind)) continue;
        const Seg &sg = P.segs[edge_seg(P, P.ps.cfgs[slot].config)].seg;
        pair_eval_one(*sg.robot, global_obs<double>(sg), P.nmd, P.ps.skel + (size_t)slot * (kMaxDof + 1) * 3, link, j,
                      kind, P.ps.acc[slot]);
    }
}

__global__ void k_edge_pair_fold(const __grid_constant__ EdgeParams P) {
    const uint32_t n = min(*P.ps.cfg_count, P.ps.cfg_cap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const PairCfg c = P.ps.cfgs[k];
        if (c.status == kPairs && P.ps.acc[k].coll) atomicMax(&P.kmax[c.config], c.seg);
    }
}

// Warp-per-check edge pass (rpm_wide.cuh).
template <int MODE, bool MULTI>
__global__ void __launch_bounds__(kWideThreads, MODE == 0 ? 1 : 2) k_edges_wide(const __grid_constant__ EdgeParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ MultiState<typename std::conditional<MODE == 0, double, float>::type> ms[kWideWarps];
    bulk_init(&bar);
    edge_wide_body<MODE, MULTI>(P, smem, &bar, ms);
}

// 3. Fold per recorded configuration in the reference's link order: the
// first link holding a hit (settled FP32 or FP64) ends the scan; its profile
// entry is the hit with the lowest obstacle index; earlier links take the
// smaller of the settled FP32 minimum and the FP64 minimum.
__global__ void k_pair_fold(const __grid_constant__ KParams P) {
    const uint32_t n = min(*P.ps.cfg_count, P.ps.cfg_cap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const PairCfg c = P.ps.cfgs[k];
        if (c.status != kPairs) continue;
        const Seg &sg = P.segs[c.seg];
        const PairAcc &a = P.ps.acc[k];
        const int L = sg.robot->D;
        const int64_t q = c.config;
        if (sg.valid && a.coll) sg.valid[q] = 0;
        if (!sg.dist && !sg.profile) continue;
        float *prof = sg.profile ? sg.profile + q * L : nullptr;
        int first = -1;
        for (int i = 0; i < L; ++i) {
            const unsigned long long h = a.hkey[i];
            if (i == c.hit_link) {
                if (prof && h != ~0ull && (int)(h >> 32) < c.hit_j) prof[i] = __uint_as_float((uint32_t)h);
                first = i;
                break;
            }
            if (h != ~0ull) {
                if (prof) prof[i] = __uint_as_float((uint32_t)h);
                first = i;
                break;
            }
            if (prof && a.lkey[i] != 0x7fffffff) {
                const float v = Key<float>::value(a.lkey[i]);
                prof[i] = smin(prof[i], v);
            }
        }
        if (prof && first >= 0)
            for (int i = first + 1; i < L; ++i) prof[i] = 0.f;
        if (sg.dist) {
            if (first >= 0) sg.dist[q] = 0.0;
            else if (a.dkey != 0x7fffffffffffffffLL) sg.dist[q] = smin(sg.dist[q], Key<double>::value(a.dkey));
        }
    }
}

// Skeleton points of each configuration (computeSkeleton), widened to double:
// MODE 0 FP64, MODE 1 the reference's float skeleton, MODE 2 the FP32 FK of
// the FP32 bulk pass.
template <int MODE>
__global__ void k_skeleton(const DevRobot *rbp, const float *q, int64_t C, double *out) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const DevRobot &rb = *rbp;
    const int D = rb.D;
    SkelWalker<MODE> sw;
    sw.begin();
    for (int k = 0; k <= D; ++k) {
        if constexpr (MODE == 0) {
            double p[3];
            sw.point(rb, q + c * D, k, p);
            for (int i = 0; i < 3; ++i) out[(c * (D + 1) + k) * 3 + i] = p[i];
        } else {
            float p[3];
            sw.point(rb, q + c * D, k, p);
            for (int i = 0; i < 3; ++i) out[(c * (D + 1) + k) * 3 + i] = (double)p[i];
        }
    }
}

// ---------------------------------------------------------------- edges --
// Checks per edge and their exclusive offsets within blocks of kEdgeScanBlock
// edges; block totals go to bprefix[b + 1] for the block scan.  With a single
// block the prefix is final here (no scan pass).  Zeroes the launch's counters.
__global__ void __launch_bounds__(kEdgeScanBlock) k_edge_prep(const __grid_constant__ EdgeParams P) {
    __shared__ int32_t warp_sum[kEdgeScanBlock / 32];
    const int64_t e = (int64_t)blockIdx.x * kEdgeScanBlock + threadIdx.x;
    if (blockIdx.x == 0 && threadIdx.x < 4) P.counters[threadIdx.x] = 0u;
    if (blockIdx.x == 0 && threadIdx.x < 2) P.work[threadIdx.x] = 0ull;
    int n = 0;
    if (e < P.E) {
        n = edge_geom(P, edge_seg(P, e), e).n;
        P.n_e[e] = n;
        P.kmax[e] = 0;
        P.full[e] = 0;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = n;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warp_sum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = warp_sum[lane];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, off);
            if (lane >= off) t += y;
        }
        warp_sum[lane] = t;   // inclusive over warps
    }
    __syncthreads();
    const int excl = x - n + (wid > 0 ? warp_sum[wid - 1] : 0);
    if (e < P.E) P.local[e] = excl;
    if (threadIdx.x == kEdgeScanBlock - 1) {
        P.bprefix[blockIdx.x + 1] = warp_sum[31];
        if (gridDim.x == 1) P.bprefix[0] = 0;
    }
}

// Exclusive scan of the block totals (one CTA; bprefix[0] = 0).
__global__ void k_edge_scan(const __grid_constant__ EdgeParams P, int nblocks) {
    if (threadIdx.x == 0) {
        int64_t acc = 0;
        P.bprefix[0] = 0;
        for (int b = 1; b <= nblocks; ++b) {
            acc += P.bprefix[b];
            P.bprefix[b] = acc;
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_edges_exact(const __grid_constant__ EdgeParams P) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ WarpShared<T> wsh[kThreads / 32];
    __shared__ float qbuf[kThreads / 32][32 * kMaxDof];
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    if (P.nseg_lane != 1) {   // several segments: robots and scenes from global memory
        edge_warps<MODE, T>(P, nullptr, nullptr, nm, wsh[threadIdx.x >> 5], qbuf[threadIdx.x >> 5]);
        return;
    }
    const Seg &sg = P.segs[0].seg;
    bulk_init(&bar);
    if (!stage<MODE>(sg, smem, &bar, P.status)) return;
    const DevRobot &rb = *reinterpret_cast<const DevRobot *>(smem);
    const T *rows = reinterpret_cast<const T *>(smem + sizeof(DevRobot));
    const float *frows = (MODE == 0) ? reinterpret_cast<const float *>(smem + sizeof(DevRobot) + kDRows * sg.n_pad * sizeof(double))
                                     : reinterpret_cast<const float *>(rows);
    const ObsView<T> ob{rows, frows + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad, MODE == 0 ? frows : nullptr};
    edge_warps<MODE, T>(P, &rb, &ob, nm, wsh[threadIdx.x >> 5], qbuf[threadIdx.x >> 5]);
}

// FP64 recheck of the checks the FP32 edge pass left unsettled (one warp each).
__global__ void __launch_bounds__(kThreads) k_edge_recheck(const __grid_constant__ EdgeParams P) {
    __shared__ float qbuf[kThreads / 32][kMaxDof];
    const uint32_t n = min(*P.recheck_count, P.recheck_cap);
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (uint32_t it = blockIdx.x * (blockDim.x / 32) + wid; it < n; it += warps) {
        const uint64_t ent = P.recheck[it];
        const int64_t e = (int64_t)(ent >> 20);
        const int k = (int)(ent & 0xfffff);
        if (k <= *(volatile int32_t *)&P.kmax[e]) continue;
        const int s = edge_seg(P, e);
        if (lane == 0) {
            const EdgeGeom gm = edge_geom(P, s, e);
            edge_config(gm.a, gm.b, gm.D, gm.n, k, gm.dist, qbuf[wid]);
        }
        __syncwarp();
        const Seg &sg = P.segs[s].seg;
        uint8_t v = 1;
        config_exact_warp<0, double>(*sg.robot, global_obs<double>(sg), qbuf[wid], P.nmd, Want{true, false, false}, &v,
                                     nullptr, nullptr);
        v = (uint8_t)__shfl_sync(0xffffffffu, (int)v, 0);
        if (lane == 0 && v == 0) atomicMax(&P.kmax[e], k);
        __syncwarp();
    }
}

// Edges whose unsettled checks overflowed the list: every remaining check in
// FP64, nearest q2 first (one warp per edge).
__global__ void __launch_bounds__(kThreads) k_edge_full(const __grid_constant__ EdgeParams P) {
    __shared__ float qbuf[kThreads / 32][kMaxDof];
    if (*P.overflow == 0) return;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t e = (int64_t)blockIdx.x * (blockDim.x / 32) + wid; e < P.E; e += warps) {
        if (!P.full[e]) continue;
        const int s = edge_seg(P, e);
        const Seg &sg = P.segs[s].seg;
        const EdgeGeom gm = edge_geom(P, s, e);
        for (int k = gm.n; k > P.kmax[e]; --k) {
            if (lane == 0) edge_config(gm.a, gm.b, gm.D, gm.n, k, gm.dist, qbuf[wid]);
            __syncwarp();
            uint8_t v = 1;
            config_exact_warp<0, double>(*sg.robot, global_obs<double>(sg), qbuf[wid], P.nmd, Want{true, false, false},
                                         &v, nullptr, nullptr);
            v = (uint8_t)__shfl_sync(0xffffffffu, (int)v, 0);
            __syncwarp();
            if (v == 0) {
                if (lane == 0) atomicMax(&P.kmax[e], k);
                break;
            }
        }
    }
}

__global__ void k_edge_final(const __grid_constant__ EdgeParams P) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= P.E) return;
    const EdgeSeg &es = P.segs[edge_seg(P, e)];
    const int64_t le = e - es.e0;
    const int km = P.kmax[e];
    es.seg.valid[le] = km == 0 ? 1 : 0;
    if (es.checks_out) es.checks_out[le] = km == 0 ? P.n_e[e] : P.n_e[e] - km + 1;
}

cudaError_t launch_edge_prep(const EdgeParams &p, cudaStream_t st) {
    const int nb = (int)((p.E + kEdgeScanBlock - 1) / kEdgeScanBlock);
    if (nb == 0) return cudaSuccess;
    k_edge_prep<<<nb, kEdgeScanBlock, 0, st>>>(p);
    if (nb > 1) k_edge_scan<<<1, 32, 0, st>>>(p, nb);
    return cudaGetLastError();
}

cudaError_t launch_edges(int mode, const EdgeParams &p, int grid, size_t smem, cudaStream_t st) {
    if (mode == RPM_PREC_FP64) {
        static std::atomic<uint64_t> attr{0};
        ensure_smem_limit(k_edges_exact<0>, 160 * 1024, attr);
        k_edges_exact<0><<<grid, kThreads, smem, st>>>(p);
    } else {
        static std::atomic<uint64_t> attr{0};
        ensure_smem_limit(k_edges_exact<1>, 160 * 1024, attr);
        k_edges_exact<1><<<grid, kThreads, smem, st>>>(p);
    }
    return cudaGetLastError();
}

template <int MODE, bool MULTI>
static cudaError_t launch_wide_edges(const EdgeParams &p, int grid, size_t smem, cudaStream_t st) {
    static std::atomic<uint64_t> attr{0};
    ensure_smem_limit(k_edges_wide<MODE, MULTI>, 200 * 1024, attr);
    k_edges_wide<MODE, MULTI><<<grid, kWideThreads, smem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_edges_wide(int mode, const EdgeParams &p, int grid, size_t smem, cudaStream_t st) {
    const bool multi = p.nseg - p.nseg_lane > 1;
    if (mode == RPM_PREC_FP32_RECHECK) return launch_edges_wide_fp32(p, grid, smem, st);
    if (mode == RPM_PREC_FP64) return multi ? launch_wide_edges<0, true>(p, grid, smem, st) : launch_wide_edges<0, false>(p, grid, smem, st);
    return multi ? launch_wide_edges<1, true>(p, grid, smem, st) : launch_wide_edges<1, false>(p, grid, smem, st);
}

cudaError_t launch_edge_recheck_final(const EdgeParams &p, int grid, bool pairs, cudaStream_t st) {
    if (pairs) {
        k_edge_pair_skel<<<grid * 4, kThreads, 0, st>>>(p);
        k_edge_pair_eval<<<grid * 2, kThreads, 0, st>>>(p);
        k_edge_pair_fold<<<grid, kThreads, 0, st>>>(p);
    }
    k_edge_recheck<<<grid, kThreads, 0, st>>>(p);
    k_edge_full<<<grid, kThreads, 0, st>>>(p);
    const unsigned fb = (unsigned)((p.E + 255) / 256);
    if (fb) k_edge_final<<<fb, 256, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_check_exact(int mode, const KParams &p, int64_t blocks, size_t smem, cudaStream_t st) {
    if (mode == RPM_PREC_FP64) {
        static std::atomic<uint64_t> attr{0};
        ensure_smem_limit(k_check_exact<0>, 200 * 1024, attr);
        k_check_exact<0><<<(unsigned)blocks, kThreads, smem, st>>>(p);
    } else {
        static std::atomic<uint64_t> attr{0};
        ensure_smem_limit(k_check_exact<1>, 200 * 1024, attr);
        k_check_exact<1><<<(unsigned)blocks, kThreads, smem, st>>>(p);
    }
    return cudaGetLastError();
}

size_t wide_smem_bytes(int mode, int ns, int nb) { return WideLayout::of(mode, ns, nb).total; }

cudaError_t launch_check_wide(int mode, const KParams &p, int64_t blocks, size_t smem, cudaStream_t st) {
    if (mode == RPM_PREC_FP32_RECHECK) return launch_check_wide_fp32(p, blocks, smem, st);
    if (mode == RPM_PREC_FP64) {
        static std::atomic<uint64_t> attr{0};
        ensure_smem_limit(k_check_wide<0>, 200 * 1024, attr);
        k_check_wide<0><<<(unsigned)blocks, kWideThreads, smem, st>>>(p);
    } else {
        static std::atomic<uint64_t> attr{0};
        ensure_smem_limit(k_check_wide<1>, 200 * 1024, attr);
        k_check_wide<1><<<(unsigned)blocks, kWideThreads, smem, st>>>(p);
    }
    return cudaGetLastError();
}

// ------------------------------------------------------ nearest points --
// One (link i, obstacle j) pair of computeDistance with nearest points: the
// distance after the min_dist_tol clamp (:367-368); with 'store' its points go
// to near ([n][6][L] of the configuration).  Ground pairs the reference skips
// carry (0, 0, 0), (0, 0, -MAX_DISTANCE).
template <int MODE, typename T>
__device__ __forceinline__ T near_pair(const NearParams &P, const DevRobot &rb, const Num<T> &nm, const T *A,
                                       const T *B, int i, int j, const float *ground, float *near, int L, bool store) {
    const T r = MODE == 0 ? (T)rb.radius_d[i] : (T)rb.radius_f[i];
    T d, pts[6];
    bool has = true;
    const T tol = MODE == 0 ? (T)P.obs_d[(size_t)kRowTol * P.n_pad + j] : (T)P.obs_f[(size_t)kRowTol * P.n_pad + j];
    if (ground[j] != 0.f && i < rb.ground_included) {
        d = nm.maxd;
        pts[0] = pts[1] = pts[2] = pts[3] = pts[4] = T(0);
        pts[5] = -nm.maxd;
    } else {
        T o[6];
        for (int k = 0; k < 6; ++k)
            o[k] = MODE == 0 ? (T)P.obs_d[(size_t)k * P.n_pad + j] : (T)P.obs_f[(size_t)k * P.n_pad + j];
        d = capsule_box_pts(nm, A, B, r, o, pts, has);
    }
    if (d > tol) d = nm.maxd;   // :367-368
    if (store)
        for (int k = 0; k < 6; ++k) near[((size_t)j * 6 + k) * L + i] = (float)pts[k];
    return d;
}

// computeDistance(q, true) with nearest points (RealVectorSpace.cpp:318-392),
// one warp per configuration: links in order, lanes over the obstacles, every
// pair evaluated; the link minimum and the first hit (lowest obstacle index
// with d <= 0 after the min_dist_tol clamp) are warp reductions.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_distance_nearest(const __grid_constant__ NearParams P) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    __shared__ T skel[kThreads / 32][(kMaxDof + 1) * 3];
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c = (int64_t)blockIdx.x * (kThreads / 32) + w;
    if (c >= P.C) return;
    const DevRobot &rb = *P.robot;
    const int D = rb.D, L = D;
    if (lane == 0) {
        SkelWalker<MODE> sw;
        sw.begin();
        for (int k = 0; k <= D; ++k) sw.point(rb, P.q + c * D, k, skel[w] + 3 * k);
    }
    __syncwarp();
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    const float *ground = P.obs_f + (size_t)kRowGround * P.n_pad;
    float *near = P.nearest + (size_t)c * P.n * 6 * L;
    T d_c = nm.maxd;
    int hit = -1;
    for (int i = 0; i < L && hit < 0; ++i) {
        const T *A = skel[w] + 3 * i, *B = A + 3;
        T lmin = nm.maxd, hv = T(0);
        int hj = 0x7fffffff;
        for (int j = lane; j < P.n; j += 32) {
            const T d = near_pair<MODE, T>(P, rb, nm, A, B, i, j, ground, near, L, true);
            lmin = smin(lmin, d);
            if (d <= T(0) && j < hj) { hj = j; hv = d; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            lmin = smin(lmin, __shfl_xor_sync(full, lmin, off));
            const int oj = __shfl_xor_sync(full, hj, off);
            const T ov = __shfl_xor_sync(full, hv, off);
            if (oj < hj) { hj = oj; hv = ov; }
        }
        if (hj != 0x7fffffff) {   // the reference returns at its first hit
            hit = i;
            if (lane == 0) P.profile[c * L + i] = (float)hv;
        } else {
            if (lane == 0) P.profile[c * L + i] = (float)lmin;
            d_c = smin(d_c, lmin);
        }
    }
    if (lane == 0) {
        if (hit >= 0)
            for (int k = hit + 1; k < L; ++k) P.profile[c * L + k] = 0.f;
        P.dist[c] = hit >= 0 ? 0.0 : (double)d_c;
        P.flag[c] = hit >= 0 ? 0 : 1;
    }
}

// computeDistance(q, true) with nearest points for a few configurations: one
// CTA per configuration and one thread per (link, obstacle) pair, so a single
// state (the adapter's path, the current state of a DRGBT step) takes one
// tree's latency instead of a warp walking its links in turn.  The per-link
// minimum and first hit are shared-memory atomics on order-preserving keys,
// which give the i-major / j-minor result; the reference's early exit then
// decides which links the profile keeps.  Points are written for every pair:
// where the reference stops at a hit the configuration's points are flagged
// invalid (flag 0), as in k_distance_nearest.
// Threads per CTA: 512 for the reference numerics (a pair each up to 512
// pairs, where 256 threads leave some two trees in a row), 256 for the FP64
// form (its registers).
template <int MODE> constexpr int near_cta_threads() { return MODE == 1 ? 512 : 256; }
constexpr int64_t kNearCtaMaxConfigs = 64;

template <int MODE>
__global__ void __launch_bounds__(near_cta_threads<MODE>()) k_distance_nearest_cta(const __grid_constant__ NearParams P) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    __shared__ T skel[(kMaxDof + 1) * 3];
    __shared__ double sc[2 * kMaxDof];
    __shared__ typename Key<T>::type lkey[kMaxDof];
    __shared__ int hj[kMaxDof];
    __shared__ T hv[kMaxDof];
    const int64_t c = blockIdx.x;
    const DevRobot &rb = *P.robot;
    const int D = rb.D, L = D;
    const float *q = P.q + c * D;
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    if (threadIdx.x < 32) {   // joint sines in parallel, then the chain spread over the warp (the same bits)
        warp_sincos(q, D, sc);
        __syncwarp();
        skel_coop<MODE, T>(rb, sc, skel);
    }
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        lkey[i] = Key<T>::of(nm.maxd);
        hj[i] = 0x7fffffff;
    }
    __syncthreads();
    if constexpr (MODE == 1) {
        if (P.skel_out)
            for (int k = threadIdx.x; k < 3 * (D + 1); k += blockDim.x) P.skel_out[c * 3 * (D + 1) + k] = skel[k];
    }
    const float *ground = P.obs_f + (size_t)kRowGround * P.n_pad;
    float *near = P.nearest + (size_t)c * P.n * 6 * L;
    const int npairs = L * P.n;
    for (int p = threadIdx.x; p < npairs; p += blockDim.x) {
        const int i = p / P.n, j = p - i * P.n;
        const T d = near_pair<MODE, T>(P, rb, nm, skel + 3 * i, skel + 3 * i + 3, i, j, ground, near, L, true);
        if (d == d) atomicMin(&lkey[i], Key<T>::of(d));   // std::min ignores NaN
        if (d <= T(0)) atomicMin(&hj[i], j);
    }
    __syncthreads();
    // each link's hit value: its lowest hitting obstacle, evaluated again (the same bits)
    for (int i = threadIdx.x; i < L; i += blockDim.x)
        if (hj[i] != 0x7fffffff)
            hv[i] = near_pair<MODE, T>(P, rb, nm, skel + 3 * i, skel + 3 * i + 3, i, hj[i], ground, near, L, false);
    __syncthreads();
    if (threadIdx.x == 0) {
        T d_c = nm.maxd;
        int hit = -1;
        for (int i = 0; i < L; ++i) {
            if (hj[i] != 0x7fffffff) {   // the reference returns at its first hit
                hit = i;
                P.profile[c * L + i] = (float)hv[i];
                break;
            }
            const T lm = Key<T>::value(lkey[i]);
            P.profile[c * L + i] = (float)lm;
            d_c = smin(d_c, lm);
        }
        if (hit >= 0)
            for (int k = hit + 1; k < L; ++k) P.profile[c * L + k] = 0.f;
        P.dist[c] = hit >= 0 ? 0.0 : (double)d_c;
        P.flag[c] = hit >= 0 ? 0 : 1;
    }
}

// computeDistanceUnderestimation (RealVectorSpace.cpp:402-446) from the
// nearest points in P.nearest: per link the smallest distance of its two
// skeleton points to the planes through the obstacle points O with normals
// (R - O) / |R - O| (Eigen's normalized(): unchanged when |R - O| = 0), minus
// the radius; pairs whose O has norm MAX_DISTANCE are passed over.  The
// reference returns 0 at the first negative value without updating the
// state: flag 0, distance 0, profile not written.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_distance_underest(const __grid_constant__ NearParams P) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    __shared__ T skel[kThreads / 32][(kMaxDof + 1) * 3];
    __shared__ T prof[kThreads / 32][kMaxDof];
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c = (int64_t)blockIdx.x * (kThreads / 32) + w;
    if (c >= P.C) return;
    const DevRobot &rb = *P.robot;
    const int D = rb.D, L = D;
    if (lane == 0) {
        SkelWalker<MODE> sw;
        sw.begin();
        for (int k = 0; k <= D; ++k) sw.point(rb, P.q + c * D, k, skel[w] + 3 * k);
    }
    __syncwarp();
    const T maxd = MODE == 0 ? (T)P.nmd.maxd : (T)P.nmf.maxd;
    const float *near = P.nearest + (size_t)c * P.n * 6 * L;
    T d_c = maxd;
    bool negative = false;
    for (int i = 0; i < L && !negative; ++i) {
        const T *S0 = skel[w] + 3 * i, *S1 = S0 + 3;
        const T r = MODE == 0 ? (T)rb.radius_d[i] : (T)rb.radius_f[i];
        T lmin = maxd;
        bool neg = false;
        for (int j = lane; j < P.n; j += 32) {
            T O[3], R[3];
            for (int k = 0; k < 3; ++k) {
                R[k] = (T)near[((size_t)j * 6 + k) * L + i];
                O[k] = (T)near[((size_t)j * 6 + 3 + k) * L + i];
            }
            if (sqrtT(dot3(O, O)) == maxd) continue;
            T u[3] = {R[0] - O[0], R[1] - O[1], R[2] - O[2]};
            const T z = dot3(u, u);
            if (z > T(0)) {
                const T nz = sqrtT(z);
                for (int k = 0; k < 3; ++k) u[k] = u[k] / nz;
            }
            T a[3] = {S0[0] - O[0], S0[1] - O[1], S0[2] - O[2]};
            T b[3] = {S1[0] - O[0], S1[1] - O[1], S1[2] - O[2]};
            const T d = smin(dot3(a, u), dot3(b, u)) - r;
            if (d < T(0)) neg = true;
            lmin = smin(lmin, d);
        }
        negative = __any_sync(full, neg);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) lmin = smin(lmin, __shfl_xor_sync(full, lmin, off));
        if (lane == 0) prof[w][i] = lmin;
        d_c = smin(d_c, lmin);
    }
    __syncwarp();
    if (negative) {
        if (lane == 0) { P.dist[c] = 0.0; P.flag[c] = 0; }
        return;
    }
    for (int i = lane; i < L; i += 32) P.profile[c * L + i] = (float)prof[w][i];
    if (lane == 0) { P.dist[c] = (double)d_c; P.flag[c] = 1; }
}

cudaError_t launch_distance_nearest(int mode, const NearParams &p, cudaStream_t st) {
    if (p.C > 0 && p.C <= kNearCtaMaxConfigs) {   // a few states: one CTA each
        if (mode == RPM_PREC_FP32_REF) k_distance_nearest_cta<1><<<(unsigned)p.C, near_cta_threads<1>(), 0, st>>>(p);
        else k_distance_nearest_cta<0><<<(unsigned)p.C, near_cta_threads<0>(), 0, st>>>(p);
        return cudaGetLastError();
    }
    const unsigned grid = (unsigned)((p.C + kThreads / 32 - 1) / (kThreads / 32));
    if (grid == 0) return cudaSuccess;
    if (mode == RPM_PREC_FP32_REF) k_distance_nearest<1><<<grid, kThreads, 0, st>>>(p);
    else k_distance_nearest<0><<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_distance_underest(int mode, const NearParams &p, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.C + kThreads / 32 - 1) / (kThreads / 32));
    if (grid == 0) return cudaSuccess;
    if (mode == RPM_PREC_FP32_REF) k_distance_underest<1><<<grid, kThreads, 0, st>>>(p);
    else k_distance_underest<0><<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_pair_recheck(const KParams &p, int grid, cudaStream_t st) {
    k_pair_skel<<<grid * 4, kThreads, 0, st>>>(p);
    if (p.ps.order) {
        k_pair_key<<<grid, kThreads, 0, st>>>(p);
        k_pair_scatter<<<grid, kThreads, 0, st>>>(p);
    }
    k_pair_eval<<<grid * 2, kThreads, 0, st>>>(p);
    k_pair_fold<<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_recheck(const KParams &p, int grid, cudaStream_t st) {
    k_recheck<<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_skeleton(int mode, const DevRobot *rb, int D, const float *q, int64_t C, double *out, cudaStream_t st) {
    (void)D;
    const unsigned grid = (unsigned)((C + 127) / 128);
    if (grid == 0) return cudaSuccess;
    if (mode == RPM_PREC_FP64) k_skeleton<0><<<grid, 128, 0, st>>>(rb, q, C, out);
    else if (mode == RPM_PREC_FP32_REF) k_skeleton<1><<<grid, 128, 0, st>>>(rb, q, C, out);
    else k_skeleton<2><<<grid, 128, 0, st>>>(rb, q, C, out);
    return cudaGetLastError();
}

}  // namespace rpm

// ----------------------------------------------------------------- spines --
namespace rpm {

// computeEnclosingRadii: one thread per configuration.
__global__ void __launch_bounds__(kThreads) k_enclosing_radii(const __grid_constant__ SpineParams P) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.C) return;
    const DevRobot &rb = *P.robot;
    const int D = rb.D;
    float sk[3 * (kMaxDof + 1)], row[kMaxDof + 1];
    skel_ref(rb, P.q + c * D, sk);
    float *out = P.radii + c * D * (D + 1);
    for (int i = 0; i < D; ++i) {
        enclosing_row(rb, sk, i, row);
        for (int j = 0; j <= D; ++j) out[i * (D + 1) + j] = row[j];
    }
}

// extendSpine: one thread per spine.
__global__ void __launch_bounds__(kThreads) k_extend_spines(const __grid_constant__ SpineParams P) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.C) return;
    const DevRobot &rb = *P.robot;
    const int D = rb.D;
    float sk[3 * (kMaxDof + 1)], sk_end[3 * (kMaxDof + 1)];
    skel_ref(rb, P.q + c * D, sk);
    P.status[c] = extend_spine(rb, P.q + c * D, sk, P.dist[c], P.profile + c * D, P.qe + c * D, P.num_iter,
                               P.expanded != 0, P.q_new + c * D, sk_end);
}

// computeReachedState: one warp per horizon state, its state in shared memory
// (SpineWarp) and the spine spread over the lanes (extend_spine_warp); the
// lanes split the obstacles of computeDistanceUnderestimation, whose first
// negative value (any lane, any link) makes the reference return 0 without
// updating the state.
// The underestimation planes of the current state's nearest points, one per
// (link i, obstacle j) at [i * n + j]: the unit normal u = normalized(R - O)
// (unchanged when zero) and the point O, with skip = 1 where |O| is
// MAX_DISTANCE (a pair the reference passes over).  They do not change over
// the horizon, so a CTA computes them once (the same operations as per use).
struct __align__(16) Plane {   // 32 bytes: two 16-byte shared-memory loads
    float u[3], O[3];
    int skip, pad;
};

__device__ __forceinline__ Plane make_plane(const SpineParams &P, int L, int i, int j) {
    Plane pl;
    float R[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        R[k] = P.cur_near[((size_t)j * 6 + k) * L + i];
        pl.O[k] = P.cur_near[((size_t)j * 6 + 3 + k) * L + i];
    }
    pl.skip = sqrtf(dot3f(pl.O, pl.O)) == P.maxd;
    pl.pad = 0;
    pl.u[0] = R[0] - pl.O[0]; pl.u[1] = R[1] - pl.O[1]; pl.u[2] = R[2] - pl.O[2];
    const float z = dot3f(pl.u, pl.u);
    if (z > 0.f) {
        const float nz = sqrtf(z);
#pragma unroll
        for (int k = 0; k < 3; ++k) pl.u[k] = pl.u[k] / nz;
    }
    return pl;
}

__global__ void __launch_bounds__(kThreads) k_reached_states(const __grid_constant__ SpineParams P) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    __shared__ SpineWarp sw_all[kThreads / 32];
    extern __shared__ __align__(16) unsigned char planes_smem[];
    Plane *planes = P.planes ? reinterpret_cast<Plane *>(planes_smem) : nullptr;
    if (planes) {
        for (int p = threadIdx.x; p < P.L * P.n; p += blockDim.x) planes[p] = make_plane(P, P.L, p / P.n, p % P.n);
        __syncthreads();
    }
    const int64_t h = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (h >= P.C) return;
    SpineWarp &w = sw_all[threadIdx.x >> 5];
    const DevRobot &rb = *P.robot;
    const int D = rb.D, L = D;
    if (lane < D) {
        w.qn[lane] = P.q_cur[lane];
        w.qe[lane] = P.qe[h * D + lane];
    }
    const float d_cur = (float)P.cur_dist[0];
    int status = kStTrapped;
    if (d_cur > 0.f) {
        if (lane < L) w.pn[lane] = P.cur_prof[lane];
        float dn = d_cur;
        status = kStNone;
        if (P.cur_skel) {   // the skeleton of q_cur from the nearest-point kernel (the same bits)
            for (int k = lane; k < 3 * (D + 1); k += 32) w.skn[k] = P.cur_skel[k];
            __syncwarp();
        } else {
            skel_ref_shared(rb, w.qn, w.skn, w.sc);
        }
        for (int layer = 0; layer < P.num_layers; ++layer) {
            status = extend_spine_warp(rb, w, dn, P.num_iter, P.expanded != 0);
            if (lane < D) w.qn[lane] = w.qs[lane];
            for (int k = lane; k < 3 * (D + 1); k += 32) w.skn[k] = w.sk[k];
            __syncwarp();
            // all links at once: G lanes per link (a power of two, G L <= 32),
            // each over a strided share of the obstacles.  Every value is the
            // reference's; min is exact and free of order here (no NaN, no
            // -0), and "any negative" is what its early return amounts to (on
            // a negative value neither the minima nor the profile are used)
            int G = 32;
            while (G * L > 32) G >>= 1;
            const int i = lane / G, sub = lane & (G - 1);
            float lmin = P.maxd;
            bool neg = false;
            if (i < L) {
                const float *S0 = w.sk + 3 * i, *S1 = S0 + 3;
                const float ri = rb.radius_f[i];
                for (int j = sub; j < P.n; j += G) {
                    const Plane pl = planes ? planes[i * P.n + j] : make_plane(P, L, i, j);
                    if (pl.skip) continue;
                    const float *O = pl.O, *u = pl.u;
                    float a[3] = {S0[0] - O[0], S0[1] - O[1], S0[2] - O[2]};
                    float b[3] = {S1[0] - O[0], S1[1] - O[1], S1[2] - O[2]};
                    const float d = min_std(dot3f(a, u), dot3f(b, u)) - ri;
                    if (d < 0.f) neg = true;
                    lmin = min_std(lmin, d);
                }
            }
            const bool negative = __any_sync(full, neg);
            for (int off = G >> 1; off > 0; off >>= 1) lmin = min_std(lmin, __shfl_xor_sync(full, lmin, off));
            if (i < L && sub == 0) w.p[i] = lmin;
            float d_c = lmin;   // the links' minimum (lanes past the links hold maxd)
            for (int off = 16; off >= G; off >>= 1) d_c = min_std(d_c, __shfl_xor_sync(full, d_c, off));
            __syncwarp();
            float d;
            if (!negative) {
                d = d_c;
                dn = d_c;
                if (lane < L) w.pn[lane] = w.p[lane];
            } else {
                d = 0.f;
                dn = -1.f;
            }
            __syncwarp();
            if (d < P.d_crit || status != kStAdvanced) break;
        }
    }
    if (lane < D) P.q_new[h * D + lane] = w.qn[lane];
    if (lane == 0) P.status[h] = status;
}

cudaError_t launch_enclosing_radii(const SpineParams &p, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.C + kThreads - 1) / kThreads);
    if (grid) k_enclosing_radii<<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_extend_spines(const SpineParams &p, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.C + kThreads - 1) / kThreads);
    if (grid) k_extend_spines<<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_reached_states(const SpineParams &p, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.C + kThreads / 32 - 1) / (kThreads / 32));
    if (!grid) return cudaSuccess;
    // the plane table in shared memory when it is small next to the work of the
    // CTA's states (a few states, scenes of up to a few hundred obstacles)
    SpineParams q = p;
    const size_t bytes = (size_t)p.L * p.n * sizeof(Plane);
    q.planes = (p.L > 0 && p.n > 0 && bytes <= 16384) ? 1 : 0;
    k_reached_states<<<grid, kThreads, q.planes ? bytes : 0, st>>>(q);
    return cudaGetLastError();
}

}  // namespace rpm

namespace rpm {

// MotionValidity::check: one warp per motion, checks in order with early exit;
// the lanes split the static obstacles, then the moving boxes of the check.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_motion_validity(const __grid_constant__ MotionParams P) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t m = (int64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (m >= P.M) return;
    const DevRobot &rb = *P.robot;
    const int D = rb.D, L = D;
    const float *q1 = P.q_prev + m * D, *q2 = P.q_cur + m * D;
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    const ObsView<T> ob{MODE == 0 ? reinterpret_cast<const T *>(P.obs_d) : reinterpret_cast<const T *>(P.obs_f),
                        P.obs_f + (size_t)kRowGround * P.n_pad, P.n, P.n_pad};
    float dist;
    edge_count(q1, q2, D, 1.f, 1, dist);   // getNorm in index order
    int bad = 0;
    for (int k = 1; k <= P.N && !bad; ++k) {
        const float step = dist * (float)k / (float)P.N;
        float q[kMaxDof];
        if (dist > 0.f) edge_point(q1, q2, D, step / dist, q);
        else for (int i = 0; i < D; ++i) q[i] = q2[i];
        SkelWalker<MODE> sw;
        sw.begin();
        T A[3], B[3];
        sw.point(rb, q, 0, A);
        for (int i = 0; i < L; ++i) {
            sw.point(rb, q, i + 1, B);
            const T r = LinkConst<T>::r(rb, i), rn = LinkConst<T>::rn(rb, i);
            const bool gskip = i < rb.ground_included;
            bool hit = false;
            for (int j = lane; j < P.n && !hit; j += 32) {
                if (P.moving[j] || (gskip && ob.is_ground(j))) continue;
                T o[6];
                ob.box(j, o);
                hit = coll_box_call<T, ExactPol>(nm, A, B, r, rn, o).v;
            }
            for (int mi = lane; mi < P.n_mov && !hit; mi += 32) {
                if (gskip && ob.is_ground(P.mov_idx[mi])) continue;
                T o[6];
                const float *src = P.mov_aabb + ((size_t)(k - 1) * P.n_mov + mi) * 6;
#pragma unroll
                for (int c = 0; c < 6; ++c) o[c] = (T)src[c];
                hit = coll_box_call<T, ExactPol>(nm, A, B, r, rn, o).v;
            }
            if (__any_sync(full, hit)) { bad = k; break; }
#pragma unroll
            for (int c = 0; c < 3; ++c) A[c] = B[c];
        }
    }
    if (lane == 0) {
        P.valid[m] = bad ? 0 : 1;
        if (P.checks) P.checks[m] = bad ? bad : P.N;
    }
}

cudaError_t launch_motion_validity(int mode, const MotionParams &p, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.M + kThreads / 32 - 1) / (kThreads / 32));
    if (grid == 0) return cudaSuccess;
    if (mode == RPM_PREC_FP64) k_motion_validity<0><<<grid, kThreads, 0, st>>>(p);
    else k_motion_validity<1><<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

// ------------------------------------------------------------- primitive probe --
// One case per thread through the same tree instances the check kernels use.
template <int MODE>
__global__ void k_probe_exact(const __grid_constant__ ProbeParams P, bool only_unsettled) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    if (only_unsettled && P.settled[i] != 0) return;
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    T A[3], B[3], X[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) { A[k] = (T)P.a[3 * i + k]; B[k] = (T)P.b[3 * i + k]; }
#pragma unroll
    for (int k = 0; k < 6; ++k) X[k] = (T)P.x[6 * i + k];
    const float rf = P.r[i];
    const T r = (T)rf;
    // r * sqrt(3) / 3 with sqrt(3) in double, as CollisionAndDistance.cpp:7 and the robot upload compute it
    const double rn_d = (double)rf * sqrt(3.0) / 3;
    const T rn = (T)rn_d;
    double v;
    const int kind = P.kind[i];
    if (kind == 0) v = coll_box_call<T, ExactPol>(nm, A, B, r, rn, X).v ? 1.0 : 0.0;
    else if (kind == 1) v = (double)capsule_box_call<T, ExactPol>(nm, A, B, r, X).v;
    else {
        ExactPol pol;
        v = (double)seg_seg(pol, nm, A, B, X, X + 3).v;
    }
    P.value[i] = v;
    if (P.settled && !only_unsettled) P.settled[i] = 1;
}

cudaError_t launch_probe_exact(int mode, const ProbeParams &p, bool only_unsettled, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.n + 127) / 128);
    if (grid == 0) return cudaSuccess;
    if (mode == 0) k_probe_exact<0><<<grid, 128, 0, st>>>(p, only_unsettled);
    else k_probe_exact<1><<<grid, 128, 0, st>>>(p, only_unsettled);
    return cudaGetLastError();
}

// ---------------------------------------------------- decision margins --
// How close each configuration's FP64 answers lie to a decision boundary of
// the reference's trees: the margins of RobustPol (metres over the error
// amplification of the compared quantities) evaluated in FP64 on the FP64
// skeleton, one warp per configuration, lanes over the obstacles.
//   margin_valid: isValid is an OR over the pairs, so a collision is as
//     robust as its most robust colliding pair and a free configuration as
//     its least robust pair;
//   margin_dist: the smallest margin among the pairs that can set d_c
//     (clamped distance within 1e-3 m of the minimum; with the min_dist_tol
//     and contact-band rules of the FP32 pass), or for a collision the
//     largest margin among the pairs at distance 0 or below.
// A configuration on which FP32 and FP64 arithmetic disagree must have a
// margin inside the FP32 rounding band.
__global__ void __launch_bounds__(kThreads) k_decision_margins(const __grid_constant__ NearParams P) {
    __shared__ double skel[kThreads / 32][(kMaxDof + 1) * 3];
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c = (int64_t)blockIdx.x * (kThreads / 32) + w;
    if (c >= P.C) return;
    const DevRobot &rb = *P.robot;
    const int D = rb.D, L = D;
    if (lane == 0) {
        SkelWalker<0> sw;
        sw.begin();
        for (int k = 0; k <= D; ++k) sw.point(rb, P.q + c * D, k, skel[w] + 3 * k);
    }
    __syncwarp();
    const Num<double> nm = P.nmd;
    const float *ground = P.obs_f + (size_t)kRowGround * P.n_pad;
    const double inf = 1e300;
    // isValid: robust OR over the pairs; distance: pass 1 finds d_c
    bool coll = false;
    double m_true = 0.0, m_all = inf, dmin = nm.maxd, m_hit = 0.0;
    bool hit = false;
    for (int pass = 0; pass < 2; ++pass) {
        double m_near = inf;
        for (int i = 0; i < L; ++i) {
            const double *A = skel[w] + 3 * i, *B = A + 3;
            const double r = rb.radius_d[i], rn = rb.rnew_d[i];
            for (int j = lane; j < P.n; j += 32) {
                if (ground[j] != 0.f && i < rb.ground_included) continue;
                double o[6];
                for (int k = 0; k < 6; ++k) o[k] = P.obs_d[(size_t)k * P.n_pad + j];
                const double tol = P.obs_d[(size_t)kRowTol * P.n_pad + j];
                if (pass == 0) {
                    const RB rr = coll_box_call<double, RobustPol>(nm, A, B, r, rn, o);
                    if (rr.v) { coll = true; m_true = fmax(m_true, (double)rr.m); }
                    m_all = fmin(m_all, (double)rr.m);
                }
                const ValM<double> dv = capsule_box_call<double, RobustPol>(nm, A, B, r, o);
                double d = dv.v;
                float m = dv.m;
                const float band = dv.ia * (kDecide / kBand);
                m = fminf(m, fabsf((float)(d - tol)) * band);
                if (d != 0.0) m = fminf(m, fabsf((float)(d > tol ? nm.maxd : d)) * band);
                if (d > tol) d = nm.maxd;
                if (pass == 0) {
                    if (d == d) dmin = fmin(dmin, d);
                    if (d <= 0.0) { hit = true; m_hit = fmax(m_hit, (double)m); }
                } else if (d <= dmin + 1e-3) {
                    m_near = fmin(m_near, (double)m);
                }
            }
        }
        if (pass == 0) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                coll = __shfl_xor_sync(full, (int)coll, off) != 0 || coll;
                m_true = fmax(m_true, __shfl_xor_sync(full, m_true, off));
                m_all = fmin(m_all, __shfl_xor_sync(full, m_all, off));
                dmin = fmin(dmin, __shfl_xor_sync(full, dmin, off));
                hit = __shfl_xor_sync(full, (int)hit, off) != 0 || hit;
                m_hit = fmax(m_hit, __shfl_xor_sync(full, m_hit, off));
            }
            if (hit) break;   // d_c = 0: the margin is that of the most robust hit
        } else {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) m_near = fmin(m_near, __shfl_xor_sync(full, m_near, off));
            m_hit = m_near;
        }
    }
    if (lane == 0) {
        P.margin_valid[c] = coll ? m_true : m_all;
        P.margin_dist[c] = m_hit;
    }
}

cudaError_t launch_decision_margins(const NearParams &p, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.C + kThreads / 32 - 1) / (kThreads / 32));
    if (grid == 0) return cudaSuccess;
    k_decision_margins<<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace rpm
