// rpm_wide.cuh -- warp-per-configuration drivers of RealVectorSpace::isValid(q)
// (RealVectorSpace.cpp:277-309) and computeDistance(q) (:318-392) over a
// spatially sorted, leaf-bounded copy of the obstacles.
//
// Used for large scenes and small requests, where lane-per-configuration
// leaves the GPU mostly idle and each lane walks hundreds of obstacles in
// series.  Here a warp first runs the forward kinematics of G configurations
// (lane = configuration, skeleton points kept in shared memory), then checks
// them one at a time with the lanes spread over the obstacles:
//   * leaves of 8 obstacles (a top-down median split of their centres) carry
//     their union bounds and their largest / smallest min_dist_tol, so one gap
//     test rejects a whole leaf; lanes cull 32 leaves at a time and then test
//     the obstacles of up to four surviving leaves at a time (4 x 8 lanes);
//   * isValid keeps the leaves within r*sqrt(2) of the link's bounding box
//     (the reach of the reference's capsule-box tree);
//   * distance visits the leaves in nearest-first bands (gap at most twice
//     the nearest live gap plus 2 (r + EQUALITY_THRESHOLD + margin)) and
//     re-prunes after each band, so the running minimum tightens the
//     threshold for the leaves still to visit.
// Every pair the lane-per-configuration driver would evaluate with a tree and
// that can change an output is evaluated here too, with the same arithmetic;
// results combine by the same rules (OR; minimum of ordered keys; first hit =
// lowest ORIGINAL obstacle index), so outputs are bit-identical to it.
#pragma once
#include <type_traits>

#include "rpm_check.cuh"
#include "rpm_edges.cuh"
#include "rpm_launch.cuh"

namespace rpm {

constexpr int kWideWarps = 8;                       // warps per CTA
constexpr int kWideThreads = kWideWarps * 32;
constexpr int kWidePtsBytes = 2048;                 // skeleton buffer per warp
constexpr int kLeaf = 8;                            // obstacles per leaf
constexpr int kBlkRec = 8;                          // lo[3] hi[3] max tol, min tol (float)
constexpr int kLeafPerLane = 9;                     // leaves per lane in the distance search
constexpr int kMaxLeaves = 32 * kLeafPerLane;
constexpr uint32_t kGroundBit = 0x80000000u;        // idx row: ground obstacle
constexpr uint32_t kPadIdx = 0x7fffffffu;           // idx row: padding slot (bounds +inf / -inf)
// static, moving and ground obstacles each pad to whole leaves
static_assert(kMaxLeaves * kLeaf >= kMaxObstacles + 3 * (kLeaf - 1), "sorted layout too small");
// Automatic layout (rpm_api.cu): warp-per-configuration for scenes of at
// least kWideMinObstacles obstacles (profiles: batches up to
// kWideMaxProfileBatch), by the kWide32Batch* thresholds below in the
// FP32+recheck form without profiles, otherwise for kWideMidObstacles with
// batches up to kWideMidBatch, and for kWideSmallObstacles with batches up to
// kWideSmallBatch (FP64) or kWideSmallBatch32 (FP32 forms) without profiles.
constexpr int kWideMinObstacles = 150;
constexpr int64_t kWideMaxProfileBatch = 16384;
constexpr int kWideMidObstacles = 40;
constexpr int64_t kWideMidBatch = 8192;
constexpr int kWideSmallObstacles = 8;
constexpr int64_t kWideSmallBatch = 512;
constexpr int64_t kWideSmallBatch32 = 4096;
// FP32+recheck form without profiles: warp-per-configuration while the batch
// holds at most this many configurations, for scenes of at least 80 / 40 / 20
// obstacles (below 20, the small-scene rule above).  Measured crossovers of
// the two layouts for xarm6 and spatial 10- and 22-DOF robots.
constexpr int64_t kWide32Batch80 = 32768;
constexpr int64_t kWide32Batch40 = 16384;
constexpr int64_t kWide32Batch20 = 8192;
// ... except a single request of at least this many configurations, which the
// lane layout checks in binned order with its per-warp culling: faster than the
// warp layout at every scene size measured (10-1000 obstacles).
constexpr int64_t kLaneBinnedBatch = 32768;
// Edge batches (rpm_api.cu): warp-per-check for scenes of at least this many
// obstacles (measured crossover for spatial 10-DOF edges at 0.05 rad: the
// lane pass 10 % faster at 100 boxes, the warp pass 19 % faster at 130).
constexpr int kWideEdgeObstacles = 110;
// FP32+recheck edges, whose lane pass culls obstacles per warp: the warp pass
// only from this many obstacles and batches above this many edges (measured on
// spatial 10-DOF edges at 0.05 rad: the lane pass faster at every size up to
// 500 boxes and up to 32,768 edges at 1000 boxes; 1.7x slower at 1000 boxes
// and 262,144 edges).
constexpr int kWideEdgeObstacles32 = 700;
constexpr int64_t kWideEdgeBatch32 = 65536;

// Sorted copy of one scene version: slot s holds original obstacle idx[s].
// Static obstacles come first, then moving ones, then ground ones, each group
// in whole leaves, so a leaf is ground-only iff its first slot is ground.
template <typename T> struct SortedView {
    const T *rows;          // [7][ns]: AABB, min_dist_tol
    const uint32_t *idx;    // [ns]
    const float *blk;       // [nb][kBlkRec] leaf records
    int ns, nb;
    RPM_HD void box(int s, T *o) const {
#pragma unroll
        for (int k = 0; k < 6; ++k) o[k] = rows[k * ns + s];
    }
    RPM_HD T tol(int s) const { return rows[kRowTol * ns + s]; }
    RPM_HD bool ground_leaf(int l) const { return (idx[l * kLeaf] & kGroundBit) != 0u; }
    RPM_HD void leaf(int l, T *o) const {
#pragma unroll
        for (int k = 0; k < 6; ++k) o[k] = (T)blk[l * kBlkRec + k];
    }
};

#ifdef __CUDACC__
// Position of the (n+1)-th set bit of m (-1 if m has fewer).
__device__ __forceinline__ int nth_bit(unsigned m, int n) {
    for (int k = 0; k < n; ++k) m &= m - 1u;
    return m ? __ffs(m) - 1 : -1;
}

// Drop the lowest four set bits of m (the leaves of one round).
__device__ __forceinline__ unsigned drop4(unsigned m) {
#pragma unroll
    for (int k = 0; k < 4; ++k) m &= m - 1u;
    return m;
}

template <int MODE, typename T>
__device__ __forceinline__ void wide_push(uint32_t *q, int &nq, bool c, uint32_t item) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, c);
    if (c) q[nq + __popc(m & ((1u << lane) - 1u))] = item;
    nq += __popc(m);
    __syncwarp();
}

// Remove the first 32 entries of a queue holding nq >= 32.
__device__ __forceinline__ void wide_pop32(uint32_t *q, int &nq) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    if (lane < nq - 32) q[lane] = q[32 + lane];
    nq -= 32;
    __syncwarp();
}

// Where unsettled pairs go: the sink (may be null), this configuration's
// record (-1 until its first unsettled pair) and the sticky list-full flag.
struct WideSink {
    const PairSink *ps;
    int slot;
    bool full;
};

// After a drain (all lanes): list this configuration's unsettled pairs
// (each lane its own link and obstacle), allocating its record on the first.
__device__ __forceinline__ void wide_flush(WideSink &sk, bool pend, int link, int j, int kind) {
    const unsigned full = 0xffffffffu;
    if (!sk.ps || !__any_sync(full, pend)) return;
    if (sk.slot < 0 && !sk.full) {
        int s = -1;
        if ((threadIdx.x & 31) == 0) s = alloc_record(sk.ps);
        sk.slot = __shfl_sync(full, s, 0);
        sk.full = sk.slot < 0;
    }
    bool f = false;
    if (pend) f = sk.slot < 0 || !push_pair(sk.ps, sk.slot, link, j, kind);
    sk.full = sk.full || __any_sync(full, f);
}

template <int MODE, typename T>
__device__ __forceinline__ void wide_drain_bool(const uint32_t *q, int nitems, const SortedView<T> &ob, const Num<T> &nm,
                                                const T *A, const T *B, T r, T rn, int i, WideSink &sk, bool &hit,
                                                bool &unc) {
    typedef typename PolOf<MODE>::type P;
    const int lane = threadIdx.x & 31;
    bool c = false, u = false;
    int j = 0;
    if (lane < nitems) {
        const int s = (int)q[lane];
        T o[6];
        ob.box(s, o);
        const RB rr = coll_box_call<T, P>(nm, A, B, r, rn, o);
        j = (int)(ob.idx[s] & ~kGroundBit);
        if (P::robust && rr.m < kDecide) u = true;
        else c = rr.v;
    }
    hit = hit || __any_sync(0xffffffffu, c);
    unc = unc || __any_sync(0xffffffffu, u);
    wide_flush(sk, u, i, j, 0);
}

template <int MODE, typename T>
__device__ __forceinline__ void wide_drain_dist(const uint32_t *q, int nitems, const DevRobot &rb, const SortedView<T> &ob,
                                                const Num<T> &nm, const T *A, const T *B, int i, WideSink &sk,
                                                typename Key<T>::type &lkey, int &hj, T &hv, bool &unc) {
    typedef typename Key<T>::type K;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    K kk = Key<T>::of(nm.maxd);
    int jj = 0x7fffffff;
    T vv = T(0);
    bool u = false;
    int j = 0;
    if (lane < nitems) {
        const int s = (int)q[lane];
        bool settled;
        const T d = pair_distance<MODE, T>(rb, ob, nm, A, B, i, s, settled);
        j = (int)(ob.idx[s] & ~kGroundBit);
        if (!settled) {
            u = true;
        } else if (d == d) {   // the reference's std::min ignores NaN
            kk = Key<T>::of(d);
            if (d <= T(0)) { jj = j; vv = d; }
        }
    }
    wide_flush(sk, u, i, j, 1);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const K ok = __shfl_xor_sync(full, kk, off);
        kk = ok < kk ? ok : kk;
        const int oj = __shfl_xor_sync(full, jj, off);
        const T ov = __shfl_xor_sync(full, vv, off);
        if (oj < jj) { jj = oj; vv = ov; }
    }
    lkey = kk < lkey ? kk : lkey;
    if (jj < hj) { hj = jj; hv = vv; }
    unc = unc || __any_sync(full, u);
}

// ---------------------------------------------------------------------------
// isValid and / or computeDistance without the per-link profile, for the G
// configurations of a warp at once.  Neither output depends on the order in
// which links and pairs are visited (isValid is an OR, the distance a minimum
// over all pairs with any hit giving 0), so seeds and candidate pairs of all
// G configurations share two queues, and drains stay full even when each
// configuration has few candidates:
//   seeds : for each (configuration, link), the obstacle with the smallest
//           gap in the link's nearest leaf; their settled distances give each
//           configuration its first threshold;
//   main  : for each (configuration, link), one leaf cull against both
//           thresholds (r*sqrt(2) for isValid; best + r + EQUALITY_THRESHOLD
//           + margin, bounded by the leaf's tolerances, for the distance),
//           obstacle tests of up to four leaves at a time, and items pushed to
//           the isValid and distance queues, each drained 32 at a time;
//           configurations already settled are skipped.  Per
// configuration the warp keeps, in shared memory, its flags, the ordered key
// of its settled minimum, a settled hit and its pair-recheck record; drains
// update them with shared atomics.  Items: g << 21 | link << 16 | slot.
template <typename T> struct MultiState {
    int flags[32];                        // bit0 collision, bit1 / bit2 unsettled isValid / distance pair, bit3 list full
    typename Key<T>::type best[32];       // ordered key of the settled minimum
    int hit_link[32];                     // a link with a settled hit (-1: none)
    int hit_j[32];
    int slot[32];                         // pair-recheck record (-1: none yet)
    int need[32];
    uint32_t pend[32];                    // drain lane's unsettled pair: 1 << 31 | kind << 30 | j << 10 | link << 5 | g
    uint32_t qb[64], qd[64];
};

template <int MODE, typename T>
__device__ __forceinline__ void multi_flush(MultiState<T> &ms, const PairSink *ps) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t pe = ms.pend[lane];
    if (!__any_sync(full, pe != 0u)) return;
    const int g = (int)(pe & 31u);
    if (pe) ms.need[g] = 1;
    __syncwarp();
    if (ms.need[lane]) {
        ms.need[lane] = 0;
        if (ms.slot[lane] < 0 && !(ms.flags[lane] & 8)) {
            const int sl = alloc_record(ps);
            if (sl >= 0) ms.slot[lane] = sl;
            else atomicOr(&ms.flags[lane], 8);
        }
    }
    __syncwarp();
    if (pe) {
        const int sl = ms.slot[g];
        const int link = (int)((pe >> 5) & 31u), j = (int)((pe >> 10) & 2047u), kind = (int)((pe >> 30) & 1u);
        if (sl < 0 || !push_pair(ps, sl, link, j, kind)) atomicOr(&ms.flags[g], 8);
    }
    __syncwarp();
}

// FLAT: the collision tree with its rectangle test inlined (kernels without the distance tree).
template <int MODE, typename T, bool FLAT = false>
__device__ __forceinline__ void multi_drain_bool(MultiState<T> &ms, int nitems, const DevRobot &rb,
                                                 const SortedView<T> &ob, const Num<T> &nm, const T *pts, int stride,
                                                 const PairSink *ps) {
    typedef typename PolOf<MODE>::type P;
    const int lane = threadIdx.x & 31;
    uint32_t pe = 0u;
    if (lane < nitems) {
        const uint32_t it = ms.qb[lane];
        const int g = (int)(it >> 21), link = (int)((it >> 16) & 31u), s = (int)(it & 0xffffu);
        const T *A = pts + g * stride + 3 * link;
        T o[6];
        ob.box(s, o);
        const RB rr = coll_box_call<T, P, FLAT>(nm, A, A + 3, LinkConst<T>::r(rb, link), LinkConst<T>::rn(rb, link), o);
        if (P::robust && rr.m < kDecide) {
            atomicOr(&ms.flags[g], 2);
            pe = 0x80000000u | ((ob.idx[s] & 2047u) << 10) | ((uint32_t)link << 5) | (uint32_t)g;
        } else if (rr.v) {
            atomicOr(&ms.flags[g], 1);
        }
    }
    __syncwarp();
    if (ps) {
        ms.pend[lane] = pe;
        __syncwarp();
        multi_flush<MODE, T>(ms, ps);
    }
}

template <int MODE, typename T>
__device__ __forceinline__ void multi_drain_dist(MultiState<T> &ms, int nitems, const DevRobot &rb,
                                                 const SortedView<T> &ob, const Num<T> &nm, const T *pts, int stride,
                                                 const PairSink *ps) {
    const int lane = threadIdx.x & 31;
    uint32_t pe = 0u;
    if (lane < nitems) {
        const uint32_t it = ms.qd[lane];
        const int g = (int)(it >> 21), link = (int)((it >> 16) & 31u), s = (int)(it & 0xffffu);
        const T *A = pts + g * stride + 3 * link;
        bool settled;
        const T d = pair_distance<MODE, T>(rb, ob, nm, A, A + 3, link, s, settled);
        const uint32_t j = ob.idx[s] & ~kGroundBit;
        if (!settled) {
            atomicOr(&ms.flags[g], 4);
            pe = 0x80000000u | 0x40000000u | ((j & 2047u) << 10) | ((uint32_t)link << 5) | (uint32_t)g;
        } else if (d == d) {   // the reference's std::min ignores NaN
            atomicMin(&ms.best[g], Key<T>::of(d));
            if (d <= T(0) && atomicCAS(&ms.hit_link[g], -1, link) == -1) ms.hit_j[g] = (int)j;
        }
    }
    __syncwarp();
    if (ps) {
        ms.pend[lane] = pe;
        __syncwarp();
        multi_flush<MODE, T>(ms, ps);
    }
}

// Checks configurations 0..G-1 (skeletons at pts + g * stride) for isValid
// and / or the distance; 'live' marks the configurations to check.  On return
// lane g < G holds configuration g's results: *valid (0 / 1), *dist, the
// status (kSettled / kPairs / kFull), its record and first settled hit.
// KIND 1: isValid only, fixed at compile time (the edge checks), so the
// distance tree and its queue compile away and the collision tree is FLAT.
template <int MODE, typename T, int KIND = 0>
__device__ void wide_multi_np(MultiState<T> &ms, const DevRobot &rb, const SortedView<T> &ob, const T *pts,
                              int stride, int G, unsigned live, const Num<T> &nm, Want w_in, const PairSink *ps,
                              uint8_t &valid, double &dist, int &status, int &slot, int &hit_link, int &hit_j) {
    const Want w{w_in.valid, KIND == 1 ? false : w_in.dist, w_in.profile};
    constexpr bool kFlat = KIND == 1;
    typedef typename Key<T>::type K;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const T inf = T(1) / T(0);
    const int L = rb.D;
    const T dmargin = (MODE == 2) ? T(kBand) : LinkConst<T>::margin();
    ms.flags[lane] = 0;
    ms.best[lane] = Key<T>::of(nm.maxd);
    ms.hit_link[lane] = -1;
    ms.hit_j[lane] = 0x7fffffff;
    ms.slot[lane] = -1;
    ms.need[lane] = 0;
    ms.pend[lane] = 0u;
    __syncwarp();
    int nqb = 0, nqd = 0;
    // ------------------------------------------------------------- seeds
    if (w.dist) {
        for (int g = 0; g < G; ++g) {
            if (!((live >> g) & 1u)) continue;
            const T *pg = pts + g * stride;
            for (int i = 0; i < L; ++i) {
                T lo[3], hi[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const T a = pg[3 * i + k], b = pg[3 * i + 3 + k];
                    lo[k] = a < b ? a : b;
                    hi[k] = a < b ? b : a;
                }
                const bool gskip = i < rb.ground_included;
                T gb = inf;
                int lb = 0x7fffffff;
                for (int l = lane; l < ob.nb; l += 32) {
                    if (gskip && ob.ground_leaf(l)) continue;
                    T o[6];
                    ob.leaf(l, o);
                    const T gg = gap2_bb(lo, hi, o);
                    if (gg < gb || lb == 0x7fffffff) { gb = gg; lb = l; }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const T og = __shfl_xor_sync(full, gb, off);
                    const int ol = __shfl_xor_sync(full, lb, off);
                    if (og < gb || (!(gb < og) && ol < lb)) { gb = og; lb = ol; }
                }
                if (lb == 0x7fffffff) continue;
                const int sidx = lb * kLeaf + (lane & (kLeaf - 1));
                const uint32_t id = ob.idx[sidx];
                T gg = inf;
                if (id != kPadIdx && !(gskip && (id & kGroundBit))) {
                    T o[6];
                    ob.box(sidx, o);
                    gg = gap2_bb(lo, hi, o);
                }
                int sb = (gg < inf) ? sidx : 0x7fffffff;
#pragma unroll
                for (int off = kLeaf / 2; off > 0; off >>= 1) {
                    const T og = __shfl_xor_sync(full, gg, off);
                    const int os = __shfl_xor_sync(full, sb, off);
                    if (og < gg || (!(gg < og) && os < sb)) { gg = og; sb = os; }
                }
                if (sb == 0x7fffffff) continue;
                wide_push<MODE, T>(ms.qd, nqd, lane == 0, ((uint32_t)g << 21) | ((uint32_t)i << 16) | (uint32_t)sb);
                if (nqd >= 32) {
                    multi_drain_dist<MODE, T>(ms, 32, rb, ob, nm, pts, stride, ps);
                    wide_pop32(ms.qd, nqd);
                }
            }
        }
        if (nqd > 0) multi_drain_dist<MODE, T>(ms, nqd, rb, ob, nm, pts, stride, ps);
        nqd = 0;
        __syncwarp();
    }
    // -------------------------------------------------------------- main
    for (int g = 0; g < G; ++g) {
        if (!((live >> g) & 1u)) continue;
        const T *pg = pts + g * stride;
        for (int i = 0; i < L; ++i) {
            const bool need_b = w.valid && !(ms.flags[g] & 1);
            const bool need_d = w.dist && ms.hit_link[g] < 0;
            if (!need_b && !need_d) break;
            T lo[3], hi[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const T a = pg[3 * i + k], b = pg[3 * i + 3 + k];
                lo[k] = a < b ? a : b;
                hi[k] = a < b ? b : a;
            }
            const T r = LinkConst<T>::r(rb, i);
            const bool gskip = i < rb.ground_included;
            const T tb = r * T(1.41421356237309515) + BoolMargin<MODE, T>::m();
            const T tb2 = tb * tb;
            const T slack = r + nm.eq + dmargin;
            const T best = Key<T>::value(ms.best[g]);
            for (int l0 = 0; l0 < ob.nb; l0 += 32) {
                const int l = l0 + lane;
                bool cl = false;
                if (l < ob.nb && !(gskip && ob.ground_leaf(l))) {
                    T o[6];
                    ob.leaf(l, o);
                    const T gg = gap2_bb(lo, hi, o);
                    const bool cb = need_b && !(gg > tb2);
                    bool cd = false;
                    if (need_d) {
                        const T smax = smin(best, (T)ob.blk[l * kBlkRec + 6]) + slack;
                        const T slo = smin(best, (T)ob.blk[l * kBlkRec + 7]) + slack;
                        cd = !(slo > T(0) && gg > smax * smax);
                    }
                    cl = cb || cd;
                }
                unsigned ml = __ballot_sync(full, cl);
                while (ml != 0u) {
                    const int bit = nth_bit(ml, lane >> 3);
                    ml = drop4(ml);
                    bool pb = false, pd = false;
                    uint32_t item = 0u;
                    if (bit >= 0) {
                        const int sidx = (l0 + bit) * kLeaf + (lane & (kLeaf - 1));
                        const uint32_t id = ob.idx[sidx];
                        item = ((uint32_t)g << 21) | ((uint32_t)i << 16) | (uint32_t)sidx;
                        if (id != kPadIdx && !(gskip && (id & kGroundBit))) {
                            T o[6];
                            ob.box(sidx, o);
                            const T g2 = gap2_bb(lo, hi, o);
                            pb = need_b && !(g2 > tb2);
                            if (need_d) {
                                const T sv = smin(best, ob.tol(sidx)) + slack;
                                pd = !(sv > T(0) && g2 > sv * sv);
                            }
                        }
                    }
                    if (need_b) {
                        wide_push<MODE, T>(ms.qb, nqb, pb, item);
                        if (nqb >= 32) {
                            multi_drain_bool<MODE, T, kFlat>(ms, 32, rb, ob, nm, pts, stride, ps);
                            wide_pop32(ms.qb, nqb);
                        }
                    }
                    if (need_d) {
                        wide_push<MODE, T>(ms.qd, nqd, pd, item);
                        if (nqd >= 32) {
                            multi_drain_dist<MODE, T>(ms, 32, rb, ob, nm, pts, stride, ps);
                            wide_pop32(ms.qd, nqd);
                        }
                    }
                }
            }
        }
    }
    if (nqb > 0) multi_drain_bool<MODE, T, kFlat>(ms, nqb, rb, ob, nm, pts, stride, ps);
    if (nqd > 0) multi_drain_dist<MODE, T>(ms, nqd, rb, ob, nm, pts, stride, ps);
    __syncwarp();
    // ---- results of configuration 'lane'
    const int fl = ms.flags[lane];
    const bool collided = fl & 1;
    hit_link = ms.hit_link[lane];
    hit_j = ms.hit_j[lane];
    slot = ms.slot[lane];
    valid = collided ? 0 : 1;
    dist = hit_link >= 0 ? 0.0 : (double)Key<T>::value(ms.best[lane]);
    const bool bad_b = w.valid && !collided && (fl & 2);
    const bool bad_d = w.dist && (fl & 4) && hit_link < 0;
    status = !(bad_b || bad_d) ? kSettled : ((ps && slot >= 0 && !(fl & 8)) ? kPairs : kFull);
    (void)sizeof(K);
}

// One configuration, the whole warp.  pts = skeleton points [(D+1)][3];
// gl = per-warp scratch of nb leaf gaps.  Returns kSettled, kPairs or kFull
// (always kSettled for the exact forms) and the first settled hit (link,
// original obstacle index); lane 0 writes the outputs.
template <int MODE, typename T>
__device__ int wide_config(uint32_t *q, T *gl, const DevRobot &rb, const SortedView<T> &ob, const T *pts,
                           const Num<T> &nm, Want w, uint8_t *valid_out, double *dist_out, float *prof_out,
                           WideSink &sk, int &hit_link, int &hit_j) {
    typedef typename Key<T>::type K;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const T inf = T(1) / T(0);
    bool need_b = w.valid, need_d = w.dist || w.profile;
    bool collided = false, unc_b = false, unc_d = false;
    T best = nm.maxd;
    int hit = -1;
    hit_j = 0x7fffffff;
    const int L = rb.D;
    const int kspan = (ob.nb + 31) / 32;   // leaf slices of 32
    const T dmargin = (MODE == 2) ? T(kBand) : LinkConst<T>::margin();
    for (int i = 0; i < L && (need_b || need_d); ++i) {
        T A[3], B[3], lo[3], hi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            A[k] = pts[3 * i + k];
            B[k] = pts[3 * (i + 1) + k];
            lo[k] = A[k] < B[k] ? A[k] : B[k];
            hi[k] = A[k] < B[k] ? B[k] : A[k];
        }
        const T r = LinkConst<T>::r(rb, i);
        const bool gskip = i < rb.ground_included;
        // ---------------------------------------------------------- isValid
        if (need_b) {
            const T tb = r * T(1.41421356237309515) + BoolMargin<MODE, T>::m();
            const T tb2 = tb * tb;
            const T rn = LinkConst<T>::rn(rb, i);
            bool hb = false, ub = false;
            int nq = 0;
            for (int l0 = 0; l0 < ob.nb && !hb; l0 += 32) {
                const int l = l0 + lane;
                bool cl = false;
                if (l < ob.nb && !(gskip && ob.ground_leaf(l))) {
                    T o[6];
                    ob.leaf(l, o);
                    cl = !(gap2_bb(lo, hi, o) > tb2);
                }
                unsigned ml = __ballot_sync(full, cl);
                while (ml != 0u && !hb) {
                    const int bit = nth_bit(ml, lane >> 3);
                    ml = drop4(ml);
                    bool c = false;
                    int s = 0;
                    if (bit >= 0) {
                        s = (l0 + bit) * kLeaf + (lane & (kLeaf - 1));
                        const uint32_t id = ob.idx[s];
                        if (id != kPadIdx && !(gskip && (id & kGroundBit))) {
                            T o[6];
                            ob.box(s, o);
                            c = !(gap2_bb(lo, hi, o) > tb2);
                        }
                    }
                    wide_push<MODE, T>(q, nq, c, (uint32_t)s);
                    if (nq >= 32) {
                        wide_drain_bool<MODE, T>(q, 32, ob, nm, A, B, r, rn, i, sk, hb, ub);
                        wide_pop32(q, nq);
                    }
                }
            }
            if (nq > 0 && !hb) wide_drain_bool<MODE, T>(q, nq, ob, nm, A, B, r, rn, i, sk, hb, ub);
            __syncwarp();
            if (hb) { collided = true; need_b = false; }
            else if (ub) unc_b = true;
        }
        // --------------------------------------------------------- distance
        if (need_d) {
            const T hunt = r + nm.eq + dmargin;   // a gap above this cannot be a hit
            K lkey = Key<T>::of(nm.maxd);
            int hj = 0x7fffffff;
            T hv = T(0);
            bool ud = false;
            unsigned todo = 0u;
            for (int k = 0; k < kspan; ++k) {
                const int l = lane + 32 * k;
                if (l < ob.nb) {
                    T g = inf;
                    if (!(gskip && ob.ground_leaf(l))) {
                        T o[6];
                        ob.leaf(l, o);
                        g = gap2_bb(lo, hi, o);
                        todo |= 1u << k;
                    }
                    gl[l] = g;
                }
            }
            __syncwarp();
            int nq = 0;
            bool stop = false;
            while (!stop) {
                const bool hunting = hj != 0x7fffffff;
                const T thr0 = w.profile ? Key<T>::value(lkey) : smin(best, Key<T>::value(lkey));
                // prune (thresholds only shrink, so a pruned leaf stays pruned) and find the nearest live leaf
                T gmin = inf;
                for (int k = 0; k < kspan; ++k) {
                    if (!((todo >> k) & 1u)) continue;
                    const int l = lane + 32 * k;
                    const T g = gl[l];
                    bool alive;
                    if (hunting) {
                        alive = !(g > hunt * hunt);
                    } else {
                        const T smax = smin(thr0, (T)ob.blk[l * kBlkRec + 6]) + r + nm.eq + dmargin;
                        const T slo = smin(thr0, (T)ob.blk[l * kBlkRec + 7]) + r + nm.eq + dmargin;
                        alive = !(slo > T(0) && g > smax * smax);
                    }
                    if (!alive) todo &= ~(1u << k);
                    else if (g < gmin) gmin = g;
                }
                if (!__any_sync(full, todo != 0u)) break;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const T o = __shfl_xor_sync(full, gmin, off);
                    gmin = o < gmin ? o : gmin;
                }
                // this band: live leaves with gap <= 2 * nearest gap + 2 (r + eq + margin)
                const T gb = hunting ? inf : T(2) * sqrt(gmin) + T(2) * (r + nm.eq + dmargin);
                const T gb2 = gb * gb;
                unsigned band = 0u;
                for (int k = 0; k < kspan; ++k)
                    if (((todo >> k) & 1u) && !(gl[lane + 32 * k] > gb2)) band |= 1u << k;
                todo &= ~band;
                for (int k = 0; k < kspan && !stop; ++k) {
                    unsigned ml = __ballot_sync(full, (band >> k) & 1u);
                    while (ml != 0u && !stop) {
                        const int bit = nth_bit(ml, lane >> 3);
                        ml = drop4(ml);
                        bool c = false;
                        int s = 0;
                        if (bit >= 0) {
                            s = (bit + 32 * k) * kLeaf + (lane & (kLeaf - 1));
                            const uint32_t id = ob.idx[s];
                            if (id != kPadIdx && !(gskip && (id & kGroundBit))) {
                                T o[6];
                                ob.box(s, o);
                                const T g2 = gap2_bb(lo, hi, o);
                                if (hunting) {
                                    c = w.profile && (int)(id & ~kGroundBit) < hj && !(g2 > hunt * hunt);
                                } else {
                                    const T sv = smin(thr0, ob.tol(s)) + r + nm.eq + dmargin;
                                    c = !(sv > T(0) && g2 > sv * sv);
                                }
                            }
                        }
                        wide_push<MODE, T>(q, nq, c, (uint32_t)s);
                        if (nq >= 32) {
                            wide_drain_dist<MODE, T>(q, 32, rb, ob, nm, A, B, i, sk, lkey, hj, hv, ud);
                            wide_pop32(q, nq);
                            stop = hj != 0x7fffffff && !w.profile;   // the distance is 0 whatever else is found
                        }
                    }
                }
                if (nq > 0 && !stop) wide_drain_dist<MODE, T>(q, nq, rb, ob, nm, A, B, i, sk, lkey, hj, hv, ud);
                nq = 0;
                __syncwarp();
                if (hj != 0x7fffffff && !w.profile) stop = true;
            }
            __syncwarp();
            if (ud) unc_d = true;
            if (hj != 0x7fffffff) {
                // the partial minimum at the first hit is the hit's own value
                hit = i;
                hit_j = hj;
                need_d = false;
                if (w.profile && lane == 0) prof_out[i] = (float)hv;
            } else {
                const T lmin = Key<T>::value(lkey);
                if (w.profile && lane == 0) prof_out[i] = (float)lmin;
                best = smin(best, lmin);
            }
        }
    }
    if (lane == 0) {
        if (w.profile && hit >= 0)
            for (int k = hit + 1; k < L; ++k) prof_out[k] = 0.f;
        if (w.valid) *valid_out = collided ? 0 : 1;
        if (w.dist) *dist_out = (hit >= 0) ? 0.0 : (double)best;
    }
    hit_link = hit;
    const bool bad_b = w.valid && !collided && unc_b;
    const bool bad_d = (w.dist || w.profile) && unc_d && (w.profile || hit < 0);
    if (!(bad_b || bad_d)) return kSettled;
    return (sk.ps && sk.slot >= 0 && !sk.full) ? kPairs : kFull;
}

// Shared-memory layout of the wide kernels: robot, sorted rows, index row,
// block records, per-warp skeleton buffers.  Every piece is a multiple of 16
// bytes (ns is a multiple of 32).
struct WideLayout {
    uint32_t rows, idx, blk, pts, gl, gl_warp, total;
    RPM_HD static WideLayout of(int mode, int ns, int nb) {
        WideLayout l;
        const uint32_t tsz = mode == RPM_PREC_FP64 ? 8u : 4u;
        l.rows = (uint32_t)sizeof(DevRobot);
        l.idx = l.rows + 7u * (uint32_t)ns * tsz;
        l.blk = l.idx + 4u * (uint32_t)ns;
        l.pts = l.blk + 4u * kBlkRec * (uint32_t)nb;
        l.gl = l.pts + kWideWarps * kWidePtsBytes;
        l.gl_warp = ((uint32_t)nb * tsz + 15u) & ~15u;
        l.total = l.gl + kWideWarps * l.gl_warp;
        return l;
    }
};

// Stage the robot and the sorted scene of 'sg' (all threads wait).
template <int MODE>
__device__ __forceinline__ bool wide_stage(const Seg &sg, const WideLayout &L, unsigned char *smem, uint64_t *bar,
                                           int32_t *status) {
    if (threadIdx.x == 0) {
        const uint32_t rb = (uint32_t)sizeof(DevRobot);
        const uint32_t rows = L.idx - L.rows, idx = L.blk - L.idx, blk = L.pts - L.blk;
        bulk_expect(bar, rb + rows + idx + blk);
        bulk_copy(bar, smem, sg.robot, rb);
        if (MODE == 0) bulk_copy(bar, smem + L.rows, sg.srt_d, rows);
        else bulk_copy(bar, smem + L.rows, sg.srt_f, rows);
        bulk_copy(bar, smem + L.idx, sg.srt_f + (size_t)7 * sg.ns, idx);
        bulk_copy(bar, smem + L.blk, sg.blk, blk);
    }
    return bulk_wait(bar, 0, status);
}

// Body of k_check_wide<MODE>: CTA = kWideWarps warps, each owning G = P.wide_g
// consecutive configurations of one segment.
template <int MODE>
__device__ __forceinline__ void wide_kernel_body(const KParams &P, unsigned char *smem, uint64_t *bar,
                                                 MultiState<typename std::conditional<MODE == 0, double, float>::type> *ms,
                                                 int s) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    const Seg &sg = P.segs[s];
    const WideLayout L = WideLayout::of(MODE == 0 ? RPM_PREC_FP64 : RPM_PREC_FP32_REF, sg.ns, sg.nb);
    if (!wide_stage<MODE>(sg, L, smem, bar, P.status)) return;
    const DevRobot &rb = *reinterpret_cast<const DevRobot *>(smem);
    SortedView<T> ob{reinterpret_cast<const T *>(smem + L.rows), reinterpret_cast<const uint32_t *>(smem + L.idx),
                     reinterpret_cast<const float *>(smem + L.blk), sg.ns, sg.nb};
    const unsigned full = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int G = P.wide_g;
    const int D = rb.D;
    const int64_t c0 = (int64_t)(blockIdx.x - sg.first_block) * (kWideWarps * G) + (int64_t)warp * G;
    if (c0 >= sg.count) return;   // whole warp idle
    T *pts = reinterpret_cast<T *>(smem + L.pts + warp * kWidePtsBytes);
    T *gl = reinterpret_cast<T *>(smem + L.gl + warp * L.gl_warp);
    // forward kinematics, lane = configuration
    if (lane < G && c0 + lane < sg.count) {
        SkelWalker<MODE> sw;
        sw.begin();
        const float *q = sg.q + (c0 + lane) * D;
        T *p = pts + lane * (D + 1) * 3;
        for (int k = 0; k <= D; ++k) sw.point(rb, q, k, p + 3 * k);
    }
    __syncwarp();
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    const Want w{sg.valid != nullptr, sg.dist != nullptr, sg.profile != nullptr};
    if (!w.profile) {
        const int n = (int)min((int64_t)G, sg.count - c0);
        uint8_t v;
        double d;
        int st, slot, hl, hj;
        wide_multi_np<MODE, T>(ms[warp], rb, ob, pts, (D + 1) * 3, n, n >= 32 ? full : ((1u << n) - 1u), nm, w,
                               MODE == 2 ? &P.ps : nullptr, v, d, st, slot, hl, hj);
        if (lane < n) {
            const int64_t c = c0 + lane;
            if (w.valid) sg.valid[c] = v;
            if (w.dist) sg.dist[c] = d;
            if (MODE == 2) {
                complete_record(&P.ps, slot, st, s, c, hl, hj);
                if (st == kFull) recheck_whole(P, s, c);
            }
        }
        return;
    }
    uint32_t *wq = ms[warp].qb;   // 128 contiguous entries: qb then qd
    for (int g = 0; g < G; ++g) {
        const int64_t c = c0 + g;
        if (c >= sg.count) break;
        WideSink sk{MODE == 2 ? &P.ps : nullptr, -1, false};
        int hl, hj;
        const T *pc = pts + g * (D + 1) * 3;
        const int st = wide_config<MODE, T>(wq, gl, rb, ob, pc, nm, w, w.valid ? sg.valid + c : nullptr,
                                            w.dist ? sg.dist + c : nullptr, sg.profile + c * D, sk, hl, hj);
        if (MODE == 2 && lane == 0) {
            complete_record(&P.ps, sk.slot, st, s, c, hl, hj);
            if (st == kFull) recheck_whole(P, s, c);
        }
    }
}

// Body of k_edges_wide<MODE>.  Batches with fewer edges than about two per
// stream check all their checks in parallel (flat mode below); larger ones
// run edge streams: each warp runs G edge streams.  A stream owns
// one edge and walks its checks in the reference's order (k = n_e down to 1);
// every round the warp checks the current check of all its streams together
// (one forward kinematics per lane, shared queues).  A settled collision at k
// sets the edge's largest colliding k and ends the stream (the reference
// stops there); a check left to the FP64 recheck does not stop it, since a
// collision further down still has to be found.  Finished streams take the
// next edge from a global counter.  The pass covers the warp-layout segments
// (edges from edge_split on); lanes of different segments are checked one
// segment at a time, each against its own robot and sorted scene (staged in
// shared memory when the pass has a single segment).
template <int MODE, bool MULTI>
__device__ __forceinline__ void edge_wide_body(const EdgeParams &P, unsigned char *smem, uint64_t *bar,
                                               MultiState<typename std::conditional<MODE == 0, double, float>::type> *ms) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    const int s_lo = P.nseg_lane;
    constexpr bool staged = !MULTI;   // one segment: its robot and sorted scene in shared memory
    const DevRobot *rb_st = nullptr;
    SortedView<T> ob_st{nullptr, nullptr, nullptr, 0, 0};
    uint32_t pts_off = 0;
    if (staged) {
        const Seg &sg = P.segs[s_lo].seg;
        const WideLayout L = WideLayout::of(MODE == 0 ? RPM_PREC_FP64 : RPM_PREC_FP32_REF, sg.ns, sg.nb);
        if (!wide_stage<MODE>(sg, L, smem, bar, P.status)) return;
        rb_st = reinterpret_cast<const DevRobot *>(smem);
        ob_st = SortedView<T>{reinterpret_cast<const T *>(smem + L.rows), reinterpret_cast<const uint32_t *>(smem + L.idx),
                              reinterpret_cast<const float *>(smem + L.blk), sg.ns, sg.nb};
        pts_off = L.pts;
    }
    const unsigned full = 0xffffffffu;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int G = P.wide_g;
    T *pts = reinterpret_cast<T *>(smem + pts_off + warp * kWidePtsBytes);
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    const int64_t e_lo = edge_split(P);
    // One segment's checks of the lanes in 'live' (skeletons first, then the
    // joint obstacle walk); returns this lane's outcome.
    auto check_seg = [&](int cur, bool mine, const float *q, uint8_t &v, int &st, int &slot) {
        const unsigned live = __ballot_sync(full, mine);
        const DevRobot &rb = staged ? *rb_st : *P.segs[cur].seg.robot;
        const Seg &sg = P.segs[cur].seg;
        const SortedView<T> ob = staged ? ob_st
                                        : SortedView<T>{MODE == 0 ? reinterpret_cast<const T *>(sg.srt_d)
                                                                  : reinterpret_cast<const T *>(sg.srt_f),
                                                        reinterpret_cast<const uint32_t *>(sg.srt_f + (size_t)7 * sg.ns),
                                                        sg.blk, sg.ns, sg.nb};
        const int D = P.segs[cur].D;
        if (mine) {
            SkelWalker<MODE> sw;
            sw.begin();
            T *p = pts + lane * (D + 1) * 3;
            for (int t = 0; t <= D; ++t) sw.point(rb, q, t, p + 3 * t);
        }
        __syncwarp();
        double dd;
        int hl, hj;
        wide_multi_np<MODE, T, 1>(ms[warp], rb, ob, pts, (D + 1) * 3, G, live, nm, Want{true, false, false},
                               MODE == 2 ? &P.ps : nullptr, v, dd, st, slot, hl, hj);
        __syncwarp();
        return live;
    };
    if (!P.streams) {
        // small batches: every check of every edge in parallel, G consecutive
        // flat checks (edge-major, k descending) per warp at a time
        const int64_t f_lo = flat_off(P, e_lo), f_hi = flat_off(P, P.E);
        for (;;) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&P.work[1], (unsigned long long)G);
            base = __shfl_sync(full, base, 0);
            if (f_lo + (int64_t)base >= f_hi) break;
            int64_t e = 0;
            int k = 0, s = 0;
            bool act = false;
            float q[kMaxDof];
            if (lane < G && f_lo + (int64_t)base + lane < f_hi) {
                const int64_t idx = f_lo + (int64_t)base + lane;
                e = edge_of_flat(P, idx, e_lo, P.E - 1);
                s = MULTI ? edge_seg(P, e) : s_lo;
                const int n = P.n_e[e];
                k = n - (int)(idx - flat_off(P, e));
                act = k > *(volatile int32_t *)&P.kmax[e];   // a check nearer q2 already collides
                if (act) {
                    const EdgeGeom gm = edge_geom(P, s, e);
                    edge_config(gm.a, gm.b, gm.D, n, k, gm.dist, q);
                }
            }
            unsigned todo = __ballot_sync(full, act);
            while (todo) {
                const int cur = MULTI ? __shfl_sync(full, s, __ffs(todo) - 1) : s_lo;
                const bool mine = MULTI ? (act && s == cur) : act;
                uint8_t v;
                int st, slot;
                todo &= ~check_seg(cur, mine, q, v, st, slot);
                if (mine) edge_outcome<MODE>(P, e, k, st, slot, v);
                if (!MULTI) break;
            }
        }
        return;
    }
    int64_t e = -1;      // this lane's edge (-1: none)
    int k = 0, n = 0, s = 0;   // its current check, check count and segment
    float dist = 0.f;
    bool more = true;    // edges left to take (warp-uniform)
    for (;;) {
        const bool need = lane < G && e < 0 && more;
        const unsigned nmask = __ballot_sync(full, need);
        if (nmask) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(&P.work[1], (unsigned long long)__popc(nmask));
            base = __shfl_sync(full, base, 0);
            if (need) {
                const int64_t idx = e_lo + (int64_t)base + __popc(nmask & ((1u << lane) - 1u));
                if (idx < P.E) {
                    e = idx;
                    s = MULTI ? edge_seg(P, e) : s_lo;
                    const EdgeGeom gm = edge_geom(P, s, e);
                    n = gm.n;
                    dist = gm.dist;
                    k = n;
                }
            }
            if (e_lo + (int64_t)base + __popc(nmask) >= P.E) more = false;
        }
        const bool has = lane < G && e >= 0;
        unsigned todo = __ballot_sync(full, has);
        if (todo == 0u) {
            if (!more) break;
            continue;
        }
        while (todo) {
            const int cur = MULTI ? __shfl_sync(full, s, __ffs(todo) - 1) : s_lo;
            const bool mine = MULTI ? (has && s == cur) : has;
            float q[kMaxDof];
            if (mine) {
                const EdgeSeg &es = P.segs[cur];
                edge_config(es.seg.q + (e - es.e0) * es.D, es.q2 + (e - es.e0) * es.D, es.D, n, k, dist, q);
            }
            uint8_t v;
            int st, slot;
            todo &= ~check_seg(cur, mine, q, v, st, slot);
            if (mine) {
                edge_outcome<MODE>(P, e, k, st, slot, v);
                if (st == kSettled && v == 0) e = -1;    // the reference's first collision: the edge is done
                else if (--k < 1) e = -1;                // every check clear (or left to the recheck)
            }
            if (!MULTI) break;
        }
    }
}
#endif

}  // namespace rpm
