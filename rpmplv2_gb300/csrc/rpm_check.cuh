// rpm_check.cuh -- per-configuration drivers of RealVectorSpace::isValid(q)
// (RealVectorSpace.cpp:277-309) and computeDistance(q) (:318-392).
//
// One thread owns one configuration: it walks the skeleton points in order
// (FK advanced lazily), and for link i runs over the obstacles j in the
// reference's i-major / j-minor order, so early exits and the distance
// profile's early-exit shape are exactly the reference's.
//
// Distance pruning: a pair whose bounding-box gap exceeds the current best
// (or the obstacle's min_dist_tol) by radius + EQUALITY_THRESHOLD + margin
// cannot lower the minimum or be a hit, so its exact distance is skipped.
// The result is unchanged; only work is saved.
#pragma once
#include "rpm_tree.cuh"

namespace rpm {

template <typename T> struct ObsView {
    const T *rows;        // [>=7][n_pad] : six AABB coordinates, min_dist_tol
    const float *ground;  // [n_pad] 1.0 for "ground"
    int n, n_pad;
    const float *frows = nullptr;   // FP64 form: the same rows in float (exact), for the float pre-test
    const float4 *aos = nullptr;    // FP32 pass: the float rows per obstacle as [n][8] (six coordinates,
                                    // min_dist_tol, ground), two 16-byte loads per obstacle
    RPM_HD void box(int j, T *o) const {
#pragma unroll
        for (int k = 0; k < 6; ++k) o[k] = rows[k * n_pad + j];
    }
    RPM_HD T tol(int j) const { return rows[kRowTol * n_pad + j]; }
    RPM_HD bool is_ground(int j) const { return ground[j] != 0.f; }
};

template <typename T> struct LinkConst;
template <> struct LinkConst<double> {
    RPM_HD static double r(const DevRobot &rb, int i) { return rb.radius_d[i]; }
    RPM_HD static double rn(const DevRobot &rb, int i) { return rb.rnew_d[i]; }
    RPM_HD static double margin() { return 1e-9; }
};
template <> struct LinkConst<float> {
    RPM_HD static float r(const DevRobot &rb, int i) { return rb.radius_f[i]; }
    RPM_HD static float rn(const DevRobot &rb, int i) { return rb.rnew_f[i]; }
    RPM_HD static float margin() { return 1e-5f; }
};

struct Want {
    bool valid, dist, profile;
};

// ---------------------------------------------------------------------------
// Pair-level FP64 recheck of the FP32 pass.  The FP32 pass folds only settled
// pairs into its outputs and running minima (a settled value is within the
// contact band of its FP64 value, so pruning on settled values stays exact)
// and lists every unsettled (record, link, obstacle, kind) pair.  A record is
// allocated at a configuration's first unsettled pair and completed when the
// configuration ends; only records completed with status kPairs are used.
// The FP64 kernels then run the forward kinematics of each such configuration,
// evaluate its listed pairs and fold their results into the outputs in the
// reference's link order.  Configurations whose pairs do not fit the lists are
// recomputed whole by the configuration-level recheck.
constexpr int kSettled = 0;      // outputs final
constexpr int kPairs = 1;        // outputs final after the pair recheck
constexpr int kFull = 2;         // recompute the whole configuration in FP64

struct PairCfg {
    int32_t status;              // kPairs when the pair recheck applies
    int32_t seg;                 // segment (edge checks: the check number k)
    int64_t config;              // index within its segment (edge checks: the edge)
    int32_t hit_link;            // link of the first settled hit (-1: none)
    int32_t hit_j;               // lowest obstacle index of a settled hit in that link
};

struct PairAcc {
    int lkey[kMaxDof];                    // ordered key of (float) FP64 link minimum
    unsigned long long hkey[kMaxDof];     // obstacle index << 32 | float bits, lowest-index FP64 hit per link
    long long dkey;                       // ordered key of the FP64 minimum over all links
    int coll;                             // an FP64 collision
    int pad;
};

struct PairSink {
    uint64_t *pairs;             // record << 17 | link << 12 | obstacle << 1 | kind (0 isValid, 1 distance)
    uint32_t *pair_count;
    uint32_t pair_cap;
    uint32_t cfg_cap;
    PairCfg *cfgs;
    uint32_t *cfg_count;
    double *skel;                // [cfg_cap][kMaxDof + 1][3]
    PairAcc *acc;                // [cfg_cap]
    int32_t seg_base;            // added to the launch's segment index in the records (several launches, one recheck)
    // evaluation order of the listed pairs (nullable: list order), sorted by
    // kind and by the regions of the segment's ends around the box (kPairKeys)
    uint32_t *key;               // [pair_cap]
    uint32_t *order;             // [pair_cap]
    uint32_t *hist;              // [kPairHist]: counts, then offsets, then a CTA counter
};

// Sort keys of listed pairs: kind (isValid, distance) x region of A x region
// of B (27 each: below, inside or above the box's slab on each axis), and a
// last bucket for pairs the evaluation skips.
constexpr uint32_t kPairKeys = 2 * 729 + 1;
constexpr uint32_t kPairHist = 2 * kPairKeys + 1;
// Batches from this many configurations recheck their pairs in key order.
constexpr int64_t kSortPairsMinConfigs = 65536;

#ifdef __CUDACC__
// A new record (status kSettled until completed), or -1 when the list is full.
__device__ __forceinline__ int alloc_record(const PairSink *ps) {
    const uint32_t s = atomicAdd(ps->cfg_count, 1u);
    if (s >= ps->cfg_cap) return -1;
    ps->cfgs[s].status = kSettled;
    return (int)s;
}

// Append an unsettled pair of record 'slot'; false when the list is full.
__device__ __forceinline__ bool push_pair(const PairSink *ps, int slot, int link, int j, int kind) {
    const uint32_t s = atomicAdd(ps->pair_count, 1u);
    if (s >= ps->pair_cap) return false;
    ps->pairs[s] = ((uint64_t)(uint32_t)slot << 17) | ((uint64_t)link << 12) | ((uint64_t)j << 1) | (uint64_t)kind;
    return true;
}

__device__ __forceinline__ void complete_record(const PairSink *ps, int slot, int status, int seg, int64_t config,
                                                int hit_link, int hit_j) {
    if (slot >= 0)
        ps->cfgs[slot] = PairCfg{status == kPairs ? kPairs : kSettled, seg + ps->seg_base, config, hit_link, hit_j};
}

// An unsettled pair found by a drain lane, waiting for its owner's record.
struct Pend {
    bool on;
    int owner, j, kind;
};
#endif
#if defined(RPM_MARGIN_DEBUG)
inline int g_dbg_site_b = 0, g_dbg_site_d = 0;   // host debugging only
#endif
#if defined(RPM_MARGIN_DEBUG) && !defined(__CUDA_ARCH__)
#define RPM_DBG_B(pol) (g_dbg_site_b = (pol).site)
#define RPM_DBG_D(pol) (g_dbg_site_d = (pol).site)
#else
#define RPM_DBG_B(pol) ((void)0)
#define RPM_DBG_D(pol) ((void)0)
#endif

#ifdef __CUDACC__
// One warp per configuration (used for the few configurations the FP32 pass
// leaves unsettled, so latency matters more than throughput).  Lanes split
// the obstacles of each link; the isValid OR, the per-link minimum and the
// first hit (lowest obstacle index with d <= 0) are warp reductions, which
// give exactly the sequential i-major / j-minor result.
template <int MODE, typename T>
__device__ void config_exact_warp(const DevRobot &rb, const ObsView<T> &ob, const float *q, const Num<T> &nm, Want w,
                                  uint8_t *valid_out, double *dist_out, float *prof_out) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    SkelWalker<MODE> sw;
    sw.begin();
    T A[3], B[3];
    sw.point(rb, q, 0, A);
    bool need_b = w.valid, need_d = w.dist || w.profile;
    bool collided = false;
    T best = nm.maxd;
    int hit = -1;
    const int L = rb.D;
    for (int i = 0; i < L && (need_b || need_d); ++i) {
        sw.point(rb, q, i + 1, B);
        const T r = LinkConst<T>::r(rb, i), rn = LinkConst<T>::rn(rb, i);
        const bool ground_skip = i < rb.ground_included;
        if (need_b) {
            bool mine = false;
            for (int j = lane; j < ob.n && !mine; j += 32) {
                if (ground_skip && ob.is_ground(j)) continue;
                T o[6];
                ob.box(j, o);
                mine = coll_box_call<T, ExactPol>(nm, A, B, r, rn, o).v;
            }
            if (__any_sync(full, mine)) { collided = true; need_b = false; }
        }
        if (need_d) {
            T lb = nm.maxd, hv = T(0);
            int hj = 0x7fffffff;
            for (int j = lane; j < ob.n; j += 32) {
                if (ground_skip && ob.is_ground(j)) continue;
                T o[6];
                ob.box(j, o);
                const T tol = ob.tol(j);
                T thr = w.profile ? lb : smin(best, lb);
                thr = smin(thr, tol);
                const T s = thr + r + nm.eq + LinkConst<T>::margin();
                if (s > T(0) && gap2(A, B, o) > s * s) continue;
                T d = capsule_box_call<T, ExactPol>(nm, A, B, r, o).v;
                if (d > tol) d = nm.maxd;
                lb = smin(lb, d);
                if (d <= T(0)) { hj = j; hv = d; break; }
            }
            int fj = hj;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) fj = min(fj, __shfl_xor_sync(full, fj, off));
            T lmin = lb;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const T other = __shfl_xor_sync(full, lmin, off);
                lmin = (other < lmin) ? other : lmin;
            }
            if (fj != 0x7fffffff) {
                const int owner = __ffs(__ballot_sync(full, hj == fj)) - 1;
                const T hval = __shfl_sync(full, hv, owner);
                hit = i;
                need_d = false;
                if (w.profile && lane == 0) prof_out[i] = (float)hval;
            } else {
                if (w.profile && lane == 0) prof_out[i] = (float)lmin;
                best = smin(best, lmin);
            }
        }
        A[0] = B[0]; A[1] = B[1]; A[2] = B[2];
    }
    if (lane == 0) {
        if (w.profile && hit >= 0)
            for (int k = hit + 1; k < L; ++k) prof_out[k] = 0.f;
        if (w.valid) *valid_out = collided ? 0 : 1;
        if (w.dist) *dist_out = (hit >= 0) ? 0.0 : (double)best;
    }
}
#endif

#ifdef __CUDACC__
// ---------------------------------------------------------------------------
// Warp-cooperative driver used by the batched kernels.
//
// A warp owns 32 configurations (lane = configuration) and walks the links in
// lockstep.  For link i every lane classifies obstacle j of its own
// configuration with the bounding-box gap alone:
//   * isValid : the reference's tree can return true only when some point of
//     the segment is within r*sqrt(2) of the box (the inner test reaches r,
//     the corner tests of :69-72 reach r*sqrt(2)), so a larger gap is a
//     settled 'no collision' and the tree is skipped;
//   * distance: a gap above min(best, min_dist_tol) + r + EQUALITY_THRESHOLD
//     cannot lower the minimum or be a hit (pruned).
// Pairs that need a tree go into one of two per-warp queues in shared memory;
// a queue is drained 32 entries at a time with every lane evaluating one
// pair, and results are combined per owner with shared-memory atomics:
// isValid by OR, the link minimum by an order-preserving integer min, the
// first hit by the minimum obstacle index.  These combine exactly as the
// sequential i-major / j-minor scan, so outputs are bit-identical to it.
// Order-preserving integer keys of T (for shared-memory atomicMin).
template <typename T> struct Key;
template <> struct Key<double> {
    typedef long long type;
    __device__ static long long of(double x) {
        const long long i = __double_as_longlong(x);
        return i >= 0 ? i : i ^ 0x7fffffffffffffffLL;
    }
    __device__ static double value(long long i) { return __longlong_as_double(i >= 0 ? i : i ^ 0x7fffffffffffffffLL); }
};
template <> struct Key<float> {
    typedef int type;
    __device__ static int of(float x) {
        const int i = __float_as_int(x);
        return i >= 0 ? i : i ^ 0x7fffffff;
    }
    __device__ static float value(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }
};

template <typename T> struct WarpShared {
    T a[32][3], b[32][3];                // current link's segment per owner lane
    typename Key<T>::type lmin[32];      // ordered key of the link minimum of d'
    int hitj[32];                        // lowest obstacle index with a settled d' <= 0
    T hitv[32];                          // d' at that index
    int flags[32];                       // bit0 collision, bit1 isValid unsettled, bit2 distance unsettled
    int slot[32];                        // pair-recheck record per owner (-1: none yet)
    int need[32];                        // owner has pairs waiting for a record
    uint32_t pend[32];                   // drain lane's unsettled pair (pend_of)
    uint32_t qb[64], qd[64];             // queues: owner | j << 5 (| link << 16 in warp_check_any)
};

// Queue items and pending pairs: owner (bits 0-4) | obstacle << 5 (bits 5-15)
// | link << 16 (bits 16-20); a pending pair adds kind << 30 and bit 31.
__device__ __forceinline__ uint32_t pend_of(uint32_t item, int link, int kind) {
    return 0x80000000u | ((uint32_t)kind << 30) | ((uint32_t)link << 16) | (item & 0xffffu);
}

// After a drain: give every owner with waiting pairs a record, then list the
// pairs (an owner without a record, or a full pair list, marks bit 8).
template <typename T>
__device__ __forceinline__ void flush_pending(WarpShared<T> &sh, const PairSink *ps) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t pe = sh.pend[lane];
    const Pend pp{pe != 0u, (int)(pe & 31u), (int)((pe >> 5) & 2047u), (int)((pe >> 30) & 1u)};
    const int link = (int)((pe >> 16) & 31u);
    if (pp.on) sh.need[pp.owner] = 1;
    __syncwarp();
    if (sh.need[lane]) {
        sh.need[lane] = 0;
        if (sh.slot[lane] < 0 && !(sh.flags[lane] & 8)) {
            const int s = alloc_record(ps);
            if (s >= 0) sh.slot[lane] = s;
            else atomicOr(&sh.flags[lane], 8);
        }
    }
    __syncwarp();
    if (pp.on) {
        const int s = sh.slot[pp.owner];
        if (s < 0 || !push_pair(ps, s, link, pp.j, pp.kind)) atomicOr(&sh.flags[pp.owner], 8);
    }
    __syncwarp();
}

template <int MODE> struct PolOf { typedef ExactPol type; };
template <> struct PolOf<2> { typedef RobustPol type; };

template <int MODE, typename T> struct BoolMargin;
template <int MODE> struct BoolMargin<MODE, double> { __device__ static double m() { return 1e-9; } };
template <int MODE> struct BoolMargin<MODE, float> { __device__ static float m() { return MODE == 2 ? kDecide : 1e-5f; } };

// flags bits: 1 settled collision, 2 unsettled isValid pair, 4 unsettled
// distance pair (bits 1-4 per link), 8 pair list full (per configuration).
// FLAT: the isValid tree with its rectangle test inlined (coll_box), for
// kernels that run no distance tree.
template <int MODE, typename T, bool FLAT = false>
__device__ __forceinline__ void drain_bool(WarpShared<T> &sh, const DevRobot &rb, const ObsView<T> &ob, const Num<T> &nm,
                                           int i, int nitems, const PairSink *ps) {
    typedef typename PolOf<MODE>::type P;
    const int lane = threadIdx.x & 31;
    uint32_t pe = 0u;
    if (lane < nitems) {
        const uint32_t e = sh.qb[lane];
        const int owner = (int)(e & 31u), j = (int)(e >> 5);
        T o[6];
        ob.box(j, o);
        const RB rr = coll_box_call<T, P, FLAT>(nm, sh.a[owner], sh.b[owner], LinkConst<T>::r(rb, i),
                                                LinkConst<T>::rn(rb, i), o);
        const bool c = rr.v;
        if (P::robust && rr.m < kDecide) {
            atomicOr(&sh.flags[owner], 2);
            pe = pend_of(e, i, 0);
        } else if (c) {
            atomicOr(&sh.flags[owner], 1);
        }
    }
    if (ps) {
        sh.pend[lane] = pe;
        if (__any_sync(0xffffffffu, pe != 0u)) flush_pending(sh, ps);
    }
}

template <int MODE, typename T, typename V>
__device__ __forceinline__ T pair_distance(const DevRobot &rb, const V &ob, const Num<T> &nm, const T *A,
                                           const T *B, int i, int j, bool &settled) {
    typedef typename PolOf<MODE>::type P;
    T o[6];
    ob.box(j, o);
    const ValM<T> dv = capsule_box_call<T, P>(nm, A, B, LinkConst<T>::r(rb, i), o);
    const T tol = ob.tol(j);
    T d = dv.v;
    float m = dv.m;
    if (P::robust) {
        // the clamp to MAX_DISTANCE and the hit test are decisions on d too
        const float band = dv.ia * (kDecide / kBand);
        m = fminf(m, fabsf((float)(d - tol)) * band);
        if (d != T(0)) m = fminf(m, fabsf((float)(d > tol ? nm.maxd : d)) * band);
    }
    if (d > tol) d = nm.maxd;   // :367-368
    settled = !P::robust || m >= kDecide;
    return d;
}

template <int MODE, typename T, bool FLAT = false>
__device__ __forceinline__ void drain_dist(WarpShared<T> &sh, const DevRobot &rb, const ObsView<T> &ob, const Num<T> &nm,
                                           int i, int nitems, const PairSink *ps) {
    const int lane = threadIdx.x & 31;
    uint32_t pe = 0u;
    if (lane < nitems) {
        const uint32_t e = sh.qd[lane];
        const int owner = (int)(e & 31u), j = (int)(e >> 5);
        bool settled;
        const T d = pair_distance<MODE, T>(rb, ob, nm, sh.a[owner], sh.b[owner], i, j, settled);
        if (!settled) {
            atomicOr(&sh.flags[owner], 4);
            pe = pend_of(e, i, 1);
        } else if (d == d) {   // the reference's std::min ignores NaN
            atomicMin(&sh.lmin[owner], Key<T>::of(d));
            if (d <= T(0)) atomicMin(&sh.hitj[owner], j);
        }
        __syncwarp(__activemask());
        if (d <= T(0) && settled && sh.hitj[owner] == j) sh.hitv[owner] = d;   // one entry per (owner, j)
    }
    if (ps) {
        sh.pend[lane] = pe;
        if (__any_sync(0xffffffffu, pe != 0u)) flush_pending(sh, ps);
    }
}

// Lower bound of the segment-box distance from the segment's bounding box
// (lo, hi) and the box: the same arithmetic as gap2.
template <typename T> __device__ __forceinline__ T gap2_bb(const T *lo, const T *hi, const T *o) {
    T g2 = T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        T g = o[c] - hi[c];
        const T g2b = lo[c] - o[3 + c];
        g = g > g2b ? g : g2b;
        g = g > T(0) ? g : T(0);
        g2 = g2 + g * g;
    }
    return g2;
}

// Append this lane's item to a warp queue (positions by ballot rank) and
// drain the queue 32 entries at a time.  The ballot gates the rest: for most
// obstacles no lane of the warp queues a pair.  REFRESH reloads the lane's
// register copies of what the drain changes.
#define RPM_PUSH_AND_DRAIN(Q, N, want, item, DRAIN, REFRESH)                           \
    do {                                                                               \
        const unsigned m_ = __ballot_sync(0xffffffffu, (want));                         \
        if (m_ != 0u) {                                                                \
            if (want) sh.Q[(N) + __popc(m_ & lt_mask)] = (item);                       \
            (N) += __popc(m_);                                                         \
            if ((N) >= 32) {                                                           \
                __syncwarp();                                                          \
                DRAIN<MODE, T, kFlat>(sh, rb, ob, nm, i, 32, ps);                      \
                __syncwarp();                                                          \
                if (lane < (N) - 32) sh.Q[lane] = sh.Q[32 + lane];                     \
                (N) -= 32;                                                             \
                REFRESH;                                                               \
                __syncwarp();                                                          \
            }                                                                          \
        }                                                                              \
    } while (0)

// Returns, per lane, kSettled, kPairs or kFull (always kSettled for the exact
// forms); outputs of unsettled configurations are provisional.  With a pair
// sink, *slot receives the lane's record (-1: none) and *hit_link / *hit_j its
// first settled hit (link, obstacle); the caller completes the record.  Once a
// lane has a settled hit it only looks for an earlier hit (lower obstacle
// index), which is all the profile's first-hit semantics need.
// KIND fixes the outputs at compile time so the unused tree and its queue
// compile away: 0 = as 'w' says, 1 = isValid only, 2 = distance / profile
// only, 3 = distance only (no profile).
template <int MODE, typename T, int KIND = 0>
__device__ int warp_check(WarpShared<T> &sh, const DevRobot &rb, const ObsView<T> &ob, const float *q, bool active,
                          const Num<T> &nm, Want w_in, uint8_t *valid_out, double *dist_out, float *prof_out,
                          const PairSink *ps = nullptr, int *slot = nullptr, int *hit_link = nullptr,
                          int *hit_j = nullptr) {
    const Want w{(KIND == 2 || KIND == 3) ? false : w_in.valid, KIND == 1 ? false : w_in.dist,
                 (KIND == 1 || KIND == 3) ? false : w_in.profile};
    constexpr bool kFlat = KIND == 1;   // the isValid tree alone: its rectangle test inlined
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    SkelWalker<MODE> sw;
    sw.begin();
    T A[3] = {T(0), T(0), T(0)}, B[3] = {T(0), T(0), T(0)};
    if (active) sw.point(rb, q, 0, A);
    bool need_b = active && w.valid, need_d = active && (w.dist || w.profile);
    bool collided = false, unc_b = false, unc_d = false;
    T best = nm.maxd;
    int hit = -1, hit_obs = 0x7fffffff;
    const int L = rb.D;
    const T dmargin = (MODE == 2) ? T(kBand) : LinkConst<T>::margin();
    sh.flags[lane] = 0;
    sh.slot[lane] = -1;
    sh.need[lane] = 0;
    for (int i = 0; i < L; ++i) {
        if (!__any_sync(full, need_b || need_d)) break;
        if (active) sw.point(rb, q, i + 1, B);
        const T r = LinkConst<T>::r(rb, i);
        const T tb = r * T(1.41421356237309515) + BoolMargin<MODE, T>::m();
        const T tb2 = tb * tb;
        const T hunt = r + nm.eq + dmargin;          // a gap above this cannot be a hit
        const T hunt2 = hunt * hunt;
        const bool ground_skip = i < rb.ground_included;
        const bool dist_link = need_d;
        T lo[3], hi[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = A[k] < B[k] ? A[k] : B[k];
            hi[k] = A[k] < B[k] ? B[k] : A[k];
            sh.a[lane][k] = A[k];
            sh.b[lane][k] = B[k];
        }
        sh.lmin[lane] = Key<T>::of(nm.maxd);
        sh.hitj[lane] = 0x7fffffff;
        sh.hitv[lane] = T(0);
        // FP64 form: a float pre-test of each pair's gap, from the segment box
        // rounded outwards and thresholds raised by 1e-5 m, so the FP64 gap and
        // threshold arithmetic below runs only for pairs near one of its
        // decisions.  A pair the pre-test passes over is one the FP64 test
        // passes over too (the float gap errs by under 1e-6 m), so the queued
        // pairs, and the outputs, are the same.
        float lof[3] = {0.f, 0.f, 0.f}, hif[3] = {0.f, 0.f, 0.f};
        float tbf2 = 0.f, huntf2 = 0.f, slackf = 0.f, bestf = 0.f;
        const bool pre = (MODE == 0) && ob.frows != nullptr;
        if constexpr (MODE == 0) {
            if (pre) {
#pragma unroll
                for (int k = 0; k < 3; ++k) { lof[k] = __double2float_rd(lo[k]); hif[k] = __double2float_ru(hi[k]); }
                tbf2 = __double2float_ru((tb + 1e-5) * (tb + 1e-5));
                huntf2 = __double2float_ru((hunt + 1e-5) * (hunt + 1e-5));
                slackf = __double2float_ru(r + nm.eq + dmargin + 1e-5);
                bestf = __double2float_ru(w.profile ? nm.maxd : best);
            }
        }
        __syncwarp();
        // Register copies of the lane's per-link state that only the drains
        // change: a settled collision (flags bit 0), the first settled hit
        // (hitj) and the link minimum (lmin).
        bool hitb = false;
        int hj = 0x7fffffff;
        T cur = nm.maxd;
        int nb = 0, nd = 0;
        // the obstacle loop's body for obstacle j
        auto obstacle = [&](const int j) {
            const bool wb = need_b && !hitb;
            const bool wd = need_d && (hj == 0x7fffffff || (w.profile && j < hj));
            bool qb = false, qd = false;
            bool near = wb || wd;
            T o[6];
            T tj = T(0);
            bool have = false;   // o and tj loaded from the per-obstacle copy
            if constexpr (MODE == 2) {
                if (ob.aos != nullptr) {
                    const float4 a = ob.aos[2 * j], b = ob.aos[2 * j + 1];
                    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y;
                    tj = b.z;
                    near = near && !(ground_skip && b.w != 0.f);
                    have = true;
                }
            }
            if (!have) near = near && !(ground_skip && ob.is_ground(j));
            if constexpr (MODE == 0) {
                if (near && pre) {
                    float of[6];
#pragma unroll
                    for (int k = 0; k < 6; ++k) of[k] = ob.frows[k * ob.n_pad + j];
                    const float g2f = gap2_bb(lof, hif, of);
                    bool maybe = wb && !(g2f > tbf2);
                    if (wd && !maybe) {
                        if (hj != 0x7fffffff) {
                            maybe = !(g2f > huntf2);
                        } else {
                            const float tolf = ob.frows[kRowTol * ob.n_pad + j];
                            const float sf = (bestf < tolf ? bestf : tolf) + slackf;
                            maybe = !(tolf > 0.f) || !(g2f > sf * sf * 1.00001f);
                        }
                    }
                    near = maybe;
                }
            }
            if (near) {
                if (!have) ob.box(j, o);
                const T g2 = gap2_bb(lo, hi, o);
                qb = wb && !(g2 > tb2);
                if (wd) {
                    if (hj != 0x7fffffff) {
                        qd = !(g2 > hunt2);
                    } else {
                        T thr = w.profile ? cur : smin(best, cur);
                        thr = smin(thr, have ? tj : ob.tol(j));
                        const T s = thr + r + nm.eq + dmargin;
                        qd = !(s > T(0) && g2 > s * s);
                    }
                }
            }
            const uint32_t item = (uint32_t)lane | ((uint32_t)j << 5);
            if constexpr (KIND != 2 && KIND != 3)
                RPM_PUSH_AND_DRAIN(qb, nb, qb, item, drain_bool, hitb = (sh.flags[lane] & 1) != 0);
            if constexpr (KIND != 1)
                RPM_PUSH_AND_DRAIN(qd, nd, qd, item, drain_dist, (hj = sh.hitj[lane], cur = Key<T>::value(sh.lmin[lane])));
                };
        if constexpr (MODE == 2) {
            // The FP32 pass culls per warp, as warp_check_any does: the bounding box of
            // this link's segments over the lanes still working, tested against 32
            // obstacles at a time with the largest threshold of any lane, so an obstacle
            // it rejects is one no lane's own test would queue.
            float ulo[3], uhi[3];
            const bool working = need_b || need_d;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                ulo[c] = !working ? INFINITY : (lo[c] == lo[c] ? (float)lo[c] : -INFINITY);
                uhi[c] = !working ? -INFINITY : (hi[c] == hi[c] ? (float)hi[c] : INFINITY);
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    ulo[c] = fminf(ulo[c], __shfl_xor_sync(full, ulo[c], off));
                    uhi[c] = fmaxf(uhi[c], __shfl_xor_sync(full, uhi[c], off));
                }
            }
            for (int base = 0; base < ob.n; base += 32) {
                const bool wb_l = need_b && !hitb;
                const bool wd_l = need_d && (hj == 0x7fffffff || w.profile);
                const bool hunt_l = wd_l && hj != 0x7fffffff;
                const bool any_b = __any_sync(full, wb_l);
                const bool any_hunt = __any_sync(full, hunt_l);
                const bool any_d = __any_sync(full, wd_l && !hunt_l);
                float xl = (wd_l && !hunt_l) ? (float)(w.profile ? cur : smin(best, cur)) : -INFINITY;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) xl = fmaxf(xl, __shfl_xor_sync(full, xl, off));
                bool cand = false;
                const int jl = base + lane;
                if (jl < ob.n) {
                    float o[6], tj;
                    bool gr;
                    if (ob.aos != nullptr) {
                        const float4 a = ob.aos[2 * jl], b = ob.aos[2 * jl + 1];
                        o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y;
                        tj = b.z;
                        gr = b.w != 0.f;
                    } else {
#pragma unroll
                        for (int k = 0; k < 6; ++k) o[k] = (float)ob.rows[k * ob.n_pad + jl];
                        tj = (float)ob.tol(jl);
                        gr = ob.is_ground(jl);
                    }
                    if (!(ground_skip && gr)) {
                        const float g2 = gap2_bb(ulo, uhi, o);
                        cand = any_b && !(g2 > (float)tb2);
                        if (any_hunt) cand = cand || !(g2 > (float)hunt2);
                        if (any_d) {
                            const float sd = smin(xl, tj) + (float)r + (float)nm.eq + (float)dmargin;
                            cand = cand || !(sd > 0.f && g2 > sd * sd);
                        }
                    }
                }
                unsigned cm = __ballot_sync(full, cand);
                while (cm != 0u) {
                    const int j = base + __ffs(cm) - 1;
                    cm &= cm - 1u;
                    obstacle(j);
                }
            }
        } else {
            for (int j = 0; j < ob.n; ++j) obstacle(j);
        }
        __syncwarp();
        if (nb > 0) drain_bool<MODE, T, kFlat>(sh, rb, ob, nm, i, nb, ps);
        if (nd > 0) drain_dist<MODE, T>(sh, rb, ob, nm, i, nd, ps);
        __syncwarp();
        // ---- fold this link's results into the lane's configuration
        const int fl = sh.flags[lane];
        if (need_b) {
            if (fl & 1) { collided = true; need_b = false; }
            if (fl & 2) unc_b = true;
        }
        if (dist_link) {
            if (fl & 4) unc_d = true;
            const int hj = sh.hitj[lane];
            const T lmin = Key<T>::value(sh.lmin[lane]);
            if (hj != 0x7fffffff) {
                // the partial minimum at the first hit is the hit's own value
                hit = i;
                hit_obs = hj;
                need_d = false;
                if (w.profile) prof_out[i] = (float)sh.hitv[lane];
            } else {
                if (w.profile) prof_out[i] = (float)lmin;
                best = smin(best, lmin);
            }
        }
        sh.flags[lane] = fl & ~7;   // the per-link bits have been folded
        __syncwarp();
        A[0] = B[0]; A[1] = B[1]; A[2] = B[2];
    }
    if (slot) *slot = sh.slot[lane];
    if (!active) return kSettled;
    if (w.profile && hit >= 0)
        for (int k = hit + 1; k < L; ++k) prof_out[k] = 0.f;
    if (w.valid) *valid_out = collided ? 0 : 1;
    if (w.dist) *dist_out = (hit >= 0) ? 0.0 : (double)best;
    if (hit_link) *hit_link = hit;
    if (hit_j) *hit_j = hit_obs;
    const bool bad_b = w.valid && !collided && unc_b;
    const bool bad_d = (w.dist || w.profile) && unc_d && (w.profile || hit < 0);
    if (!(bad_b || bad_d)) return kSettled;
    return (ps && sh.slot[lane] >= 0 && !(sh.flags[lane] & 8)) ? kPairs : kFull;
}

// ---------------------------------------------------------------------------
// Order-free kinds of the FP32 pass: isValid alone (KIND 1) and the distance
// alone, without a profile (KIND 3).  Both outputs are folds over all (link,
// obstacle) pairs that do not depend on the pairs' order: isValid is the OR
// of the pair tests (RealVectorSpace.cpp:277-309), and the distance is 0 if
// some pair has d <= 0, else the minimum over all pairs (:318-392; the early
// exits and the per-link profile change only which pairs the reference
// evaluates, not these two values).  So this driver
//   * runs the lane's whole FP32 forward kinematics first and keeps the
//     skeleton in shared memory ([3 * point + coordinate][NT] floats);
//   * visits the links in an order that meets collisions and small distances
//     early (xArm6: links 2-5, then the base links 0 and 1; serial chains: the
//     distal link first);
//   * keeps one queue of (owner, link, obstacle) items across links, drained
//     when 32 items wait, so almost every drain runs a full warp; the
//     distance's pruning threshold is the lane's running minimum over all
//     links so far.
// A lane stops at its first settled collision (KIND 1) or settled hit
// (KIND 3).  Outputs and pair records are the same as warp_check's.
__device__ __forceinline__ int any_order_link(const DevRobot &rb, int k) {
    if (rb.kind == RPM_ROBOT_XARM6) return k + 2 < 6 ? k + 2 : k - 4;
    return rb.D - 1 - k;
}

template <int KIND, int NT>
__device__ __forceinline__ void drain_any(WarpShared<float> &sh, const float *skel, const DevRobot &rb,
                                          const ObsView<float> &ob, const Num<float> &nm, const uint32_t *queue,
                                          int nitems, const PairSink *ps) {
    const int lane = threadIdx.x & 31;
    uint32_t pe = 0u;
    if (lane < nitems) {
        const uint32_t e = queue[lane];
        const int owner = (int)(e & 31u), j = (int)((e >> 5) & 2047u), li = (int)((e >> 16) & 31u);
        const float *sk = skel + (threadIdx.x & ~31) + owner;
        float A[3], B[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            A[k] = sk[(3 * li + k) * NT];
            B[k] = sk[(3 * li + 3 + k) * NT];
        }
        if constexpr (KIND == 1) {
            float o[6];
            ob.box(j, o);
            const RB rr = coll_box_call<float, RobustPol, true>(nm, A, B, rb.radius_f[li], rb.rnew_f[li], o);
            if (rr.m < kDecide) {
                atomicOr(&sh.flags[owner], 2);
                pe = pend_of(e, li, 0);
            } else if (rr.v) {
                atomicOr(&sh.flags[owner], 1);
            }
        } else {
            bool settled;
            const float d = pair_distance<2, float>(rb, ob, nm, A, B, li, j, settled);
            if (!settled) {
                atomicOr(&sh.flags[owner], 4);
                pe = pend_of(e, li, 1);
            } else if (d == d) {   // the reference's std::min ignores NaN
                atomicMin(&sh.lmin[owner], Key<float>::of(d));
                if (d <= 0.f) atomicOr(&sh.flags[owner], 1);
            }
        }
    }
    if (ps) {
        sh.pend[lane] = pe;
        if (__any_sync(0xffffffffu, pe != 0u)) flush_pending(sh, ps);
    }
}

// Returns kSettled, kPairs or kFull per lane, as warp_check does; *slot
// receives the lane's pair-recheck record (-1: none).  skel points to this
// CTA's skeleton buffer of (rb.D + 1) * 3 * NT floats.
template <int KIND, int NT>
__device__ int warp_check_any(WarpShared<float> &sh, float *skel, const DevRobot &rb, const ObsView<float> &ob,
                              const float *q, bool active, const Num<float> &nm, uint8_t *valid_out,
                              double *dist_out, const PairSink *ps, int *slot) {
    static_assert(KIND == 1 || KIND == 3, "isValid alone or the distance alone");
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int L = rb.D;
    float *mine = skel + threadIdx.x;
    {
        SkelWalker<2> sw;
        sw.begin();
        for (int p = 0; p <= L; ++p) {
            float P[3] = {0.f, 0.f, 0.f};
            if (active) sw.point(rb, q, p, P);
            mine[(3 * p) * NT] = P[0];
            mine[(3 * p + 1) * NT] = P[1];
            mine[(3 * p + 2) * NT] = P[2];
        }
    }
    sh.flags[lane] = 0;
    sh.slot[lane] = -1;
    sh.need[lane] = 0;
    sh.lmin[lane] = Key<float>::of(nm.maxd);
    __syncwarp();
    uint32_t *queue = KIND == 1 ? sh.qb : sh.qd;
    bool stop = !active;          // register copy of flags bit 0 (settled collision / settled hit)
    float cur = nm.maxd;          // register copy of the running minimum (KIND 3)
    int nq = 0;
    int seed_j = -1;              // KIND 3: the obstacle every lane checked first on the first link
    if constexpr (KIND == 3) {
        // Seed.  Until a lane has a distance its threshold is MAX_DISTANCE, so the
        // first link would queue every obstacle, and the warp's cull would keep
        // them all.  So the warp first checks, on the first link it visits, the
        // non-ground obstacle nearest to the union box of its lanes' segments (its
        // lanes hold similar configurations); every lane's threshold then starts at
        // a real distance.  The pair is skipped when the loop reaches it.
        const int i0 = any_order_link(rb, 0);
        float ulo[3], uhi[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float a = mine[(3 * i0 + c) * NT], b = mine[(3 * i0 + 3 + c) * NT];
            const float l = a < b ? a : b, h = a < b ? b : a;
            ulo[c] = stop ? INFINITY : (l == l ? l : -INFINITY);
            uhi[c] = stop ? -INFINITY : (h == h ? h : INFINITY);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                ulo[c] = fminf(ulo[c], __shfl_xor_sync(full, ulo[c], off));
                uhi[c] = fmaxf(uhi[c], __shfl_xor_sync(full, uhi[c], off));
            }
        }
        float bg = INFINITY;
        int bj = 0x7fffffff;
        for (int jl = lane; jl < ob.n; jl += 32) {
            float o[6];
            bool gr;
            if (ob.aos != nullptr) {
                const float4 a = ob.aos[2 * jl], b = ob.aos[2 * jl + 1];
                o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y;
                gr = b.w != 0.f;
            } else {
                ob.box(jl, o);
                gr = ob.is_ground(jl);
            }
            if (gr) continue;
            const float g2 = gap2_bb(ulo, uhi, o);
            if (g2 < bg) { bg = g2; bj = jl; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float og = __shfl_xor_sync(full, bg, off);
            const int oj = __shfl_xor_sync(full, bj, off);
            if (og < bg || (og == bg && oj < bj)) { bg = og; bj = oj; }
        }
        if (bj != 0x7fffffff && __any_sync(full, !stop)) {
            seed_j = bj;
            const unsigned m = __ballot_sync(full, !stop);
            if (!stop) queue[__popc(m & lt_mask)] = (uint32_t)lane | ((uint32_t)bj << 5) | ((uint32_t)i0 << 16);
            __syncwarp();
            drain_any<KIND, NT>(sh, skel, rb, ob, nm, queue, __popc(m), ps);
            __syncwarp();
            stop = stop || (sh.flags[lane] & 1) != 0;
            cur = Key<float>::value(sh.lmin[lane]);
            __syncwarp();
        }
    }
    for (int k = 0; k < L; ++k) {
        if (!__any_sync(full, !stop)) break;
        const int i = any_order_link(rb, k);
        const float r = rb.radius_f[i];
        const bool ground_skip = i < rb.ground_included;
        float lo[3], hi[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float a = mine[(3 * i + c) * NT], b = mine[(3 * i + 3 + c) * NT];
            lo[c] = a < b ? a : b;
            hi[c] = a < b ? b : a;
        }
        const float tb = r * 1.41421356237309515f + kDecide;
        const float tb2 = tb * tb;
        const float rs = r + nm.eq + kBand;
        const uint32_t ibits = (uint32_t)lane | ((uint32_t)i << 16);
        // The warp's cull: the bounding box of this link's segments over the lanes
        // still working (a NaN coordinate widens it to everything), tested against 32
        // obstacles at a time, one per lane, with the largest threshold of any working
        // lane.  The gap to that box is at most the gap to any lane's own segment box,
        // so an obstacle it rejects is one no lane's own test below would queue.
        float ulo[3], uhi[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            ulo[c] = stop ? INFINITY : (lo[c] == lo[c] ? lo[c] : -INFINITY);
            uhi[c] = stop ? -INFINITY : (hi[c] == hi[c] ? hi[c] : INFINITY);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                ulo[c] = fminf(ulo[c], __shfl_xor_sync(full, ulo[c], off));
                uhi[c] = fmaxf(uhi[c], __shfl_xor_sync(full, uhi[c], off));
            }
        }
        for (int base = 0; base < ob.n; base += 32) {
            float cmax = stop ? -INFINITY : cur;   // KIND 3: the largest running minimum of a working lane
            if constexpr (KIND == 3) {
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) cmax = fmaxf(cmax, __shfl_xor_sync(full, cmax, off));
            }
            bool cand = false;
            if (base + lane < ob.n) {
                const int jl = base + lane;
                float o[6], tj;
                bool gr;
                if (ob.aos != nullptr) {
                    const float4 a = ob.aos[2 * jl], b = ob.aos[2 * jl + 1];
                    o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y;
                    tj = b.z;
                    gr = b.w != 0.f;
                } else {
                    ob.box(jl, o);
                    tj = ob.tol(jl);
                    gr = ob.is_ground(jl);
                }
                if (!(ground_skip && gr)) {
                    const float g2 = gap2_bb(ulo, uhi, o);
                    if constexpr (KIND == 1) {
                        cand = !(g2 > tb2);
                    } else {
                        const float s = smin(cmax, tj) + rs;
                        cand = !(s > 0.f && g2 > s * s);
                    }
                }
            }
            unsigned cm = __ballot_sync(full, cand);
        while (cm != 0u) {
            const int j = base + __ffs(cm) - 1;
            cm &= cm - 1u;
            float o[6], tj;
            bool gr;
            if (ob.aos != nullptr) {
                const float4 a = ob.aos[2 * j], b = ob.aos[2 * j + 1];
                o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w; o[4] = b.x; o[5] = b.y;
                tj = b.z;
                gr = b.w != 0.f;
            } else {
                ob.box(j, o);
                tj = ob.tol(j);
                gr = ob.is_ground(j);
            }
            bool qq = false;
            if (!stop && !(ground_skip && gr) && !(k == 0 && j == seed_j)) {
                const float g2 = gap2_bb(lo, hi, o);
                if constexpr (KIND == 1) {
                    qq = !(g2 > tb2);
                } else {
                    const float s = smin(cur, tj) + rs;
                    qq = !(s > 0.f && g2 > s * s);
                }
            }
            const unsigned m = __ballot_sync(full, qq);
            if (m != 0u) {
                if (qq) queue[nq + __popc(m & lt_mask)] = ibits | ((uint32_t)j << 5);
                nq += __popc(m);
                if (nq >= 32) {
                    __syncwarp();
                    drain_any<KIND, NT>(sh, skel, rb, ob, nm, queue, 32, ps);
                    __syncwarp();
                    if (lane < nq - 32) queue[lane] = queue[32 + lane];
                    nq -= 32;
                    stop = stop || (sh.flags[lane] & 1) != 0;
                    if constexpr (KIND == 3) cur = Key<float>::value(sh.lmin[lane]);
                    __syncwarp();
                }
            }
        }
        }
    }
    __syncwarp();
    if (nq > 0) drain_any<KIND, NT>(sh, skel, rb, ob, nm, queue, nq, ps);
    __syncwarp();
    const int fl = sh.flags[lane];
    if (slot) *slot = sh.slot[lane];
    if (!active) return kSettled;
    bool bad;
    if constexpr (KIND == 1) {
        const bool collided = (fl & 1) != 0;
        if (valid_out) *valid_out = collided ? 0 : 1;
        bad = !collided && (fl & 2);
    } else {
        const bool hit = (fl & 1) != 0;
        if (dist_out) *dist_out = hit ? 0.0 : (double)Key<float>::value(sh.lmin[lane]);
        bad = !hit && (fl & 4);
    }
    if (!bad) return kSettled;
    return (ps && sh.slot[lane] >= 0 && !(fl & 8)) ? kPairs : kFull;
}
#endif

}  // namespace rpm
