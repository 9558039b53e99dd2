// rpm_wide.cuh -- warp-per-configuration drivers of RealVectorSpace::isValid(q)
// (RealVectorSpace.cpp:277-309) and computeDistance(q) (:318-392) over a
// spatially sorted, block-bounded copy of the obstacles.
//
// Used for large scenes and small requests, where lane-per-configuration
// leaves the GPU mostly idle and each lane walks hundreds of obstacles in
// series.  Here a warp first runs the forward kinematics of G configurations
// (lane = configuration, skeleton points kept in shared memory), then checks
// them one at a time with the lanes spread over the obstacles:
//   * blocks of 32 obstacles (Morton order of their centres) carry their union
//     bounds and their largest / smallest min_dist_tol, so one gap test rejects
//     a whole block;
//   * isValid scans the blocks whose gap is within r*sqrt(2) of the link's
//     bounding box (the reach of the reference's capsule-box tree);
//   * distance visits blocks nearest-first and drains candidate pairs as they
//     fill a 32-entry queue, so the running minimum tightens the threshold for
//     the blocks still to visit.
// Every pair the lane-per-configuration driver would evaluate with a tree and
// that can change an output is evaluated here too, with the same arithmetic;
// results combine by the same rules (OR; minimum of ordered keys; first hit =
// lowest ORIGINAL obstacle index), so outputs are bit-identical to it.
#pragma once
#include <type_traits>

#include "rpm_check.cuh"
#include "rpm_launch.cuh"

namespace rpm {

constexpr int kWideWarps = 8;                       // warps per CTA
constexpr int kWideThreads = kWideWarps * 32;
constexpr int kWidePtsBytes = 2048;                 // skeleton buffer per warp
constexpr int kBlk = 32;                            // obstacles per block
constexpr int kBlkRec = 8;                          // lo[3] hi[3] max tol, min tol (float)
constexpr int kBlkPerLane = 3;                      // blocks per lane in the distance search
constexpr int kMaxSorted = kBlk * 32 * kBlkPerLane; // sorted slots per scene (>= kMaxObstacles + 2 * kBlk)
constexpr uint32_t kGroundBit = 0x80000000u;        // idx row: ground obstacle
constexpr uint32_t kPadIdx = 0x7fffffffu;           // idx row: padding slot (bounds +inf / -inf)
static_assert(kMaxSorted >= kMaxObstacles + 2 * kBlk, "sorted layout too small");
// Automatic layout: warp-per-configuration for scenes of at least
// kWideMinObstacles obstacles, or for batches too small to give each SM four
// lane-per-configuration warps when links x obstacles reaches kWideMinPairs.
constexpr int kWideMinObstacles = 128;
constexpr int kWideMinPairs = 512;

// Sorted copy of one scene version: slot s holds original obstacle idx[s].
// Non-ground obstacles come first in Morton order, ground obstacles start on a
// block boundary after them, so a block is ground-only iff its first slot is.
template <typename T> struct SortedView {
    const T *rows;          // [7][ns]: AABB, min_dist_tol
    const uint32_t *idx;    // [ns]
    const float *blk;       // [nb][kBlkRec]
    int ns, nb;
    RPM_HD void box(int s, T *o) const {
#pragma unroll
        for (int k = 0; k < 6; ++k) o[k] = rows[k * ns + s];
    }
    RPM_HD T tol(int s) const { return rows[kRowTol * ns + s]; }
    RPM_HD bool ground_block(int b) const { return (idx[b * kBlk] & kGroundBit) != 0u; }
};

#ifdef __CUDACC__
// Skeleton points per warp that fit the per-warp buffer.
template <typename T> __host__ __device__ constexpr int wide_g_max(int D) {
    return kWidePtsBytes / ((D + 1) * 3 * (int)sizeof(T));
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

template <int MODE, typename T>
__device__ __forceinline__ void wide_drain_bool(const uint32_t *q, int nitems, const SortedView<T> &ob, const Num<T> &nm,
                                                const T *A, const T *B, T r, T rn, bool &hit, bool &unc) {
    typedef typename PolOf<MODE>::type P;
    const int lane = threadIdx.x & 31;
    bool c = false, u = false;
    if (lane < nitems) {
        T o[6];
        ob.box((int)q[lane], o);
        P pol;
        const bool cc = coll_box(pol, nm, A, B, r, rn, o);
        if (P::robust && pol.m < kDecide) u = true;
        else c = cc;
    }
    hit = hit || __any_sync(0xffffffffu, c);
    unc = unc || __any_sync(0xffffffffu, u);
}

template <int MODE, typename T>
__device__ __forceinline__ void wide_drain_dist(const uint32_t *q, int nitems, const DevRobot &rb, const SortedView<T> &ob,
                                                const Num<T> &nm, const T *A, const T *B, int i,
                                                typename Key<T>::type &lkey, int &hj, T &hv, bool &unc) {
    typedef typename Key<T>::type K;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    K kk = Key<T>::of(nm.maxd);
    int jj = 0x7fffffff;
    T vv = T(0);
    bool u = false;
    if (lane < nitems) {
        const int s = (int)q[lane];
        bool settled;
        const T d = pair_distance<MODE, T>(rb, ob, nm, A, B, i, s, settled);
        u = !settled;
        if (d == d) {   // the reference's std::min ignores NaN
            kk = Key<T>::of(d);
            if (d <= T(0) && settled) { jj = (int)(ob.idx[s] & ~kGroundBit); vv = d; }
        }
    }
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

// One configuration, the whole warp.  pts = skeleton points [(D+1)][3].
// Returns whether the outputs are settled (always true for the exact forms);
// lane 0 writes the outputs.
template <int MODE, typename T>
__device__ bool wide_config(uint32_t *q, const DevRobot &rb, const SortedView<T> &ob, const T *pts, const Num<T> &nm,
                            Want w, uint8_t *valid_out, double *dist_out, float *prof_out) {
    typedef typename Key<T>::type K;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const T inf = T(1) / T(0);
    bool need_b = w.valid, need_d = w.dist || w.profile;
    bool collided = false, unc_b = false, unc_d = false;
    T best = nm.maxd;
    int hit = -1;
    const int L = rb.D;
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
            for (int b0 = 0; b0 < ob.nb && !hb; b0 += 32) {
                const int b = b0 + lane;
                bool cb = false;
                if (b < ob.nb && !(gskip && ob.ground_block(b))) {
                    const float *bk = ob.blk + b * kBlkRec;
                    T o[6];
#pragma unroll
                    for (int k = 0; k < 6; ++k) o[k] = (T)bk[k];
                    cb = !(gap2_bb(lo, hi, o) > tb2);
                }
                unsigned mb = __ballot_sync(full, cb);
                while (mb != 0u && !hb) {
                    const int bb = __ffs(mb) - 1;
                    mb &= mb - 1u;
                    const int s = (b0 + bb) * kBlk + lane;
                    const uint32_t id = ob.idx[s];
                    bool c = false;
                    if (id != kPadIdx && !(gskip && (id & kGroundBit))) {
                        T o[6];
                        ob.box(s, o);
                        c = !(gap2_bb(lo, hi, o) > tb2);
                    }
                    wide_push<MODE, T>(q, nq, c, (uint32_t)s);
                    if (nq >= 32) {
                        wide_drain_bool<MODE, T>(q, 32, ob, nm, A, B, r, rn, hb, ub);
                        wide_pop32(q, nq);
                    }
                }
            }
            if (nq > 0 && !hb) wide_drain_bool<MODE, T>(q, nq, ob, nm, A, B, r, rn, hb, ub);
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
            T g2b[kBlkPerLane], tmax[kBlkPerLane], tmin[kBlkPerLane];
            unsigned todo = 0u;
#pragma unroll
            for (int k = 0; k < kBlkPerLane; ++k) {
                const int b = lane + 32 * k;
                g2b[k] = inf; tmax[k] = T(0); tmin[k] = T(0);
                if (b < ob.nb && !(gskip && ob.ground_block(b))) {
                    const float *bk = ob.blk + b * kBlkRec;
                    T o[6];
#pragma unroll
                    for (int c = 0; c < 6; ++c) o[c] = (T)bk[c];
                    g2b[k] = gap2_bb(lo, hi, o);
                    tmax[k] = (T)bk[6];
                    tmin[k] = (T)bk[7];
                    todo |= 1u << k;
                }
            }
            int nq = 0;
            bool seeded = false;
            for (;;) {
                const bool hunting = hj != 0x7fffffff;
                const T thr0 = w.profile ? Key<T>::value(lkey) : smin(best, Key<T>::value(lkey));
                // nearest block still alive (thresholds only shrink, so a pruned block stays pruned)
                T bg = inf;
                int sel = 0x7fffffff;
#pragma unroll
                for (int k = 0; k < kBlkPerLane; ++k) {
                    if (!((todo >> k) & 1u)) continue;
                    bool alive;
                    if (hunting) {
                        alive = !(g2b[k] > hunt * hunt);
                    } else {
                        const T smax = smin(thr0, tmax[k]) + r + nm.eq + dmargin;
                        const T slo = smin(thr0, tmin[k]) + r + nm.eq + dmargin;
                        alive = !(slo > T(0) && g2b[k] > smax * smax);
                    }
                    if (!alive) todo &= ~(1u << k);
                    else if (g2b[k] < bg || sel == 0x7fffffff) { bg = g2b[k]; sel = lane + 32 * k; }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const T og = __shfl_xor_sync(full, bg, off);
                    const int ob_ = __shfl_xor_sync(full, sel, off);
                    if (og < bg || (!(bg < og) && ob_ < sel)) { bg = og; sel = ob_; }
                }
                if (sel == 0x7fffffff) break;
                if ((sel & 31) == lane) todo &= ~(1u << (sel >> 5));
                const int s = sel * kBlk + lane;
                const uint32_t id = ob.idx[s];
                bool c = false;
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
                wide_push<MODE, T>(q, nq, c, (uint32_t)s);
                if (nq >= 32 || (nq > 0 && !seeded)) {
                    const int take = nq < 32 ? nq : 32;
                    wide_drain_dist<MODE, T>(q, take, rb, ob, nm, A, B, i, lkey, hj, hv, ud);
                    if (take == 32) wide_pop32(q, nq);
                    else nq = 0;
                    seeded = true;
                    if (hj != 0x7fffffff && !w.profile) break;   // the distance is 0 whatever else is found
                }
            }
            if (nq > 0 && !(hj != 0x7fffffff && !w.profile))
                wide_drain_dist<MODE, T>(q, nq, rb, ob, nm, A, B, i, lkey, hj, hv, ud);
            __syncwarp();
            if (ud) unc_d = true;
            if (hj != 0x7fffffff) {
                // the partial minimum at the first hit is the hit's own value
                hit = i;
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
    const bool bad_b = w.valid && !collided && unc_b;
    const bool bad_d = (w.dist || w.profile) && unc_d && (w.profile || hit < 0);
    return !(bad_b || bad_d);
}

// Shared-memory layout of the wide kernels: robot, sorted rows, index row,
// block records, per-warp skeleton buffers.  Every piece is a multiple of 16
// bytes (ns is a multiple of 32).
struct WideLayout {
    uint32_t rows, idx, blk, pts, total;
    RPM_HD static WideLayout of(int mode, int ns, int nb) {
        WideLayout l;
        const uint32_t tsz = mode == RPM_PREC_FP64 ? 8u : 4u;
        l.rows = (uint32_t)sizeof(DevRobot);
        l.idx = l.rows + 7u * (uint32_t)ns * tsz;
        l.blk = l.idx + 4u * (uint32_t)ns;
        l.pts = l.blk + 4u * kBlkRec * (uint32_t)nb;
        l.total = l.pts + kWideWarps * kWidePtsBytes;
        return l;
    }
};

// Body of k_check_wide<MODE>: CTA = kWideWarps warps, each owning G = P.wide_g
// consecutive configurations of one segment.
template <int MODE>
__device__ __forceinline__ void wide_kernel_body(const KParams &P, unsigned char *smem, uint64_t *bar,
                                                 uint32_t (*wq)[64], int s) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    const Seg &sg = P.segs[s];
    const WideLayout L = WideLayout::of(MODE == 0 ? RPM_PREC_FP64 : RPM_PREC_FP32_REF, sg.ns, sg.nb);
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
    if (!bulk_wait(bar, 0, P.status)) return;
    const DevRobot &rb = *reinterpret_cast<const DevRobot *>(smem);
    SortedView<T> ob{reinterpret_cast<const T *>(smem + L.rows), reinterpret_cast<const uint32_t *>(smem + L.idx),
                     reinterpret_cast<const float *>(smem + L.blk), sg.ns, sg.nb};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int G = P.wide_g;
    const int D = rb.D;
    const int64_t c0 = (int64_t)(blockIdx.x - sg.first_block) * (kWideWarps * G) + (int64_t)warp * G;
    if (c0 >= sg.count) return;   // whole warp idle
    T *pts = reinterpret_cast<T *>(smem + L.pts + warp * kWidePtsBytes);
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
    for (int g = 0; g < G; ++g) {
        const int64_t c = c0 + g;
        if (c >= sg.count) break;
        const bool ok = wide_config<MODE, T>(wq[warp], rb, ob, pts + g * (D + 1) * 3, nm, w,
                                             w.valid ? sg.valid + c : nullptr, w.dist ? sg.dist + c : nullptr,
                                             w.profile ? sg.profile + c * D : nullptr);
        if (MODE == 2 && !ok && lane == 0) {
            const uint32_t slot = atomicAdd(P.recheck_count, 1u);
            P.recheck[slot] = ((uint64_t)s << 40) | (uint64_t)c;
        }
    }
}
#endif

}  // namespace rpm
