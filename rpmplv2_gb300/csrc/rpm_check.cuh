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

// Exact forms: MODE 0 = FP64 (T double), MODE 1 = the reference's numerics (T float).
template <int MODE, typename T>
__host__ __device__ void config_exact(const DevRobot &rb, const ObsView<T> &ob, const float *q, const Num<T> &nm, Want w,
                             uint8_t *valid_out, double *dist_out, float *prof_out) {
    SkelWalker<MODE> sw;
    sw.begin();
    T A[3], B[3];
    sw.point(rb, q, 0, A);
    bool need_b = w.valid, need_d = w.dist || w.profile;
    bool collided = false;
    T best = nm.maxd;
    int hit = -1;
    T hit_val = T(0);
    const int L = rb.D;
    for (int i = 0; i < L && (need_b || need_d); ++i) {
        sw.point(rb, q, i + 1, B);
        const T r = LinkConst<T>::r(rb, i), rn = LinkConst<T>::rn(rb, i);
        const bool ground_skip = i < rb.ground_included;
        const bool dist_link = need_d;
        T link_best = nm.maxd;
        for (int j = 0; j < ob.n && (need_b || need_d); ++j) {
            if (ground_skip && ob.is_ground(j)) continue;   // :285 (bool) and :336-341 (d = MAX)
            T o[6];
            ob.box(j, o);
            if (need_b) {
                ExactPol pol;
                if (coll_box(pol, nm, A, B, r, rn, o)) { collided = true; need_b = false; }
            }
            if (need_d) {
                const T tol = ob.tol(j);
                T thr = w.profile ? link_best : smin(best, link_best);
                thr = smin(thr, tol);
                const T s = thr + r + nm.eq + LinkConst<T>::margin();
                if (s > T(0) && gap2(A, B, o) > s * s) continue;
                ExactPol pol;
                T d = capsule_box(pol, nm, A, B, r, o).v;
                if (d > tol) d = nm.maxd;                     // :367-368
                link_best = smin(link_best, d);               // :370
                if (link_best <= T(0)) { hit = i; hit_val = link_best; need_d = false; }   // :371-378
            }
        }
        if (w.profile && dist_link) prof_out[i] = (hit == i) ? (float)hit_val : (float)link_best;
        if (hit < 0) best = smin(best, link_best);
        A[0] = B[0]; A[1] = B[1]; A[2] = B[2];
    }
    if (w.profile && hit >= 0)
        for (int k = hit + 1; k < L; ++k) prof_out[k] = 0.f;   // d_c_profile is zero-initialised (:325)
    if (w.valid) *valid_out = collided ? 0 : 1;
    if (w.dist) *dist_out = (hit >= 0) ? 0.0 : (double)best;
}

// FP32 bulk pass.  Returns true when every decision that shaped the requested
// outputs was settled (branch margins >= kDecide, clearances outside the
// contact band kBand).  Returns false when the configuration must be
// recomputed in FP64; the outputs it wrote are then provisional and the FP64
// recheck overwrites every one of them.
static __host__ __device__ bool config_fp32(const DevRobot &rb, const ObsView<float> &ob, const float *q,
                                            const Num<float> &nm, Want w, uint8_t *valid_out, double *dist_out,
                                            float *prof_out) {
    SkelWalker<2> sw;
    sw.begin();
    float A[3], B[3];
    sw.point(rb, q, 0, A);
    bool need_b = w.valid, need_d = w.dist || w.profile;
    bool collided = false, unc_b = false, unc_d = false;
    float best = nm.maxd;
    int hit = -1;
    const int L = rb.D;
    for (int i = 0; i < L && (need_b || need_d); ++i) {
        sw.point(rb, q, i + 1, B);
        const float r = rb.radius_f[i], rn = rb.rnew_f[i];
        const bool ground_skip = i < rb.ground_included;
        const bool dist_link = need_d;
        float link_best = nm.maxd;
        for (int j = 0; j < ob.n && (need_b || need_d); ++j) {
            if (ground_skip && ob.is_ground(j)) continue;
            float o[6];
            ob.box(j, o);
            if (need_b) {
                RobustPol pol;
                bool c = coll_box(pol, nm, A, B, r, rn, o);
                if (pol.m < kDecide) { unc_b = true; RPM_DBG_B(pol); }
                else if (c) { collided = true; need_b = false; }
            }
            if (need_d) {
                const float tol = ob.tol(j);
                float thr = w.profile ? link_best : fminf(best, link_best);
                thr = fminf(thr, tol);
                const float s = thr + r + nm.eq + kBand;
                if (s > 0.f && gap2(A, B, o) > s * s) continue;
                RobustPol pol;
                Val<float> dv = capsule_box(pol, nm, A, B, r, o);
                float d = dv.v;
                // clearance decisions use the contact band (scaled onto kDecide)
                const float band = dv.ia * (kDecide / kBand);
                RPM_NOTE(pol, fabsf(d - tol) * band);
                if (d > tol) d = nm.maxd;
                if (d != 0.f) RPM_NOTE(pol, fabsf(d) * band);   // exact zeros come from settled branches
                if (pol.m < kDecide) { unc_d = true; RPM_DBG_D(pol); }
                link_best = (d < link_best) ? d : link_best;
                if (link_best <= 0.f) { hit = i; need_d = false; }
            }
        }
        if (w.profile && dist_link) prof_out[i] = link_best;   // the hit value when hit == i
        if (hit < 0) best = fminf(best, link_best);
        A[0] = B[0]; A[1] = B[1]; A[2] = B[2];
    }
    if (w.profile && hit >= 0)
        for (int k = hit + 1; k < L; ++k) prof_out[k] = 0.f;
    if (w.valid) *valid_out = collided ? 0 : 1;
    if (w.dist) *dist_out = (hit >= 0) ? 0.0 : (double)best;
    // A settled collision decides isValid; a settled hit decides the scalar
    // distance (0), but not the profile's first-hit position.
    const bool bad_b = w.valid && !collided && unc_b;
    const bool bad_d = (w.dist || w.profile) && unc_d && (w.profile || hit < 0);
    return !(bad_b || bad_d);
}

}  // namespace rpm
