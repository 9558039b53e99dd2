// rpm_nearest.cuh -- computeDistance with nearest points (RealVectorSpace.cpp:
// 318-392) and computeDistanceUnderestimation (:402-446) for the single-state
// adapter path, in the exact forms (FP64, and the reference's FP32 numerics).
//
// The nearest points of a (link, obstacle) pair are the robot point (on the
// skeleton segment) and the obstacle point that CapsuleToBox::compute
// (CollisionAndDistance.cpp:409-448) leaves in its 3x2 matrix:
//   * a projecting endpoint and its projection on the first face it projects
//     on (faces in the order x_min, y_min, z_min, x_max, y_max, z_max);
//   * the pair of the box edge or corner whose distance is the first strictly
//     smaller one (distanceToMoreLineSegments :576-595, distanceLineSegToLineSeg
//     :217-320, distanceLineSegToPoint :323-342);
//   * left as they are when a crossing sets the distance to 0, and absent when
//     an endpoint lies inside or a segment distance snaps to 0.
// The distances are computed with the same operations, in the same order, as
// the value-only trees of rpm_tree.cuh, so they are identical to them.
#pragma once
#include "rpm_tree.cuh"

namespace rpm {

// distanceLineSegToLineSeg with nearest points (pts = point on AB, point on CD).
template <typename T>
RPM_HD T seg_seg_pts(const Num<T> &nm, const T *A, const T *B, const T *C, const T *D, T *pts, bool &has) {
    T BA[3], DC[3], CD[3], AC[3], AB[3];
    sub3(B, A, BA); sub3(D, C, DC); sub3(C, D, CD); sub3(A, C, AC); sub3(A, B, AB);
    const T alpha1 = dot3(BA, BA), alpha2 = dot3(BA, DC);
    const T beta1 = dot3(CD, BA), beta2 = dot3(CD, DC);
    const T gamma1 = dot3(AC, AB), gamma2 = dot3(AC, CD);
    const T s = (alpha1 * gamma2 - alpha2 * gamma1) / (alpha1 * beta2 - alpha2 * beta1);
    const T t = (gamma1 - beta1 * s) / alpha1;
    if (t > T(0) && t < T(1) && s > T(0) && s < T(1)) {
        T P0[3], P1[3], df[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            P0[k] = A[k] + t * BA[k];
            P1[k] = C[k] + s * DC[k];
            df[k] = P1[k] - P0[k];
        }
        const T d = norm3(df);
        if (d < nm.eq) { has = false; return T(0); }
#pragma unroll
        for (int k = 0; k < 3; ++k) { pts[k] = P0[k]; pts[3 + k] = P1[k]; }
        has = true;
        return d;
    }
    const T alpha3 = dot3(CD, CD);
    T AD[3], BC[3];
    sub3(A, D, AD); sub3(B, C, BC);
    const T opt[4] = {dot3(AC, AB) / alpha1, dot3(AD, AB) / alpha1, dot3(AC, DC) / alpha3, dot3(BC, DC) / alpha3};
    T d = nm.maxd;
    has = true;   // the reference returns its matrix here (set by the first smaller candidate)
    for (int i = 0; i < 4; ++i) {
        T P0[3], P1[3];
        const T o = opt[i];
        if (i < 2) {   // C (i = 0) or D (i = 1) against AB
            const T *Q = i == 0 ? C : D;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                P0[k] = o < T(0) ? A[k] : (o > T(1) ? B[k] : A[k] + o * BA[k]);
                P1[k] = Q[k];
            }
        } else {       // A (i = 2) or B (i = 3) against CD
            const T *Q = i == 2 ? A : B;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                P0[k] = Q[k];
                P1[k] = o < T(0) ? C[k] : (o > T(1) ? D[k] : C[k] + o * DC[k]);
            }
        }
        T df[3];
        sub3(P1, P0, df);
        const T dt = norm3(df);
        if (dt < d) {
            d = dt;
#pragma unroll
            for (int k = 0; k < 3; ++k) { pts[k] = P0[k]; pts[3 + k] = P1[k]; }
        }
    }
    return d;
}

// distanceLineSegToPoint with nearest points.
template <typename T>
RPM_HD T seg_point_pts(const Num<T> &nm, const T *A, const T *B, const T *C, T *pts, bool &has) {
    T BA[3], CA[3], P0[3], df[3];
    sub3(B, A, BA); sub3(C, A, CA);
    const T t = dot3(CA, BA) / dot3(BA, BA);
#pragma unroll
    for (int k = 0; k < 3; ++k) P0[k] = t < T(0) ? A[k] : (t > T(1) ? B[k] : A[k] + t * BA[k]);
    sub3(C, P0, df);
    const T d = norm3(df);
    if (d < nm.eq) { has = false; return T(0); }
#pragma unroll
    for (int k = 0; k < 3; ++k) { pts[k] = P0[k]; pts[3 + k] = C[k]; }
    has = true;
    return d;
}

// CapsuleToBox::compute with nearest points.  Returns d_c (radius subtracted
// except when an endpoint is inside); pts / has as described above.
template <typename T>
RPM_HD T capsule_box_pts(const Num<T> &nm, const T *A, const T *B, T radius, const T *o, T *pts, bool &has) {
    ExactPol pol;
    for (int k = 0; k < 6; ++k) pts[k] = T(0);
    has = true;
    // ---- projections of A and B on the six faces
    unsigned projA = 0u, projB = 0u;
    T distA = nm.maxd, distB = nm.maxd;
    for (int c = 0; c < 3; ++c) {
        const int u = (c == 0) ? 1 : 0, v = (c == 2) ? 1 : 2;
        for (int i = 0; i < 2; ++i) {
            const T *X = i ? B : A;
            if (X[u] >= o[u] && X[u] <= o[3 + u] && X[v] >= o[v] && X[v] <= o[3 + v]) {
                if (X[c] > o[c] && X[c] < o[3 + c]) { has = false; return T(0); }
                unsigned &pj = i ? projB : projA;
                T &dj = i ? distB : distA;
                if (X[c] <= o[c]) { pj |= 1u << c; dj = o[c] - X[c]; }
                else if (X[c] >= o[3 + c]) { pj |= 1u << (3 + c); dj = X[c] - o[3 + c]; }
            }
        }
    }
    T d = nm.maxd;
    if (projA | projB) {
        const int ip = (distA < distB) ? 0 : 1;
        d = (distB < distA) ? distB : distA;
        const T *X = ip ? B : A;
        const unsigned pm = ip ? projB : projA;
        int face = 0;                         // first face (index order) it projects on
        while (!((pm >> face) & 1u)) ++face;
        for (int k = 0; k < 3; ++k) { pts[k] = X[k]; pts[3 + k] = X[k]; }
        pts[3 + face % 3] = o[face];
        if ((projA & projB) == 0u) {
            // checkEdges (:476-540): the projected face's rectangle, then its edges facing the other point
            const int cf = (pm & 1u) ? 0 : (pm & 8u) ? 3 : (pm & 2u) ? 1 : (pm & 16u) ? 4 : (pm & 4u) ? 2 : 5;
            if (coll_rect(pol, nm, A, B, T(0), o, cf)) return T(0) - radius;   // crossing: points kept
            const T *Q = ip ? A : B;
            const int c = cf > 2 ? cf - 3 : cf;
            const int u = (c == 0) ? 1 : 0, v = (c == 2) ? 1 : 2;
            const int fb = (cf > 2 ? 1 : 0) << c;
            int corners[4], n = 0;
            const T qu = Q[u], qv = Q[v];
            if (qu < o[u]) { corners[n++] = fb; corners[n++] = fb | (1 << v); }
            else if (qu > o[3 + u]) { corners[n++] = fb | (1 << u); corners[n++] = fb | (1 << u) | (1 << v); }
            if (qv < o[v]) { corners[n++] = fb; corners[n++] = fb | (1 << u); }
            else if (qv > o[3 + v]) { corners[n++] = fb | (1 << v); corners[n++] = fb | (1 << u) | (1 << v); }
            for (int k = 0; k < n; k += 2) {
                T Cc[3], Dd[3], tp[6];
                bool hp;
                corner(o, corners[k], Cc);
                corner(o, corners[k + 1], Dd);
                const T dt = seg_seg_pts(nm, A, B, Cc, Dd, tp, hp);
                if (dt <= T(0)) { d = T(0); break; }
                if (dt < d) {
                    d = dt;
                    for (int q = 0; q < 6; ++q) pts[q] = tp[q];
                }
            }
        }
        return d - radius;
    }
    // ---- checkOtherCases (:597-755): region of the segment per axis
    int rg[3];
    for (int c = 0; c < 3; ++c) {
        if (A[c] < o[c] && B[c] < o[c]) rg[c] = 0;
        else if (A[c] > o[3 + c] && B[c] > o[3 + c]) rg[c] = 2;
        else rg[c] = 1;
    }
    const int mids = (rg[0] == 1) + (rg[1] == 1) + (rg[2] == 1);
    const int base = (rg[0] == 2 ? 1 : 0) | (rg[1] == 2 ? 2 : 0) | (rg[2] == 2 ? 4 : 0);
    if (mids == 0) {   // a corner
        T Cc[3];
        corner(o, base, Cc);
        d = seg_point_pts(nm, A, B, Cc, pts, has);
        return d - radius;
    }
    if (mids == 1) {   // one box edge; its result replaces d_c and the matrix
        const int k = (rg[0] == 1) ? 0 : (rg[1] == 1 ? 1 : 2);
        T Cc[3], Dd[3];
        corner(o, base, Cc);
        corner(o, base | (1 << k), Dd);
        d = seg_seg_pts(nm, A, B, Cc, Dd, pts, has);
        return d - radius;
    }
    int kind, fu = 0, fv = 0, ne;
    if (mids == 2) {
        const int f = (rg[0] != 1) ? 0 : (rg[1] != 1 ? 1 : 2);
        kind = kEdgesFaceLoop;
        ne = 4;
        fu = (f == 0) ? 1 : 0;
        fv = (f == 2) ? 1 : 2;
    } else {
        for (int f = 0; f < 6; ++f)
            if (coll_rect(pol, nm, A, B, T(0), o, f)) return T(0) - radius;   // crossing: matrix as it is
        kind = kEdgesAll12;
        ne = 12;
    }
    for (int k = 0; k < ne; ++k) {
        int c0, c1;
        edge_of(kind, 0u, base, fu, fv, k, c0, c1);
        T Cc[3], Dd[3], tp[6];
        bool hp;
        corner(o, c0, Cc);
        corner(o, c1, Dd);
        const T dt = seg_seg_pts(nm, A, B, Cc, Dd, tp, hp);
        if (dt <= T(0)) { d = T(0); break; }
        if (dt < d) {
            d = dt;
            for (int q = 0; q < 6; ++q) pts[q] = tp[q];
        }
    }
    return d - radius;
}

// Parameters of the nearest-point and underestimation kernels.
struct NearParams {
    const DevRobot *robot;
    const float *obs_f;      // [8][n_pad]
    const double *obs_d;     // [7][n_pad]
    int32_t n, n_pad;
    const float *q;          // [C][D]
    int64_t C;
    Num<double> nmd;
    Num<float> nmf;
    double *dist;            // [C]
    float *profile;          // [C][L]
    float *nearest;          // [C][n][6][L] (output of the first kernel, input of the second)
    uint8_t *flag;           // [C] nearest points valid / underestimation complete
    double *margin_valid;    // [C] decision margins (rpm_decision_margins)
    double *margin_dist;     // [C]
    float *skel_out;         // [C][3 (D + 1)] the reference's float skeleton (one CTA per state), nullable
};

cudaError_t launch_distance_nearest(int mode, const NearParams &p, cudaStream_t st);
cudaError_t launch_distance_underest(int mode, const NearParams &p, cudaStream_t st);
cudaError_t launch_decision_margins(const NearParams &p, cudaStream_t st);

}  // namespace rpm
