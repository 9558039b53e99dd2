// rpm_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the "oracle").
//
// A CPU restatement of RPMPLv2's RealVectorSpace collision and distance path,
// used by tests/ and by bench.py's CPU-baseline leg as the checker.  It is never
// linked into, loaded by, or called from the product library.
//
// It follows the reference source branch by branch:
//   collisionCapsuleToBox        src/state_spaces/real_vector_space/CollisionAndDistance.cpp:4-42
//   collisionCapsuleToRectangle  CollisionAndDistance.cpp:46-111
//   checkCases / get3DPoint      CollisionAndDistance.cpp:113-155
//   distanceLineSegToLineSeg     CollisionAndDistance.cpp:217-320
//   distanceLineSegToPoint       CollisionAndDistance.cpp:323-342
//   CapsuleToBox (compute, projectionLineSegOnSide, checkEdges, getLineSegments,
//                 distanceToMoreLineSegments, checkOtherCases)  CollisionAndDistance.cpp:395-755
//   RealVectorSpace::isValid(q) / isValid(q1,q2) / computeDistance / interpolateEdge
//                                src/state_spaces/real_vector_space/RealVectorSpace.cpp:75-88, 261-392
//   xArm6 FK + skeleton          src/robots/xArm6.cpp:107-134, 209-235
//   Planar2DOF-family FK + skeleton src/robots/Planar2DOF.cpp:82-130 (Spatial10DOF.cpp:5-9)
//   fcl world AABB of a box      src/environments/objects/Box.cpp:6-7 (fcl 0.7 CollisionObject::computeAABB)
//
// Two numeric instantiations:
//   ref32 -- the reference's own numerics: FK in double, skeleton rounded to
//            float (xArm6.cpp:215-231), float narrow phase; Eigen fixed-size-3
//            reductions evaluated as x0 + (x1 + x2); r_new computed in double
//            (sqrt(3) is the double overload, CollisionAndDistance.cpp:7).
//   ref64 -- the same code with double everywhere.
// Build with -ffp-contract=off so that no multiply-add is fused.
//
// Trigonometry of the FK: KDL calls libm sin/cos.  The oracle offers libm
// (trig = 1) and a Cody-Waite + Taylor-series sincos (trig = 0, default) whose
// bits are identical on every IEEE-754 machine; the GPU FP64 form uses the same
// published method, so FP64 results can be compared bit for bit.
#include "../include/rpm_gpu.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ------------------------------------------------------------------ sincos --
// Cody-Waite reduction by pi/2 split into three parts (P1, P2 carry 33
// significant bits so k*P1 and k*P2 are exact for |k| < 2^20), then Taylor
// series of sin and cos on [-pi/4, pi/4] (terms through r^17 and r^18).
const double kTwoOverPi = 0x1.45f306dc9c883p-1;
const double kP1 = 0x1.921fb54400000p+0;
const double kP2 = 0x1.0b4611a600000p-34;
const double kP3 = 0x1.3198a2e037073p-69;
const double kS[8] = {-0x1.5555555555555p-3, 0x1.1111111111111p-7, -0x1.a01a01a01a01ap-13, 0x1.71de3a556c734p-19,
                      -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33, -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49};
const double kC[9] = {-0x1.0000000000000p-1, 0x1.5555555555555p-5, -0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16,
                      -0x1.27e4fb7789f5cp-22, 0x1.1eed8eff8d898p-29, -0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45,
                      -0x1.6827863b97d97p-53};

void taylor_sincos(double x, double *s_out, double *c_out) {
    double kd = std::nearbyint(x * kTwoOverPi);
    double r = x - kd * kP1;
    r = r - kd * kP2;
    r = r - kd * kP3;
    double z = r * r;
    double ps = kS[7];
    for (int i = 6; i >= 0; --i) ps = kS[i] + z * ps;
    double s = r + (r * z) * ps;
    double pc = kC[8];
    for (int i = 7; i >= 0; --i) pc = kC[i] + z * pc;
    double c = 1.0 + z * pc;
    long long k = (long long)kd;
    switch (k & 3) {
        case 0: *s_out = s; *c_out = c; break;
        case 1: *s_out = c; *c_out = -s; break;
        case 2: *s_out = -s; *c_out = -c; break;
        default: *s_out = -c; *c_out = s; break;
    }
}

void fk_sincos(double x, int trig, double *s, double *c) {
    if (trig == 1) { *s = std::sin(x); *c = std::cos(x); }
    else taylor_sincos(x, s, c);
}

// ---------------------------------------------------------------------- FK --
struct Frame { double R[9]; double p[3]; };   // R row-major

bool is_identity(const double *M) {
    return M[0] == 1.0 && M[1] == 0.0 && M[2] == 0.0 && M[3] == 0.0 && M[4] == 1.0 && M[5] == 0.0 &&
           M[6] == 0.0 && M[7] == 0.0 && M[8] == 1.0;
}

// F <- F * (origin_k) * Rot(axis_k, q_k).  KDL composes segment poses from the
// root (TreeFkSolverPos_recursive); a revolute segment's pose is the URDF
// origin frame followed by the joint rotation.
void fk_step(Frame &F, const rpm_robot_desc &rb, int k, double q, int trig) {
    const double *o = rb.origin_xyz[k];
    const double *M = rb.origin_rot[k];
    double np[3];
    for (int i = 0; i < 3; ++i) np[i] = ((F.R[3 * i + 0] * o[0] + F.R[3 * i + 1] * o[1]) + F.R[3 * i + 2] * o[2]) + F.p[i];
    for (int i = 0; i < 3; ++i) F.p[i] = np[i];
    if (!is_identity(M)) {
        double nR[9];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                nR[3 * i + j] = (F.R[3 * i + 0] * M[0 + j] + F.R[3 * i + 1] * M[3 + j]) + F.R[3 * i + 2] * M[6 + j];
        std::memcpy(F.R, nR, sizeof nR);
    }
    double s, c;
    fk_sincos(q, trig, &s, &c);
    int ia, ib;   // columns: new a = a*c + b*s ; new b = b*c - a*s
    switch (rb.joint_axis[k]) {
        case 0: ia = 1; ib = 2; break;
        case 1: ia = 2; ib = 0; break;
        default: ia = 0; ib = 1; break;
    }
    for (int i = 0; i < 3; ++i) {
        double a = F.R[3 * i + ia], b = F.R[3 * i + ib];
        F.R[3 * i + ia] = a * c + b * s;
        F.R[3 * i + ib] = b * c - a * s;
    }
}

// Skeleton in double (ref64) and with the reference's float rounding (ref32).
void skeleton(const rpm_robot_desc &rb, const float *q, int trig, double *p64, float *p32) {
    const int D = rb.num_dofs;
    Frame F;
    for (int i = 0; i < 9; ++i) F.R[i] = (i % 4 == 0) ? 1.0 : 0.0;
    F.p[0] = F.p[1] = F.p[2] = 0.0;
    if (rb.kind != RPM_ROBOT_XARM6) {
        // Planar2DOF.cpp:125-126: skeleton col k = frames[k].p, k = 0..D
        for (int k = 0; k < D; ++k) {
            fk_step(F, rb, k, (double)q[k], trig);
            for (int i = 0; i < 3; ++i) { p64[3 * k + i] = F.p[i]; p32[3 * k + i] = (float)F.p[i]; }
        }
        const double *o = rb.origin_xyz[D];
        for (int i = 0; i < 3; ++i) {
            double v = ((F.R[3 * i + 0] * o[0] + F.R[3 * i + 1] * o[1]) + F.R[3 * i + 2] * o[2]) + F.p[i];
            p64[3 * D + i] = v;
            p32[3 * D + i] = (float)v;
        }
        return;
    }
    // xArm6: frames F0..F5 (xArm6.cpp:119-129), gripper shift (:130), recipe (:215-231)
    Frame Fr[6];
    for (int k = 0; k < 6; ++k) { fk_step(F, rb, k, (double)q[k], trig); Fr[k] = F; }
    const double g = (double)rb.gripper_length;
    for (int i = 0; i < 3; ++i) Fr[5].p[i] = Fr[5].p[i] + g * Fr[5].R[3 * i + 2];
    for (int i = 0; i < 3; ++i) {
        double v0 = 0.0, v1 = Fr[1].p[i], v2 = Fr[2].p[i];
        double v3 = Fr[3].p[i] - Fr[3].R[3 * i + 2] * 0.25;
        double v4 = Fr[4].p[i];
        double v5 = Fr[4].p[i] + Fr[4].R[3 * i + 0] * 0.076;
        double z5 = Fr[5].R[3 * i + 2];
        double v6 = Fr[5].p[i] - (0.3 * g) * z5;
        double vv[7] = {v0, v1, v2, v3, v4, v5, v6};
        for (int k = 0; k < 7; ++k) p64[3 * k + i] = vv[k];
        for (int k = 0; k < 6; ++k) p32[3 * k + i] = (float)vv[k];
        // Line (*) of xArm6.cpp:231 runs in float: col(6) -= float(0.3*g) * Vector3f(z5)
        float s32 = (float)(0.3 * g);
        p32[3 * 6 + i] = (float)Fr[5].p[i] - s32 * (float)z5;
    }
}

// ---------------------------------------------------------- narrow phase --
template <typename T> struct Num {
    T eq, maxd;
};

template <typename T> inline T dot3(const T *a, const T *b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
template <typename T> inline T norm3(const T *a) { return std::sqrt(dot3(a, a)); }
template <typename T> inline T smin(T a, T b) { return (b < a) ? b : a; }   // std::min
template <typename T> inline void sub3(const T *a, const T *b, T *o) { o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2]; }

template <typename T> inline T rnew_of(T radius);
template <> inline float rnew_of<float>(float radius) { return (float)((double)radius * std::sqrt(3.0) / 3); }
template <> inline double rnew_of<double>(double radius) { return radius * std::sqrt(3.0) / 3; }

// get3DPoint (CollisionAndDistance.cpp:150-155)
template <typename T> inline void pt3(T u, T v, T value, int coord, T *o) {
    if (coord == 0) { o[0] = value; o[1] = u; o[2] = v; }
    else if (coord == 1) { o[0] = u; o[1] = value; o[2] = v; }
    else { o[0] = u; o[1] = v; o[2] = value; }
}

// distanceLineSegToLineSeg (CollisionAndDistance.cpp:217-320).  Returns d;
// pts (robot point, obstacle point) are written when has_pts is set.
template <typename T>
T seg_seg(const Num<T> &nm, const T *A, const T *B, const T *C, const T *D, T *pts, bool *has_pts) {
    T d_c = nm.maxd;
    T BA[3], DC[3], CD[3], AC[3], AB[3];
    sub3(B, A, BA); sub3(D, C, DC); sub3(C, D, CD); sub3(A, C, AC); sub3(A, B, AB);
    T alpha1 = dot3(BA, BA);
    T alpha2 = dot3(BA, DC);
    T beta1 = dot3(CD, BA);
    T beta2 = dot3(CD, DC);
    T gamma1 = dot3(AC, AB);
    T gamma2 = dot3(AC, CD);
    T s = (alpha1 * gamma2 - alpha2 * gamma1) / (alpha1 * beta2 - alpha2 * beta1);
    T t = (gamma1 - beta1 * s) / alpha1;
    *has_pts = false;
    if (t > 0 && t < 1 && s > 0 && s < 1) {
        T P1[3], P2[3], df[3];
        for (int i = 0; i < 3; ++i) { P1[i] = A[i] + t * BA[i]; P2[i] = C[i] + s * DC[i]; }
        sub3(P2, P1, df);
        d_c = norm3(df);
        if (d_c < nm.eq) return 0;
        for (int i = 0; i < 3; ++i) { pts[i] = P1[i]; pts[3 + i] = P2[i]; }
        *has_pts = true;
        return d_c;
    }
    T alpha3 = dot3(CD, CD);
    T AD[3], BC[3];
    sub3(A, D, AD); sub3(B, C, BC);
    T opt[4] = {dot3(AC, AB) / alpha1, dot3(AD, AB) / alpha1, dot3(AC, DC) / alpha3, dot3(BC, DC) / alpha3};
    for (int i = 0; i < 4; ++i) {
        T r[3], o[3];
        if (opt[i] < 0) {
            if (i == 0 || i == 2) { std::memcpy(r, A, sizeof r); std::memcpy(o, C, sizeof o); }
            else if (i == 1) { std::memcpy(r, A, sizeof r); std::memcpy(o, D, sizeof o); }
            else { std::memcpy(r, B, sizeof r); std::memcpy(o, C, sizeof o); }
        } else if (opt[i] > 1) {
            if (i == 1 || i == 3) { std::memcpy(r, B, sizeof r); std::memcpy(o, D, sizeof o); }
            else if (i == 0) { std::memcpy(r, B, sizeof r); std::memcpy(o, C, sizeof o); }
            else { std::memcpy(r, A, sizeof r); std::memcpy(o, D, sizeof o); }
        } else {
            if (i == 0) { for (int k = 0; k < 3; ++k) r[k] = A[k] + opt[i] * BA[k]; std::memcpy(o, C, sizeof o); }
            else if (i == 1) { for (int k = 0; k < 3; ++k) r[k] = A[k] + opt[i] * BA[k]; std::memcpy(o, D, sizeof o); }
            else if (i == 2) { std::memcpy(r, A, sizeof r); for (int k = 0; k < 3; ++k) o[k] = C[k] + opt[i] * DC[k]; }
            else { std::memcpy(r, B, sizeof r); for (int k = 0; k < 3; ++k) o[k] = C[k] + opt[i] * DC[k]; }
        }
        T df[3];
        sub3(o, r, df);
        T dt = norm3(df);
        if (dt < d_c) {
            d_c = dt;
            for (int k = 0; k < 3; ++k) { pts[k] = r[k]; pts[3 + k] = o[k]; }
            *has_pts = true;
        }
    }
    return d_c;
}

// distanceLineSegToPoint (CollisionAndDistance.cpp:323-342)
template <typename T> T seg_point(const Num<T> &nm, const T *A, const T *B, const T *C, T *pts, bool *has_pts) {
    T BA[3], CA[3];
    sub3(B, A, BA); sub3(C, A, CA);
    T t_opt = dot3(CA, BA) / dot3(BA, BA);
    T r[3];
    if (t_opt < 0) std::memcpy(r, A, sizeof r);
    else if (t_opt > 1) std::memcpy(r, B, sizeof r);
    else for (int k = 0; k < 3; ++k) r[k] = A[k] + t_opt * BA[k];
    T df[3];
    sub3(C, r, df);
    T d = norm3(df);
    *has_pts = false;
    if (d < nm.eq) return 0;
    for (int k = 0; k < 3; ++k) { pts[k] = r[k]; pts[3 + k] = C[k]; }
    *has_pts = true;
    return d;
}

// checkCases (CollisionAndDistance.cpp:113-148)
template <typename T>
T check_cases(const Num<T> &nm, const T *A, const T *B, const T *rec, const T *point, T obs_coord, int coord) {
    T d1 = nm.maxd, d2 = nm.maxd;
    T C[3], D[3], pts[6];
    bool hp;
    if (point[0] < rec[0]) {
        pt3(rec[0], rec[1], obs_coord, coord, C); pt3(rec[0], rec[3], obs_coord, coord, D);
        d1 = seg_seg(nm, A, B, C, D, pts, &hp);
    } else if (point[0] > rec[2]) {
        pt3(rec[2], rec[1], obs_coord, coord, C); pt3(rec[2], rec[3], obs_coord, coord, D);
        d1 = seg_seg(nm, A, B, C, D, pts, &hp);
    }
    if (d1 > 0 && point[1] < rec[1]) {
        pt3(rec[0], rec[1], obs_coord, coord, C); pt3(rec[2], rec[1], obs_coord, coord, D);
        d2 = seg_seg(nm, A, B, C, D, pts, &hp);
    } else if (d1 > 0 && point[1] > rec[3]) {
        pt3(rec[0], rec[3], obs_coord, coord, C); pt3(rec[2], rec[3], obs_coord, coord, D);
        d2 = seg_seg(nm, A, B, C, D, pts, &hp);
    }
    return smin(d1, d2);
}

// collisionCapsuleToRectangle (CollisionAndDistance.cpp:46-111)
template <typename T>
bool coll_rect(const Num<T> &nm, const T *A, const T *B, T radius, const T *obs, int coord) {
    T obs_coord = obs[coord];
    if (coord > 2) coord -= 3;
    int a = (coord == 0) ? 1 : 0, b = (coord == 2) ? 1 : 2;
    T rec[4] = {obs[a], obs[b], obs[3 + a], obs[3 + b]};
    T A_rec[2] = {A[a], A[b]}, B_rec[2] = {B[a], B[b]};
    T t = (B[coord] - A[coord]) != 0 ? (obs_coord - A[coord]) / (B[coord] - A[coord]) : nm.maxd;
    T M[2] = {A_rec[0] + t * (B_rec[0] - A_rec[0]), A_rec[1] + t * (B_rec[1] - A_rec[1])};
    T A_proj[3], B_proj[3];
    pt3(A_rec[0], A_rec[1], obs_coord, coord, A_proj);
    pt3(B_rec[0], B_rec[1], obs_coord, coord, B_proj);
    T dA[3], dB[3];
    sub3(A, A_proj, dA); sub3(B, B_proj, dB);
    auto n2 = [](T x, T y) { return std::sqrt(x * x + y * y); };
    if (t > 0 && t < 1) {
        if (M[0] > rec[0] - radius && M[0] < rec[2] + radius && M[1] > rec[1] - radius && M[1] < rec[3] + radius) {
            if ((M[0] > rec[0] - radius && M[0] < rec[2] + radius && M[1] > rec[1] && M[1] < rec[3]) ||
                (M[1] > rec[1] - radius && M[1] < rec[3] + radius && M[0] > rec[0] && M[0] < rec[2]) ||
                (M[0] < rec[0] && M[1] < rec[2] && n2(M[0] - rec[0], M[1] - rec[2]) < radius) ||
                (M[0] < rec[0] && M[1] > rec[3] && n2(M[0] - rec[0], M[1] - rec[3]) < radius) ||
                (M[0] > rec[1] && M[1] < rec[2] && n2(M[0] - rec[1], M[1] - rec[2]) < radius) ||
                (M[0] > rec[1] && M[1] > rec[3] && n2(M[0] - rec[1], M[1] - rec[3]) < radius))
                return true;
        }
    } else if (smin(norm3(dA), norm3(dB)) > radius)
        return false;

    if (radius > 0) {
        bool a_in = A_rec[0] > rec[0] && A_rec[0] < rec[2] && A_rec[1] > rec[1] && A_rec[1] < rec[3];
        bool b_in = B_rec[0] > rec[0] && B_rec[0] < rec[2] && B_rec[1] > rec[1] && B_rec[1] < rec[3];
        if (a_in) {
            if (b_in) {
                if (smin(norm3(dA), norm3(dB)) < radius) return true;
            } else {
                if (smin(check_cases(nm, A, B, rec, B_rec, obs_coord, coord), norm3(dA)) < radius) return true;
            }
        } else if (b_in) {
            if (smin(check_cases(nm, A, B, rec, A_rec, obs_coord, coord), norm3(dB)) < radius) return true;
        } else {
            if (check_cases(nm, A, B, rec, A_rec, obs_coord, coord) < radius) return true;
            if (check_cases(nm, A, B, rec, B_rec, obs_coord, coord) < radius) return true;
        }
    }
    return false;
}

// collisionCapsuleToBox (CollisionAndDistance.cpp:4-42)
template <typename T> bool coll_box(const Num<T> &nm, const T *A, const T *B, T radius, const T *obs) {
    T r_new = rnew_of<T>(radius);
    if ((A[0] > obs[0] - r_new && A[1] > obs[1] - r_new && A[2] > obs[2] - r_new && A[0] < obs[3] + r_new &&
         A[1] < obs[4] + r_new && A[2] < obs[5] + r_new) ||
        (B[0] > obs[0] - r_new && B[1] > obs[1] - r_new && B[2] > obs[2] - r_new && B[0] < obs[3] + r_new &&
         B[1] < obs[4] + r_new && B[2] < obs[5] + r_new))
        return true;
    else if ((A[0] < obs[0] - radius && B[0] < obs[0] - radius) || (A[0] > obs[3] + radius && B[0] > obs[3] + radius) ||
             (A[1] < obs[1] - radius && B[1] < obs[1] - radius) || (A[1] > obs[4] + radius && B[1] > obs[4] + radius) ||
             (A[2] < obs[2] - radius && B[2] < obs[2] - radius) || (A[2] > obs[5] + radius && B[2] > obs[5] + radius))
        return false;
    bool collision = false;
    if (A[0] < obs[0]) collision = coll_rect(nm, A, B, radius, obs, 0);
    else if (A[0] > obs[3]) collision = coll_rect(nm, A, B, radius, obs, 3);
    if (!collision) {
        if (A[1] < obs[1]) collision = coll_rect(nm, A, B, radius, obs, 1);
        else if (A[1] > obs[4]) collision = coll_rect(nm, A, B, radius, obs, 4);
        if (!collision) {
            if (A[2] < obs[2]) collision = coll_rect(nm, A, B, radius, obs, 2);
            else if (A[2] > obs[5]) collision = coll_rect(nm, A, B, radius, obs, 5);
        }
    }
    return collision;
}

// CapsuleToBox (CollisionAndDistance.cpp:395-755)
// Evaluations that reached the reference's uninitialised-matrix branch of
// getLineSegments (CollisionAndDistance.cpp:542-574 with no edge selected),
// per host thread.
thread_local int64_t g_undefined_hits = 0;

template <typename T> struct CapsuleBox {
    const Num<T> &nm;
    T A[3], B[3], radius, obs[6];
    T d_c;
    T pts[6];
    bool has_pts;
    int proj[6][2];
    T dist_AB[2];

    CapsuleBox(const Num<T> &nm_, const T *A_, const T *B_, T r_, const T *o_) : nm(nm_) {
        std::memcpy(A, A_, sizeof A); std::memcpy(B, B_, sizeof B); std::memcpy(obs, o_, sizeof obs);
        radius = r_;
        d_c = nm.maxd;
        has_pts = true;   // the reference allocates a 3x2 matrix whose content is set on every non-zero path
        std::memset(pts, 0, sizeof pts);
        std::memset(proj, 0, sizeof proj);
        dist_AB[0] = dist_AB[1] = nm.maxd;
    }
    const T *P(int i) const { return i == 0 ? A : B; }

    void projection_on_side(int min1, int min2, int min3, int max1, int max2, int max3) {
        for (int i = 0; i < 2; ++i) {
            const T *X = P(i);
            if (X[min1] >= obs[min1] && X[min1] <= obs[max1] && X[min2] >= obs[min2] && X[min2] <= obs[max2]) {
                if (X[min3] > obs[min3] && X[min3] < obs[max3]) { d_c = 0; return; }
                else if (X[min3] <= obs[min3]) { proj[min3][i] = 1; dist_AB[i] = obs[min3] - X[min3]; }
                else if (X[min3] >= obs[max3]) { proj[max3][i] = 1; dist_AB[i] = X[min3] - obs[max3]; }
            }
        }
    }

    // distanceToMoreLineSegments (:576-595) over segments given as endpoint pairs
    void more_segments(const T (*seg)[3], int nseg2) {
        for (int k = 0; k < nseg2; k += 2) {
            T tp[6];
            bool hp;
            T dt = seg_seg(nm, A, B, seg[k], seg[k + 1], tp, &hp);
            if (dt <= 0) { d_c = 0; return; }   // the reference keeps its point matrix as it is
            else if (dt < d_c) { d_c = dt; std::memcpy(pts, tp, sizeof pts); has_pts = true; }
        }
    }

    // getLineSegments (:542-574) + checkEdges (:476-540)
    void check_edges(const T *point, int idx) {
        static const int order[6] = {0, 3, 1, 4, 2, 5};
        int face = -1;
        for (int f : order) if (proj[f][idx]) { face = f; break; }
        if (face < 0) return;
        if (coll_rect(nm, A, B, T(0), obs, face)) { d_c = 0; return; }   // points left as they are
        int coord = face % 3;
        int a = (coord == 0) ? 1 : 0, b = (coord == 2) ? 1 : 2;
        T p0 = point[a], p1 = point[b];
        T min1 = obs[a], min2 = obs[b], max1 = obs[3 + a], max2 = obs[3 + b], cv = obs[face];
        T seg[4][3];
        int n = 0;
        if (p0 < min1) { pt3(min1, min2, cv, coord, seg[0]); pt3(min1, max2, cv, coord, seg[1]); n = 2; }
        else if (p0 > max1) { pt3(max1, min2, cv, coord, seg[0]); pt3(max1, max2, cv, coord, seg[1]); n = 2; }
        if (p1 < min2) { pt3(min1, min2, cv, coord, seg[n]); pt3(max1, min2, cv, coord, seg[n + 1]); n += 2; }
        else if (p1 > max2) { pt3(min1, max2, cv, coord, seg[n]); pt3(max1, max2, cv, coord, seg[n + 1]); n += 2; }
        // n == 0 leaves the reference's 3x2 matrix uninitialised (undefined); it is
        // reachable only when the segment meets the face rectangle exactly on its
        // border, and is treated here as "no edge".  g_undefined_hits counts it so
        // fixtures can leave such cases out (the reference's answer there is heap
        // garbage, not a value to match).
        if (n == 0) ++g_undefined_hits;
        more_segments(seg, n);
    }

    void set_from(T d, const T *tp, bool hp) { d_c = d; if (hp) std::memcpy(pts, tp, sizeof pts); has_pts = hp; }

    void corner_pt(int ix, int iy, int iz) {
        T Cc[3] = {obs[ix], obs[iy], obs[iz]}, tp[6];
        bool hp;
        T d = seg_point(nm, A, B, Cc, tp, &hp);
        set_from(d, tp, hp);
    }
    void edge_seg(int x0, int y0, int z0, int x1, int y1, int z1) {
        T Cc[3] = {obs[x0], obs[y0], obs[z0]}, Dd[3] = {obs[x1], obs[y1], obs[z1]}, tp[6];
        bool hp;
        T d = seg_seg(nm, A, B, Cc, Dd, tp, &hp);
        set_from(d, tp, hp);
    }
    // A closed loop of four box edges lying in one face, given by its corners.
    void face_loop(const int (*cor)[3]) {
        T seg[8][3];
        for (int e = 0; e < 4; ++e)
            for (int k = 0; k < 2; ++k) {
                const int *c = cor[(e + k) & 3];
                seg[2 * e + k][0] = obs[c[0]]; seg[2 * e + k][1] = obs[c[1]]; seg[2 * e + k][2] = obs[c[2]];
            }
        more_segments(seg, 8);
    }

    void other_cases() {
        const T *o = obs;
        if (A[0] < o[0] && B[0] < o[0]) {
            if (A[1] < o[1] && B[1] < o[1]) {
                if (A[2] < o[2] && B[2] < o[2]) corner_pt(0, 1, 2);
                else if (A[2] > o[5] && B[2] > o[5]) corner_pt(0, 1, 5);
                else edge_seg(0, 1, 2, 0, 1, 5);
            } else if (A[1] > o[4] && B[1] > o[4]) {
                if (A[2] < o[2] && B[2] < o[2]) corner_pt(0, 4, 2);
                else if (A[2] > o[5] && B[2] > o[5]) corner_pt(0, 4, 5);
                else edge_seg(0, 4, 2, 0, 4, 5);
            } else {
                if (A[2] < o[2] && B[2] < o[2]) edge_seg(0, 1, 2, 0, 4, 2);
                else if (A[2] > o[5] && B[2] > o[5]) edge_seg(0, 1, 5, 0, 4, 5);
                else { static const int c[4][3] = {{0, 1, 2}, {0, 4, 2}, {0, 4, 5}, {0, 1, 5}}; face_loop(c); }
            }
        } else if (A[0] > o[3] && B[0] > o[3]) {
            if (A[1] < o[1] && B[1] < o[1]) {
                if (A[2] < o[2] && B[2] < o[2]) corner_pt(3, 1, 2);
                else if (A[2] > o[5] && B[2] > o[5]) corner_pt(3, 1, 5);
                else edge_seg(3, 1, 2, 3, 1, 5);
            } else if (A[1] > o[4] && B[1] > o[4]) {
                if (A[2] < o[2] && B[2] < o[2]) corner_pt(3, 4, 2);
                else if (A[2] > o[5] && B[2] > o[5]) corner_pt(3, 4, 5);
                else edge_seg(3, 4, 2, 3, 4, 5);
            } else {
                if (A[2] < o[2] && B[2] < o[2]) edge_seg(3, 1, 2, 3, 4, 2);
                else if (A[2] > o[5] && B[2] > o[5]) edge_seg(3, 1, 5, 3, 4, 5);
                else { static const int c[4][3] = {{3, 1, 2}, {3, 4, 2}, {3, 4, 5}, {3, 1, 5}}; face_loop(c); }
            }
        } else {
            if (A[1] < o[1] && B[1] < o[1]) {
                if (A[2] < o[2] && B[2] < o[2]) edge_seg(0, 1, 2, 3, 1, 2);
                else if (A[2] > o[5] && B[2] > o[5]) edge_seg(0, 1, 5, 3, 1, 5);
                else { static const int c[4][3] = {{0, 1, 2}, {3, 1, 2}, {3, 1, 5}, {0, 1, 5}}; face_loop(c); }
            } else if (A[1] > o[4] && B[1] > o[4]) {
                if (A[2] < o[2] && B[2] < o[2]) edge_seg(0, 4, 2, 3, 4, 2);
                else if (A[2] > o[5] && B[2] > o[5]) edge_seg(0, 4, 5, 3, 4, 5);
                else { static const int c[4][3] = {{0, 4, 2}, {3, 4, 2}, {3, 4, 5}, {0, 4, 5}}; face_loop(c); }
            } else {
                if (A[2] < o[2] && B[2] < o[2]) { static const int c[4][3] = {{0, 1, 2}, {3, 1, 2}, {3, 4, 2}, {0, 4, 2}}; face_loop(c); }
                else if (A[2] > o[5] && B[2] > o[5]) { static const int c[4][3] = {{0, 1, 5}, {3, 1, 5}, {3, 4, 5}, {0, 4, 5}}; face_loop(c); }
                else {
                    for (int kk = 0; kk < 6; ++kk)
                        if (coll_rect(nm, A, B, T(0), obs, kk)) { d_c = 0; return; }   // points left as they are
                    // the 12 box edges: bottom loop, top loop, four verticals (:747-750)
                    static const int e12[24][3] = {
                        {0, 1, 2}, {3, 1, 2}, {3, 1, 2}, {3, 4, 2}, {3, 4, 2}, {0, 4, 2}, {0, 4, 2}, {0, 1, 2},
                        {0, 1, 5}, {3, 1, 5}, {3, 1, 5}, {3, 4, 5}, {3, 4, 5}, {0, 4, 5}, {0, 4, 5}, {0, 1, 5},
                        {0, 1, 2}, {0, 1, 5}, {3, 1, 2}, {3, 1, 5}, {3, 4, 2}, {3, 4, 5}, {0, 4, 2}, {0, 4, 5}};
                    T seg[24][3];
                    for (int k = 0; k < 24; ++k) { seg[k][0] = o[e12[k][0]]; seg[k][1] = o[e12[k][1]]; seg[k][2] = o[e12[k][2]]; }
                    more_segments(seg, 24);
                }
            }
        }
    }

    void compute() {
        projection_on_side(1, 2, 0, 4, 5, 3);
        projection_on_side(0, 2, 1, 3, 5, 4);
        projection_on_side(0, 1, 2, 3, 4, 5);
        if (d_c == 0) { has_pts = false; return; }
        int num_proj = 0;
        for (int f = 0; f < 6; ++f) num_proj = std::max(num_proj, proj[f][0] + proj[f][1]);
        if (num_proj > 0) {
            int ip = (dist_AB[0] < dist_AB[1]) ? 0 : 1;
            d_c = smin(dist_AB[0], dist_AB[1]);
            int ic = 0;
            for (int f = 1; f < 6; ++f) if (proj[f][ip] > proj[ic][ip]) ic = f;
            const T *X = P(ip);
            for (int k = 0; k < 3; ++k) { pts[k] = X[k]; pts[3 + k] = X[k]; }
            pts[3 + ic % 3] = obs[ic];
            has_pts = true;
            if (num_proj == 1) {
                if (ip == 0) check_edges(B, 0);
                else check_edges(A, 1);
            }
        } else
            other_cases();
        d_c -= radius;
    }
};

struct Obstacles {
    const float *aabb;   // n x 6
    const float *tol;    // n (nullable -> max distance)
    const uint8_t *flags;
    int n;
};

template <typename T> struct Scene {
    std::vector<T> box;   // n x 6
    std::vector<T> tol;
    std::vector<uint8_t> ground;
    int n;
    Scene(const Obstacles &ob, double maxd) : box(6 * (size_t)ob.n), tol(ob.n), ground(ob.n), n(ob.n) {
        for (int j = 0; j < n; ++j) {
            for (int k = 0; k < 6; ++k) box[6 * j + k] = (T)ob.aabb[6 * j + k];
            tol[j] = ob.tol ? (T)ob.tol[j] : (T)maxd;
            ground[j] = ob.flags ? (ob.flags[j] & RPM_OBS_GROUND) : 0;
        }
    }
};

// RealVectorSpace::isValid(q) (RealVectorSpace.cpp:277-309) on a skeleton
template <typename T>
bool is_valid(const Num<T> &nm, const rpm_robot_desc &rb, const Scene<T> &sc, const T *skel) {
    for (int i = 0; i < rb.num_dofs; ++i)
        for (int j = 0; j < sc.n; ++j) {
            if (sc.ground[j] && i < rb.ground_included) continue;
            if (coll_box(nm, skel + 3 * i, skel + 3 * (i + 1), (T)rb.capsule_radius[i], &sc.box[6 * j])) return false;
        }
    return true;
}

// RealVectorSpace::computeDistance(q, true) (RealVectorSpace.cpp:318-392).
// profile has L entries; nearest (nullable) is n x 6 x L like the
// reference's vector<MatrixXf(6, L)>.  Returns d_c; *nearest_valid is false
// when the reference sets nearest points to nullptr.
template <typename T>
T compute_distance(const Num<T> &nm, const rpm_robot_desc &rb, const Scene<T> &sc, const T *skel, T *profile,
                   T *nearest, bool *nearest_valid) {
    const int L = rb.num_dofs;
    T d_c = nm.maxd;
    for (int i = 0; i < L; ++i) profile[i] = 0;
    for (int i = 0; i < L; ++i) {
        profile[i] = nm.maxd;
        for (int j = 0; j < sc.n; ++j) {
            T d;
            T np[6];
            if (sc.ground[j] && i < rb.ground_included) {
                d = nm.maxd;
                np[0] = np[1] = np[2] = 0; np[3] = 0; np[4] = 0; np[5] = -nm.maxd;
            } else {
                CapsuleBox<T> cb(nm, skel + 3 * i, skel + 3 * (i + 1), (T)rb.capsule_radius[i], &sc.box[6 * j]);
                cb.compute();
                d = cb.d_c;
                std::memcpy(np, cb.pts, sizeof np);
            }
            if (d > sc.tol[j]) d = nm.maxd;
            profile[i] = smin(profile[i], d);
            if (profile[i] <= 0) {
                if (nearest_valid) *nearest_valid = false;
                return 0;
            }
            if (nearest)
                for (int k = 0; k < 6; ++k) nearest[((size_t)j * 6 + k) * L + i] = np[k];
        }
        d_c = smin(d_c, profile[i]);
    }
    if (nearest_valid) *nearest_valid = true;
    return d_c;
}

template <typename T> Num<T> num_of(const rpm_params *p) {
    Num<T> nm;
    nm.eq = p ? (T)p->equality_threshold : (T)1e-4;
    nm.maxd = p ? (T)p->max_distance : (T)1000;
    return nm;
}

int nthreads_of(int nt) {
#ifdef _OPENMP
    return nt > 0 ? nt : omp_get_max_threads();
#else
    (void)nt;
    return 1;
#endif
}

template <typename T>
void config_one(const Num<T> &nm, const rpm_robot_desc &rb, const Scene<T> &sc, const T *skel, uint8_t *valid,
                double *dist, float *profile) {
    const int L = rb.num_dofs;
    if (valid) *valid = is_valid(nm, rb, sc, skel) ? 1 : 0;
    if (dist || profile) {
        T prof[RPM_MAX_DOF];
        T d = compute_distance(nm, rb, sc, skel, prof, (T *)nullptr, (bool *)nullptr);
        if (dist) *dist = (double)d;
        if (profile) for (int i = 0; i < L; ++i) profile[i] = (float)prof[i];
    }
}

}  // namespace

// RealVectorSpace::computeDistanceUnderestimation (RealVectorSpace.cpp:402-446)
// from given nearest points (n x 6 x L, the reference's vector<MatrixXf(6, L)>):
// the distance of each link to the plane through the obstacle point O with
// normal (R - O) / |R - O| (Eigen's normalized(): unchanged when |R - O| = 0),
// minus the radius.  Pairs whose O has norm MAX_DISTANCE (the ground pairs the
// ground rule skips) are passed over.  *complete is false when the reference
// returns 0 at the first negative value without updating the state.
template <typename T>
T distance_underest(const Num<T> &nm, const rpm_robot_desc &rb, int n, const T *skel, const float *near, T *profile,
                    bool *complete) {
    const int L = rb.num_dofs;
    T d_c = nm.maxd;
    for (int i = 0; i < L; ++i) profile[i] = 0;
    for (int i = 0; i < L; ++i) {
        profile[i] = nm.maxd;
        for (int j = 0; j < n; ++j) {
            T O[3], R[3];
            for (int k = 0; k < 3; ++k) {
                R[k] = (T)near[((size_t)j * 6 + k) * L + i];
                O[k] = (T)near[((size_t)j * 6 + 3 + k) * L + i];
            }
            if (std::sqrt(dot3(O, O)) == nm.maxd) continue;
            T u[3] = {R[0] - O[0], R[1] - O[1], R[2] - O[2]};
            const T z = dot3(u, u);
            if (z > T(0)) {
                const T nz = std::sqrt(z);
                for (int k = 0; k < 3; ++k) u[k] = u[k] / nz;
            }
            const T *S0 = skel + 3 * i, *S1 = skel + 3 * (i + 1);
            T a[3] = {S0[0] - O[0], S0[1] - O[1], S0[2] - O[2]};
            T b[3] = {S1[0] - O[0], S1[1] - O[1], S1[2] - O[2]};
            const T d = smin(dot3(a, u), dot3(b, u)) - (T)rb.capsule_radius[i];
            if (d < T(0)) {
                *complete = false;
                return 0;
            }
            profile[i] = smin(profile[i], d);
        }
        d_c = smin(d_c, profile[i]);
    }
    *complete = true;
    return d_c;
}

// ------------------------------------------------------------------ spines --
// The bubble and spine steps of the RBT planners in the reference's float
// numerics.  Sums over dynamic-size Eigen expressions (a skeleton column,
// R->col(i).dot(delta_q)) run in index order; fixed-size 3-vector reductions
// as x0 + (x1 + x2).  Eigen's order for dynamic sizes is not pinned by any
// reference test.
enum { kStNone = 0, kStAdvanced = 1, kStTrapped = 2, kStReached = 3 };   // base::State::Status (State.h:22)

inline float maxf_std(float a, float b) { return (a < b) ? b : a; }   // std::max

// |a - b| over dynamic 3-element columns, summed in index order.
inline float col_dist(const float *a, const float *b) {
    float s = 0.f;
    for (int k = 0; k < 3; ++k) {
        const float d = a[k] - b[k];
        s = s + d * d;
    }
    return std::sqrt(s);
}

// computeEnclosingRadii from the float skeleton sk (D + 1 points): R is
// D x (D + 1), row-major.  xArm6.cpp:237-275 (radii max(r_i, r_i+1), rows 0
// and 3 projected), Spatial10DOF.cpp:11-30 (row 0 projected on {x, y}),
// Planar2DOF.cpp:132-148 (no projection).
void enclosing_radii(const rpm_robot_desc &rb, const float *sk, float *R) {
    const int D = rb.num_dofs, W = D + 1;
    for (int i = 0; i < D * W; ++i) R[i] = 0.f;
    if (rb.kind == RPM_ROBOT_XARM6) {
        float rn[RPM_MAX_DOF];
        for (int i = 0; i < D - 1; ++i) rn[i] = maxf_std(rb.capsule_radius[i], rb.capsule_radius[i + 1]);
        rn[D - 1] = rb.capsule_radius[D - 1];
        for (int i = 0; i < D - 1; ++i)
            for (int j = i + 1; j <= D; ++j) {
                const float *pj = sk + 3 * j;
                if (i == 0) {
                    if (j >= 2) R[j] = maxf_std(R[j - 1], std::sqrt(pj[0] * pj[0] + pj[1] * pj[1]) + rn[j - 1]);
                } else if (i == 3) {
                    if (j >= 5) {
                        const float *p3 = sk + 9, *p4 = sk + 12;
                        float AB[3], v[3], proj[3], w[3];
                        sub3(p4, p3, AB);
                        sub3(pj, p3, v);
                        const float t = dot3(v, AB) / dot3(AB, AB);
                        for (int k = 0; k < 3; ++k) proj[k] = p3[k] + t * AB[k];
                        sub3(pj, proj, w);
                        R[3 * W + j] = maxf_std(R[3 * W + j - 1], norm3(w) + rn[j - 1]);
                    }
                } else {
                    R[i * W + j] = maxf_std(R[i * W + j - 1], col_dist(pj, sk + 3 * i) + rn[j - 1]);
                }
            }
        return;
    }
    const bool spatial = rb.kind == RPM_ROBOT_SPATIAL;
    for (int i = 0; i < D; ++i)
        for (int j = i + 1; j <= D; ++j) {
            const float *pj = sk + 3 * j;
            const float v = (i == 0 && spatial) ? std::sqrt(pj[0] * pj[0] + pj[1] * pj[1]) : col_dist(pj, sk + 3 * i);
            R[i * W + j] = maxf_std(R[i * W + j - 1], v + rb.capsule_radius[j - 1]);
        }
}

// RBTConnect::extendSpine (RBTConnect.cpp:85-150) with self-collision checking
// off: from q (distance d, profile prof) towards qe.  Returns the status;
// q_new is the spine's end.
int extend_spine(const rpm_robot_desc &rb, int trig, const float *q, float d, const float *prof, const float *qe,
                 int num_iter, bool expanded, float *q_new) {
    const int D = rb.num_dofs, L = D, W = D + 1;
    if (d <= 0) {
        for (int k = 0; k < D; ++k) q_new[k] = q[k];
        return kStTrapped;
    }
    double p64[3 * (RPM_MAX_DOF + 1)];
    float sk0[3 * (RPM_MAX_DOF + 1)], skt[3 * (RPM_MAX_DOF + 1)], skn[3 * (RPM_MAX_DOF + 1)];
    float R[RPM_MAX_DOF * (RPM_MAX_DOF + 1)];
    float rho_profile[RPM_MAX_DOF] = {0.f}, qt[RPM_MAX_DOF], dq[RPM_MAX_DOF];
    float rho = 0.f;
    skeleton(rb, q, trig, p64, sk0);
    for (int k = 0; k < D; ++k) qt[k] = q[k];
    int status = kStAdvanced, counter = 0;
    for (;;) {
        skeleton(rb, qt, trig, p64, skt);
        enclosing_radii(rb, skt, R);
        for (int k = 0; k < D; ++k) dq[k] = std::fabs(qe[k] - qt[k]);
        float step;
        if (expanded) {
            step = INFINITY;
            for (int i = 0; i < D; ++i) {
                float s = 0.f;
                for (int k = 0; k < D; ++k) s = s + R[k * W + i + 1] * dq[k];
                step = smin(step, (prof[i] - rho_profile[i]) / s);
            }
        } else {
            float s = 0.f;
            for (int k = 0; k < D; ++k) s = s + R[k * W + D] * dq[k];
            step = (d - rho) / s;
        }
        if (step > 1.f) {
            for (int k = 0; k < D; ++k) q_new[k] = qe[k];
            status = kStReached;
        } else {
            for (int k = 0; k < D; ++k) q_new[k] = qt[k] + step * (qe[k] - qt[k]);
        }
        if (++counter == num_iter || status != kStAdvanced) return status;
        skeleton(rb, q_new, trig, p64, skn);
        float rk_prev = 0.f;
        for (int k = 1; k <= L; ++k) {
            const float rk = col_dist(sk0 + 3 * k, skn + 3 * k);
            rho_profile[k - 1] = maxf_std(rk_prev, rk);
            rk_prev = rk;
            rho = maxf_std(rho, rk);
        }
        for (int k = 0; k < D; ++k) qt[k] = q_new[k];
    }
}

// DRGBT::computeReachedState (DRGBT.cpp:475-495) without its final
// computeDistance: RGBTConnect::extendGenSpine (RGBTConnect.cpp:73-93) from
// q_cur (distance d_cur, profile prof_cur, nearest points near_cur) towards
// qe, with computeDistanceUnderestimation from q_cur's nearest points after
// every layer.
int reached_state(const Num<float> &nm, const rpm_robot_desc &rb, int trig, int n, const float *q_cur, float d_cur,
                  const float *prof_cur, const float *near_cur, const float *qe, int num_layers, int num_iter,
                  bool expanded, float d_crit, float *q_out) {
    const int D = rb.num_dofs, L = D;
    for (int k = 0; k < D; ++k) q_out[k] = q_cur[k];
    if (d_cur <= 0) return kStTrapped;
    float qn[RPM_MAX_DOF], pn[RPM_MAX_DOF], qs[RPM_MAX_DOF];
    for (int k = 0; k < D; ++k) qn[k] = q_cur[k];
    for (int i = 0; i < L; ++i) pn[i] = prof_cur[i];
    float dn = d_cur;
    int status = kStNone;
    for (int layer = 0; layer < num_layers; ++layer) {
        status = extend_spine(rb, trig, qn, dn, pn, qe, num_iter, expanded, qs);
        for (int k = 0; k < D; ++k) qn[k] = qs[k];
        double p64[3 * (RPM_MAX_DOF + 1)];
        float sk[3 * (RPM_MAX_DOF + 1)], p[RPM_MAX_DOF];
        skeleton(rb, qn, trig, p64, sk);
        bool ok = false;
        float d = distance_underest(nm, rb, n, sk, near_cur, p, &ok);
        if (ok) {
            dn = d;
            for (int i = 0; i < L; ++i) pn[i] = p[i];
        } else {
            d = 0.f;
            dn = -1.f;
        }
        if (d < d_crit || status != kStAdvanced) break;
    }
    for (int k = 0; k < D; ++k) q_out[k] = qn[k];
    return status;
}

extern "C" void orc_box_aabb(const float *dim, const float *pos, const float *quat_xyzw, float *out);

// ---------------------------------------------------------- motion validity --
// MotionValidity::check (MotionValidity.cpp:30-53) with the boxes of 'movers'
// moving by Environment::moveStraight (Environment.cpp:220-233): before check
// k (1..N) every mover's position x decreases by delta_time * max_vel and its
// AABB is recomputed as fcl does for a box.  Check k tests
// interpolateEdge(q_prev, q_cur, dist * k / N, dist) (RealVectorSpace.cpp:75-88)
// against the moved scene.  Returns the validity; *checks = the checks made.
template <typename T>
bool motion_valid(const Num<T> &nm, const rpm_robot_desc &rb, int trig, Scene<T> sc, const float *q1, const float *q2,
                  const rpm_moving_box *movers, int n_movers, float max_iter_time, int N, int *checks) {
    const int D = rb.num_dofs;
    float ss = 0.f;   // getNorm in index order
    for (int i = 0; i < D; ++i) {
        const float df = q1[i] - q2[i];
        ss = ss + df * df;
    }
    const float dist = std::sqrt(ss);
    const float dt = max_iter_time / (float)N;
    std::vector<rpm_moving_box> mv(movers, movers + n_movers);
    for (int k = 1; k <= N; ++k) {
        for (rpm_moving_box &m : mv) {
            m.pos[0] = m.pos[0] - dt * m.max_vel;
            float box[6];
            orc_box_aabb(m.dim, m.pos, m.quat_xyzw, box);
            for (int c = 0; c < 6; ++c) sc.box[6 * (size_t)m.index + c] = (T)box[c];
        }
        const float step = dist * (float)k / (float)N;
        float q[RPM_MAX_DOF];
        if (dist > 0) {
            const float r = step / dist;
            for (int i = 0; i < D; ++i) q[i] = q1[i] + (q2[i] - q1[i]) * r;
        } else {
            for (int i = 0; i < D; ++i) q[i] = q2[i];
        }
        double p64[3 * (RPM_MAX_DOF + 1)];
        float p32[3 * (RPM_MAX_DOF + 1)];
        skeleton(rb, q, trig, p64, p32);
        T sk[3 * (RPM_MAX_DOF + 1)];
        for (int i = 0; i < 3 * (D + 1); ++i) sk[i] = sizeof(T) == 4 ? (T)p32[i] : (T)p64[i];
        if (!is_valid(nm, rb, sc, sk)) {
            *checks = k;
            return false;
        }
    }
    *checks = N;
    return true;
}

extern "C" {

int orc_version(void) { return 1; }

void orc_sincos(const double *x, int64_t n, int trig, double *s, double *c) {
    for (int64_t i = 0; i < n; ++i) fk_sincos(x[i], trig, &s[i], &c[i]);
}

// Skeleton points per configuration; prec 64 -> double FK points, 32 -> the
// reference's float skeleton widened to double.
int orc_skeleton(const rpm_robot_desc *rb, const float *q, int64_t C, int prec, int trig, double *out) {
    const int D = rb->num_dofs, P = 3 * (D + 1);
    for (int64_t c = 0; c < C; ++c) {
        double p64[3 * (RPM_MAX_DOF + 1)];
        float p32[3 * (RPM_MAX_DOF + 1)];
        skeleton(*rb, q + c * D, trig, p64, p32);
        for (int k = 0; k < P; ++k) out[c * P + k] = (prec == 32) ? (double)p32[k] : p64[k];
    }
    return 0;
}

// Batched isValid / computeDistance over C configurations.
int orc_check_configs(const rpm_robot_desc *rb, const float *aabb, const float *tol, const uint8_t *flags, int n,
                      const float *q, int64_t C, int prec, int trig, const rpm_params *params, uint8_t *valid,
                      double *dist, float *profile, int nthreads) {
    const int D = rb->num_dofs, L = D;
    Obstacles ob{aabb, tol, flags, n};
    double maxd = params ? params->max_distance : 1000.0;
    if (prec == 32) {
        Scene<float> sc(ob, maxd);
        Num<float> nm = num_of<float>(params);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_of(nthreads))
        for (int64_t c = 0; c < C; ++c) {
            double p64[3 * (RPM_MAX_DOF + 1)];
            float p32[3 * (RPM_MAX_DOF + 1)];
            skeleton(*rb, q + c * D, trig, p64, p32);
            config_one(nm, *rb, sc, p32, valid ? valid + c : nullptr, dist ? dist + c : nullptr,
                       profile ? profile + c * L : nullptr);
        }
    } else {
        Scene<double> sc(ob, maxd);
        Num<double> nm = num_of<double>(params);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads_of(nthreads))
        for (int64_t c = 0; c < C; ++c) {
            double p64[3 * (RPM_MAX_DOF + 1)];
            float p32[3 * (RPM_MAX_DOF + 1)];
            skeleton(*rb, q + c * D, trig, p64, p32);
            config_one(nm, *rb, sc, p64, valid ? valid + c : nullptr, dist ? dist + c : nullptr,
                       profile ? profile + c * L : nullptr);
        }
    }
    return 0;
}

// computeDistance with nearest points for a few configurations (single-state
// adapter path).  nearest is C x n x 6 x L floats; nearest_valid is C bytes.
int orc_distance_nearest(const rpm_robot_desc *rb, const float *aabb, const float *tol, const uint8_t *flags, int n,
                         const float *q, int64_t C, int prec, int trig, const rpm_params *params, double *dist,
                         float *profile, float *nearest, uint8_t *nearest_valid) {
    const int D = rb->num_dofs, L = D;
    Obstacles ob{aabb, tol, flags, n};
    double maxd = params ? params->max_distance : 1000.0;
    const size_t NS = (size_t)n * 6 * L;
    for (int64_t c = 0; c < C; ++c) {
        double p64[3 * (RPM_MAX_DOF + 1)];
        float p32[3 * (RPM_MAX_DOF + 1)];
        skeleton(*rb, q + c * D, trig, p64, p32);
        bool nv = false;
        if (prec == 32) {
            Scene<float> sc(ob, maxd);
            Num<float> nm = num_of<float>(params);
            std::vector<float> near(NS, 0.f);
            float prof[RPM_MAX_DOF];
            float d = compute_distance(nm, *rb, sc, p32, prof, near.data(), &nv);
            dist[c] = d;
            for (int i = 0; i < L; ++i) profile[c * L + i] = prof[i];
            for (size_t k = 0; k < NS; ++k) nearest[c * NS + k] = near[k];
        } else {
            Scene<double> sc(ob, maxd);
            Num<double> nm = num_of<double>(params);
            std::vector<double> near(NS, 0.0);
            double prof[RPM_MAX_DOF];
            double d = compute_distance(nm, *rb, sc, p64, prof, near.data(), &nv);
            dist[c] = d;
            for (int i = 0; i < L; ++i) profile[c * L + i] = (float)prof[i];
            for (size_t k = 0; k < NS; ++k) nearest[c * NS + k] = (float)near[k];
        }
        nearest_valid[c] = nv ? 1 : 0;
    }
    return 0;
}

int orc_distance_underest(const rpm_robot_desc *rb, int n, const float *q, int64_t C, int prec, int trig,
                          const rpm_params *params, const float *nearest, double *dist, float *profile,
                          uint8_t *complete) {
    const int D = rb->num_dofs, L = D;
    const size_t NS = (size_t)n * 6 * L;
    for (int64_t c = 0; c < C; ++c) {
        double p64[3 * (RPM_MAX_DOF + 1)];
        float p32[3 * (RPM_MAX_DOF + 1)];
        skeleton(*rb, q + c * D, trig, p64, p32);
        bool ok = false;
        if (prec == 32) {
            float prof[RPM_MAX_DOF];
            dist[c] = distance_underest(num_of<float>(params), *rb, n, p32, nearest + c * NS, prof, &ok);
            for (int i = 0; i < L; ++i) profile[c * L + i] = prof[i];
        } else {
            double prof[RPM_MAX_DOF];
            dist[c] = distance_underest(num_of<double>(params), *rb, n, p64, nearest + c * NS, prof, &ok);
            for (int i = 0; i < L; ++i) profile[c * L + i] = (float)prof[i];
        }
        complete[c] = ok ? 1 : 0;
    }
    return 0;
}

// RealVectorSpace::isValid(q1, q2) (RealVectorSpace.cpp:261-275).  With
// step > 0 the number of checks is n = max(1, ceil(dist/step)) (uneven edge
// discretisation); with step <= 0 it is num_checks (the reference's
// NUM_INTERPOLATION_VALIDITY_CHECKS).  checks_out[e] = checks evaluated in the
// reference order (q2 first, early exit) including the first invalid one.
int orc_check_edges(const rpm_robot_desc *rb, const float *aabb, const float *tol, const uint8_t *flags, int n,
                    const float *q1, const float *q2, int64_t E, float step, int num_checks, int prec, int trig,
                    const rpm_params *params, uint8_t *valid, int32_t *checks_out, int nthreads) {
    const int D = rb->num_dofs;
    Obstacles ob{aabb, tol, flags, n};
    double maxd = params ? params->max_distance : 1000.0;
    Scene<float> sc32(ob, maxd);
    Scene<double> sc64(ob, maxd);
    Num<float> nm32 = num_of<float>(params);
    Num<double> nm64 = num_of<double>(params);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads_of(nthreads))
    for (int64_t e = 0; e < E; ++e) {
        const float *a = q1 + e * D, *b = q2 + e * D;
        // getNorm: (q1 - q2).norm(), summed in index order
        float ss = 0.f;
        for (int k = 0; k < D; ++k) { float df = a[k] - b[k]; ss = ss + df * df; }
        float dist = std::sqrt(ss);
        int64_t N = num_checks;
        if (step > 0) { N = (int64_t)std::ceil(dist / step); if (N < 1) N = 1; }
        bool ok = true;
        int32_t cnt = 0;
        for (float k = (float)N; k >= 1; k--) {
            float stp = k / (float)N * dist;
            float qk[RPM_MAX_DOF];
            if (dist > 0) {
                float ratio = stp / dist;
                for (int i = 0; i < D; ++i) qk[i] = a[i] + (b[i] - a[i]) * ratio;
            } else
                for (int i = 0; i < D; ++i) qk[i] = b[i];
            double p64[3 * (RPM_MAX_DOF + 1)];
            float p32[3 * (RPM_MAX_DOF + 1)];
            skeleton(*rb, qk, trig, p64, p32);
            ++cnt;
            bool v = (prec == 32) ? is_valid(nm32, *rb, sc32, p32) : is_valid(nm64, *rb, sc64, p64);
            if (!v) { ok = false; break; }
        }
        valid[e] = ok ? 1 : 0;
        if (checks_out) checks_out[e] = cnt;
    }
    return 0;
}

// Single primitives, for pinning against the reference's own source.
int orc_prim_collision(const float *A, const float *B, float r, const float *obs, int prec, const rpm_params *params) {
    if (prec == 32) { Num<float> nm = num_of<float>(params); return coll_box(nm, A, B, r, obs) ? 1 : 0; }
    Num<double> nm = num_of<double>(params);
    double a[3] = {A[0], A[1], A[2]}, b[3] = {B[0], B[1], B[2]}, o[6];
    for (int k = 0; k < 6; ++k) o[k] = obs[k];
    return coll_box(nm, a, b, (double)r, o) ? 1 : 0;
}

double orc_prim_distance(const float *A, const float *B, float r, const float *obs, int prec, const rpm_params *params,
                         float *pts_out, int *has_pts) {
    if (prec == 32) {
        Num<float> nm = num_of<float>(params);
        CapsuleBox<float> cb(nm, A, B, r, obs);
        cb.compute();
        if (pts_out) for (int k = 0; k < 6; ++k) pts_out[k] = cb.pts[k];
        if (has_pts) *has_pts = cb.has_pts;
        return cb.d_c;
    }
    Num<double> nm = num_of<double>(params);
    double a[3] = {A[0], A[1], A[2]}, b[3] = {B[0], B[1], B[2]}, o[6];
    for (int k = 0; k < 6; ++k) o[k] = obs[k];
    CapsuleBox<double> cb(nm, a, b, (double)r, o);
    cb.compute();
    if (pts_out) for (int k = 0; k < 6; ++k) pts_out[k] = (float)cb.pts[k];
    if (has_pts) *has_pts = cb.has_pts;
    return cb.d_c;
}

// Number of evaluations on this thread that reached the undefined branch of
// getLineSegments since the last call (then reset).
int64_t orc_undefined_hits(void) {
    const int64_t n = g_undefined_hits;
    g_undefined_hits = 0;
    return n;
}

double orc_prim_segseg(const float *A, const float *B, const float *C, const float *D, int prec, const rpm_params *params) {
    bool hp;
    if (prec == 32) { Num<float> nm = num_of<float>(params); float pts[6]; return seg_seg(nm, A, B, C, D, pts, &hp); }
    Num<double> nm = num_of<double>(params);
    double a[3] = {A[0], A[1], A[2]}, b[3] = {B[0], B[1], B[2]}, c[3] = {C[0], C[1], C[2]}, d[3] = {D[0], D[1], D[2]}, pts[6];
    return seg_seg(nm, a, b, c, d, pts, &hp);
}

// fcl 0.7 world AABB of a box: identity rotation -> translate(local AABB, pos)
// with local AABB = -/+ 0.5*dim; otherwise the cube pos -/+ |dim/2|.
void orc_box_aabb(const float *dim, const float *pos, const float *quat_xyzw, float *out) {
    float x = quat_xyzw[0], y = quat_xyzw[1], z = quat_xyzw[2], w = quat_xyzw[3];
    bool ident = (x == 0.f && y == 0.f && z == 0.f && (w == 1.f || w == -1.f));
    float h[3] = {0.5f * dim[0], 0.5f * dim[1], 0.5f * dim[2]};
    if (ident) {
        for (int k = 0; k < 3; ++k) { out[k] = (-h[k]) + pos[k]; out[3 + k] = h[k] + pos[k]; }
    } else {
        float rad = std::sqrt(h[0] * h[0] + (h[1] * h[1] + h[2] * h[2]));
        for (int k = 0; k < 3; ++k) { out[k] = pos[k] - rad; out[3 + k] = pos[k] + rad; }
    }
}

// Enclosing radii per configuration: out is C x D x (D + 1) floats.
int orc_enclosing_radii(const rpm_robot_desc *rb, const float *q, int64_t C, int trig, float *out) {
    const int D = rb->num_dofs;
    for (int64_t c = 0; c < C; ++c) {
        double p64[3 * (RPM_MAX_DOF + 1)];
        float p32[3 * (RPM_MAX_DOF + 1)];
        skeleton(*rb, q + c * D, trig, p64, p32);
        enclosing_radii(*rb, p32, out + c * D * (D + 1));
    }
    return 0;
}

// extendSpine per row: q, qe C x D; dist C; profile C x L.
int orc_extend_spines(const rpm_robot_desc *rb, const float *q, const float *qe, const float *dist, const float *profile,
                      int64_t C, int num_iter, int expanded, int trig, float *q_new, int32_t *status) {
    const int D = rb->num_dofs;
    for (int64_t c = 0; c < C; ++c)
        status[c] = extend_spine(*rb, trig, q + c * D, dist[c], profile + c * D, qe + c * D, num_iter, expanded != 0,
                                 q_new + c * D);
    return 0;
}

// computeReachedState for a horizon (H x D) from q_cur, whose computeDistance
// with nearest points runs here in the reference's float numerics.
int orc_reached_states(const rpm_robot_desc *rb, const float *aabb, const float *tol, const uint8_t *flags, int n,
                       const float *q_cur, const float *qe, int64_t H, int num_layers, int num_iter, int expanded,
                       float d_crit, int trig, const rpm_params *params, float *q_out, int32_t *status) {
    const int D = rb->num_dofs, L = D;
    const size_t NS = (size_t)n * 6 * L;
    std::vector<float> near(NS > 0 ? NS : 1, 0.f);
    float prof[RPM_MAX_DOF];
    double d = 0.0;
    uint8_t nv = 0;
    orc_distance_nearest(rb, aabb, tol, flags, n, q_cur, 1, 32, trig, params, &d, prof, near.data(), &nv);
    const Num<float> nm = num_of<float>(params);
    for (int64_t h = 0; h < H; ++h)
        status[h] = reached_state(nm, *rb, trig, n, q_cur, (float)d, prof, near.data(), qe + h * D, num_layers,
                                  num_iter, expanded != 0, d_crit, q_out + h * D);
    return 0;
}

// MotionValidity::check per motion (q_prev, q_cur: M x D), every motion from
// the same obstacle state.
int orc_motion_validity(const rpm_robot_desc *rb, const float *aabb, const float *tol, const uint8_t *flags, int n,
                        const float *q_prev, const float *q_cur, int64_t M, const rpm_moving_box *movers, int n_movers,
                        float max_iter_time, int N, int prec, int trig, const rpm_params *params, uint8_t *valid,
                        int32_t *checks) {
    const int D = rb->num_dofs;
    Obstacles ob{aabb, tol, flags, n};
    const double maxd = params ? params->max_distance : 1000.0;
    for (int64_t m = 0; m < M; ++m) {
        int k = 0;
        bool v;
        if (prec == 32) v = motion_valid(num_of<float>(params), *rb, trig, Scene<float>(ob, maxd), q_prev + m * D,
                                         q_cur + m * D, movers, n_movers, max_iter_time, N, &k);
        else v = motion_valid(num_of<double>(params), *rb, trig, Scene<double>(ob, maxd), q_prev + m * D,
                              q_cur + m * D, movers, n_movers, max_iter_time, N, &k);
        valid[m] = v ? 1 : 0;
        checks[m] = k;
    }
    return 0;
}

}  // extern "C"
