// rpm_tree.cuh -- the reference's capsule/box decision trees as device code.
//
// The two trees are written once, templated on the scalar T and on a decision
// policy P:
//   ExactPol  : every decision is a plain bool; used by the FP64 form and the
//               reference-exact FP32 form (which must reproduce the CPU bits).
//   RobustPol : every decision also carries a margin -- the distance, in
//               metres divided by the error amplification of the compared
//               quantities, from the decision boundary.  Conjunctions and
//               disjunctions combine margins as a robustness degree (a true
//               AND is as robust as its weakest term, a false AND as its most
//               decisive false term, dually for OR).  RPM_TAKE(pol, ) records the
//               margin of each decision actually taken.  If the smallest
//               recorded margin is at least kBand, the same tree evaluated in
//               FP64 on the FP64 skeleton takes the same branches.
//
// Reference (all in src/state_spaces/real_vector_space/CollisionAndDistance.cpp):
//   coll_box      collisionCapsuleToBox        :4-42
//   coll_rect     collisionCapsuleToRectangle  :46-111
//   check_cases   checkCases                   :113-148
//   seg_seg       distanceLineSegToLineSeg     :217-320   (value only)
//   seg_point     distanceLineSegToPoint       :323-342   (value only)
//   capsule_box   CapsuleToBox::compute and helpers :409-755 (value only)
// Scalar evaluation order follows the reference compiled without contraction:
// 3-vector dot products sum as x0 + (x1 + x2) (Eigen's reduction order).
#pragma once
#include <cfloat>
#include <cstdint>

#include "rpm_dev.cuh"

#define RPM_TAKE(pol, ...) (pol).take((__VA_ARGS__), __LINE__)
#define RPM_NOTE(pol, ...) (pol).note((__VA_ARGS__), __LINE__)

namespace rpm {

#if defined(RPM_MARGIN_DEBUG)
inline int g_dbg_print = 10;
#endif

struct RB {
    bool v;
    float m;
};

struct ExactPol {
    static constexpr bool robust = false;
    static constexpr float m = FLT_MAX;   // every decision is exact
    typedef bool C;
    template <typename T> RPM_HD static bool lt(T a, T b, float = 1.f) { return a < b; }
    template <typename T> RPM_HD static bool gt(T a, T b, float = 1.f) { return a > b; }
    template <typename T> RPM_HD static bool le(T a, T b, float = 1.f) { return a <= b; }
    template <typename T> RPM_HD static bool ge(T a, T b, float = 1.f) { return a >= b; }
    RPM_HD static bool all(bool a, bool b) { return a && b; }
    RPM_HD static bool all(bool a, bool b, bool c) { return a && b && c; }
    RPM_HD static bool all(bool a, bool b, bool c, bool d) { return a && b && c && d; }
    RPM_HD static bool all6(bool a, bool b, bool c, bool d, bool e, bool f) {
        return a && b && c && d && e && f;
    }
    RPM_HD static bool any(bool a, bool b) { return a || b; }
    RPM_HD static bool settled(bool a) { return a; }
    RPM_HD static bool any6(bool a, bool b, bool c, bool d, bool e, bool f) {
        return a || b || c || d || e || f;
    }
    // t > 0 && t < 1 where t = num / den
    template <typename T> RPM_HD static bool t_inside(T t, T, T) { return t > T(0) && t < T(1); }
    template <typename T> RPM_HD static bool nonzero(T x) { return x != T(0); }
    RPM_HD bool take(bool c, int = 0) { return c; }
    RPM_HD void note(float, int = 0) {}
};

struct RobustPol {
    static constexpr bool robust = true;
    typedef RB C;
    float m = FLT_MAX;
    template <typename T> RPM_HD static RB lt(T a, T b, float ia = 1.f) {
        return RB{a < b, fabsf((float)(a - b)) * ia};
    }
    template <typename T> RPM_HD static RB gt(T a, T b, float ia = 1.f) {
        return RB{a > b, fabsf((float)(a - b)) * ia};
    }
    template <typename T> RPM_HD static RB le(T a, T b, float ia = 1.f) {
        return RB{a <= b, fabsf((float)(a - b)) * ia};
    }
    template <typename T> RPM_HD static RB ge(T a, T b, float ia = 1.f) {
        return RB{a >= b, fabsf((float)(a - b)) * ia};
    }
    RPM_HD static RB all(RB a, RB b) {
        bool v = a.v && b.v;
        float m = v ? fminf(a.m, b.m) : ((!a.v && !b.v) ? fmaxf(a.m, b.m) : (!a.v ? a.m : b.m));
        return RB{v, m};
    }
    RPM_HD static RB all(RB a, RB b, RB c) { return all(all(a, b), c); }
    RPM_HD static RB all(RB a, RB b, RB c, RB d) { return all(all(a, b), all(c, d)); }
    RPM_HD static RB all6(RB a, RB b, RB c, RB d, RB e, RB f) {
        return all(all(a, b, c), all(d, e, f));
    }
    // a decision that follows from decisions already recorded
    RPM_HD static RB settled(bool a) { return RB{a, FLT_MAX}; }
    RPM_HD static RB any(RB a, RB b) {
        bool v = a.v || b.v;
        float m = v ? ((a.v && b.v) ? fmaxf(a.m, b.m) : (a.v ? a.m : b.m)) : fminf(a.m, b.m);
        return RB{v, m};
    }
    RPM_HD static RB any6(RB a, RB b, RB c, RB d, RB e, RB f) {
        return any(any(any(a, b), any(c, d)), any(e, f));
    }
    // t = num / den lies in (0, 1) exactly when A and B are strictly on opposite
    // sides of the face plane: num = obs - A_c, den - num = B_c - obs (metres).
    template <typename T> RPM_HD static RB t_inside(T t, T num, T den) {
        if (den == T(0)) return RB{false, FLT_MAX};   // t = MAX_DISTANCE
        return RB{t > T(0) && t < T(1), fminf(fabsf((float)num), fabsf((float)(den - num)))};
    }
    // The only use of 'den != 0' is to choose t = MAX_DISTANCE, which t_inside
    // already decides robustly; an exact zero here is structural (e.g. the z
    // coordinates of a planar chain are zero in FP32 and FP64 alike).
    template <typename T> RPM_HD static RB nonzero(T x) { return RB{x != T(0), FLT_MAX}; }
#ifdef RPM_MARGIN_DEBUG
    int site = 0;
    RPM_HD bool take(RB c, int line = 0) {
        if (c.m < kDecide && m >= kDecide) site = line;
        m = fminf(m, c.m);
        return c.v;
    }
    RPM_HD void note(float mm, int line = 0) {
        if (mm < kDecide && m >= kDecide) site = line;
        m = fminf(m, mm);
    }
#else
    RPM_HD bool take(RB c, int = 0) {
        m = fminf(m, c.m);
        return c.v;
    }
    RPM_HD void note(float mm, int = 0) { m = fminf(m, mm); }
#endif
};

template <typename T> struct Num {
    T eq, maxd;
};

// A value with the reciprocal of its error amplification (1 = as accurate as
// a skeleton coordinate).  ExactPol ignores ia.
template <typename T> struct Val {
    T v;
    float ia;
};

template <typename T> RPM_HD T dot3(const T *a, const T *b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
template <typename T> RPM_HD T sqrtT(T x);
template <> RPM_HD float sqrtT<float>(float x) { return sqrtf(x); }
template <> RPM_HD double sqrtT<double>(double x) { return sqrt(x); }
template <typename T> RPM_HD T norm3(const T *a) { return sqrtT(dot3(a, a)); }
template <typename T> RPM_HD T smin(T a, T b) { return (b < a) ? b : a; }   // std::min
template <typename T> RPM_HD void sub3(const T *a, const T *b, T *o) {
    o[0] = a[0] - b[0]; o[1] = a[1] - b[1]; o[2] = a[2] - b[2];
}
template <typename T> RPM_HD T absT(T x) { return x < T(0) ? -x : x; }

// get3DPoint (:150-155): insert 'value' at index 'coord'
template <typename T> RPM_HD void pt3(T u, T v, T value, int coord, T *o) {
    if (coord == 0) { o[0] = value; o[1] = u; o[2] = v; }
    else if (coord == 1) { o[0] = u; o[1] = value; o[2] = v; }
    else { o[0] = u; o[1] = v; o[2] = value; }
}

// box corner: bit0 selects x max, bit1 y max, bit2 z max
template <typename T> RPM_HD void corner(const T *o, int c, T *p) {
    p[0] = o[(c & 1) ? 3 : 0];
    p[1] = o[(c & 2) ? 4 : 1];
    p[2] = o[(c & 4) ? 5 : 2];
}

// Record, for a robust evaluation, how close a segment distance came to the
// EQUALITY_THRESHOLD snap (a discontinuity of the reference's distance).
template <typename T, typename P> RPM_HD void note_snap(P &pol, T d, T eq) {
    if (P::robust) RPM_NOTE(pol, fabsf((float)(d - eq)));
}

// distanceLineSegToLineSeg (:217-320), value only.
template <typename T, typename P>
__host__ __device__ Val<T> seg_seg(P &pol, const Num<T> &nm, const T *A, const T *B, const T *C, const T *D) {
    T BA[3], DC[3], CD[3], AC[3], AB[3];
    sub3(B, A, BA); sub3(D, C, DC); sub3(C, D, CD); sub3(A, C, AC); sub3(A, B, AB);
    T alpha1 = dot3(BA, BA);
    T alpha2 = dot3(BA, DC);
    T beta1 = dot3(CD, BA);
    T beta2 = dot3(CD, DC);
    T gamma1 = dot3(AC, AB);
    T gamma2 = dot3(AC, CD);
    T den = alpha1 * beta2 - alpha2 * beta1;
    T s = (alpha1 * gamma2 - alpha2 * gamma1) / den;
    T t = (gamma1 - beta1 * s) / alpha1;
    T alpha3 = dot3(CD, CD);
    if (P::robust) {
        // The value is continuous across the interior/boundary choice except
        // through the EQUALITY_THRESHOLD snap; near the snap the choice itself
        // must be settled (t, s measured in metres along each segment).
        T dref;
        {
            T df[3];
            for (int i = 0; i < 3; ++i) df[i] = (C[i] + s * DC[i]) - (A[i] + t * BA[i]);
            dref = norm3(df);
        }
        const float lu = sqrtf((float)alpha1), lv = sqrtf((float)alpha3);
        if (!(dref >= nm.eq + T(kDecide)) || !(dref == dref)) {
            auto inside = P::all(P::gt(t * lu, T(0)), P::lt(t * lu, (T)lu), P::gt(s * lv, T(0)), P::lt(s * lv, (T)lv));
            RPM_TAKE(pol, inside);
        }
    }
    if (t > T(0) && t < T(1) && s > T(0) && s < T(1)) {
        T df[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) df[i] = (C[i] + s * DC[i]) - (A[i] + t * BA[i]);
        T d = norm3(df);
        note_snap(pol, d, nm.eq);
        if (d < nm.eq) return Val<T>{T(0), 1.f};
        return Val<T>{d, 1.f};
    }
    T opt0 = dot3(AC, AB) / alpha1;
    T AD[3], BC[3];
    sub3(A, D, AD); sub3(B, C, BC);
    T opt1 = dot3(AD, AB) / alpha1;
    T opt2 = dot3(AC, DC) / alpha3;
    T opt3 = dot3(BC, DC) / alpha3;
    T d = nm.maxd;
    T df[3], dt;
    // i = 0: C against AB
    if (opt0 < T(0)) sub3(C, A, df);
    else if (opt0 > T(1)) sub3(C, B, df);
    else for (int k = 0; k < 3; ++k) df[k] = C[k] - (A[k] + opt0 * BA[k]);
    dt = norm3(df);
    if (dt < d) d = dt;
    // i = 1: D against AB
    if (opt1 < T(0)) sub3(D, A, df);
    else if (opt1 > T(1)) sub3(D, B, df);
    else for (int k = 0; k < 3; ++k) df[k] = D[k] - (A[k] + opt1 * BA[k]);
    dt = norm3(df);
    if (dt < d) d = dt;
    // i = 2: A against CD
    if (opt2 < T(0)) sub3(C, A, df);
    else if (opt2 > T(1)) sub3(D, A, df);
    else for (int k = 0; k < 3; ++k) df[k] = (C[k] + opt2 * DC[k]) - A[k];
    dt = norm3(df);
    if (dt < d) d = dt;
    // i = 3: B against CD
    if (opt3 < T(0)) sub3(C, B, df);
    else if (opt3 > T(1)) sub3(D, B, df);
    else for (int k = 0; k < 3; ++k) df[k] = (C[k] + opt3 * DC[k]) - B[k];
    dt = norm3(df);
    if (dt < d) d = dt;
    return Val<T>{d, 1.f};
}

// distanceLineSegToPoint (:323-342), value only.
template <typename T, typename P>
RPM_HD T seg_point(P &pol, const Num<T> &nm, const T *A, const T *B, const T *C) {
    T BA[3], CA[3], df[3];
    sub3(B, A, BA); sub3(C, A, CA);
    T t_opt = dot3(CA, BA) / dot3(BA, BA);
    if (t_opt < T(0)) sub3(C, A, df);
    else if (t_opt > T(1)) sub3(C, B, df);
    else for (int k = 0; k < 3; ++k) df[k] = C[k] - (A[k] + t_opt * BA[k]);
    T d = norm3(df);
    note_snap(pol, d, nm.eq);
    if (d < nm.eq) return T(0);
    return d;
}

// Selects in place of dynamic indexing (dynamic indices into register arrays
// would spill them to local memory).
template <typename T> RPM_HD T sel3(const T *v, int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); }
template <typename T> RPM_HD T sel6(const T *v, int k) {
    return k < 3 ? (k == 0 ? v[0] : (k == 1 ? v[1] : v[2])) : (k == 3 ? v[3] : (k == 4 ? v[4] : v[5]));
}
RPM_HD int gray2(int q) { return q ^ (q >> 1); }   // 0, 1, 3, 2: a loop around a square

// checkCases (:113-148): at most two rectangle edges, the second only while
// the first distance is positive.
template <typename T, typename P>
RPM_HD Val<T> check_cases(P &pol, const Num<T> &nm, const T *A, const T *B, const T *rec, T pu, T pv, T obs_coord,
                          int coord) {
    T d[2] = {nm.maxd, nm.maxd};
#pragma unroll 1
    for (int k = 0; k < 2; ++k) {
        // k = 0: edge u = rec0 or u = rec2 (v from rec1 to rec3); k = 1: edge v = rec1 or v = rec3
        int side = -1;
        if (k == 0) {
            if (RPM_TAKE(pol, P::lt(pu, rec[0]))) side = 0;
            else if (RPM_TAKE(pol, P::gt(pu, rec[2]))) side = 1;
        } else {
            // d_c1 is MAX_DISTANCE, an exact 0 from the snap, or a distance of at
            // least EQUALITY_THRESHOLD (the snap margin is recorded in seg_seg)
            auto d1pos = P::settled(d[0] > T(0));
            if (RPM_TAKE(pol, P::all(d1pos, P::lt(pv, rec[1])))) side = 0;
            else if (RPM_TAKE(pol, P::all(d1pos, P::gt(pv, rec[3])))) side = 1;
        }
        if (side < 0) continue;
        T C[3], D[3];
        if (k == 0) {
            const T u = side ? rec[2] : rec[0];
            pt3(u, rec[1], obs_coord, coord, C);
            pt3(u, rec[3], obs_coord, coord, D);
        } else {
            const T v = side ? rec[3] : rec[1];
            pt3(rec[0], v, obs_coord, coord, C);
            pt3(rec[2], v, obs_coord, coord, D);
        }
        d[k] = seg_seg(pol, nm, A, B, C, D).v;
    }
    return Val<T>{smin(d[0], d[1]), 1.f};
}

// collisionCapsuleToRectangle (:46-111).  'face' in 0..5 = x_min..z_max.
template <typename T, typename P>
RPM_HD bool coll_rect(P &pol, const Num<T> &nm, const T *A, const T *B, T radius, const T *obs, int face) {
    const int c = face > 2 ? face - 3 : face;
    const int a = (c == 0) ? 1 : 0, b = (c == 2) ? 1 : 2;
    const T obs_coord = sel6(obs, face);
    const T rec[4] = {sel6(obs, a), sel6(obs, b), sel6(obs, 3 + a), sel6(obs, 3 + b)};
    const T Ac = sel3(A, c), Bc = sel3(B, c);
    const T Au = sel3(A, a), Av = sel3(A, b), Bu = sel3(B, a), Bv = sel3(B, b);
    const T num = obs_coord - Ac, den = Bc - Ac;
    T t = RPM_TAKE(pol, P::nonzero(den)) ? num / den : nm.maxd;
    const T Mu = Au + t * (Bu - Au), Mv = Av + t * (Bv - Av);
    // |A - A_proj| and |B - B_proj|: the other two coordinates cancel exactly
    const T xa = Ac - obs_coord, xb = Bc - obs_coord;
    const T dA = sqrtT(xa * xa), dB = sqrtT(xb * xb);
    if (RPM_TAKE(pol, P::t_inside(t, num, den))) {
        float iaM = 1.f;
        if (P::robust) {
            float spread = fmaxf(fabsf((float)(Bu - Au)), fabsf((float)(Bv - Av)));
            float ad = fabsf((float)den);
            iaM = ad / (ad + 4.f * spread);
        }
        auto big = P::all(P::gt(Mu, rec[0] - radius, iaM), P::lt(Mu, rec[2] + radius, iaM),
                          P::gt(Mv, rec[1] - radius, iaM), P::lt(Mv, rec[3] + radius, iaM));
        if (RPM_TAKE(pol, big)) {
            const float iaN = iaM * 0.7f;
            auto c1 = P::all(P::gt(Mu, rec[0] - radius, iaM), P::lt(Mu, rec[2] + radius, iaM), P::gt(Mv, rec[1], iaM),
                             P::lt(Mv, rec[3], iaM));
            auto c2 = P::all(P::gt(Mv, rec[1] - radius, iaM), P::lt(Mv, rec[3] + radius, iaM), P::gt(Mu, rec[0], iaM),
                             P::lt(Mu, rec[2], iaM));
            // the corner tests of :69-72 use rec(1)/rec(2) as written in the reference
            T e0 = Mu - rec[0], e1 = Mv - rec[2], e2 = Mv - rec[3], e3 = Mu - rec[1];
            auto c3 = P::all(P::lt(Mu, rec[0], iaM), P::lt(Mv, rec[2], iaM), P::lt(sqrtT(e0 * e0 + e1 * e1), radius, iaN));
            auto c4 = P::all(P::lt(Mu, rec[0], iaM), P::gt(Mv, rec[3], iaM), P::lt(sqrtT(e0 * e0 + e2 * e2), radius, iaN));
            auto c5 = P::all(P::gt(Mu, rec[1], iaM), P::lt(Mv, rec[2], iaM), P::lt(sqrtT(e3 * e3 + e1 * e1), radius, iaN));
            auto c6 = P::all(P::gt(Mu, rec[1], iaM), P::gt(Mv, rec[3], iaM), P::lt(sqrtT(e3 * e3 + e2 * e2), radius, iaN));
            if (RPM_TAKE(pol, P::any6(c1, c2, c3, c4, c5, c6))) return true;
        }
    } else if (RPM_TAKE(pol, P::gt(smin(dA, dB), radius)))
        return false;

    if (radius > T(0)) {
        auto a_in = P::all(P::gt(Au, rec[0]), P::lt(Au, rec[2]), P::gt(Av, rec[1]), P::lt(Av, rec[3]));
        auto b_in = P::all(P::gt(Bu, rec[0]), P::lt(Bu, rec[2]), P::gt(Bv, rec[1]), P::lt(Bv, rec[3]));
        const bool ain = RPM_TAKE(pol, a_in);
        const bool bin = RPM_TAKE(pol, b_in);
        if (ain && bin) {                                                    // both projections
            if (RPM_TAKE(pol, P::lt(smin(dA, dB), radius))) return true;
        } else {
            // only A: min(checkCases(B_rec), |A - A_proj|); only B: min(checkCases(A_rec),
            // |B - B_proj|); neither: checkCases(A_rec), then checkCases(B_rec)
            const int n = (ain || bin) ? 1 : 2;
#pragma unroll 1
            for (int k = 0; k < n; ++k) {
                const bool use_b = ain || k == 1;
                const T pu = use_b ? Bu : Au, pv = use_b ? Bv : Av;
                Val<T> cc = check_cases(pol, nm, A, B, rec, pu, pv, obs_coord, c);
                const T v = ain ? smin(cc.v, dA) : (bin ? smin(cc.v, dB) : cc.v);
                if (RPM_TAKE(pol, P::lt(v, radius, cc.ia))) return true;
            }
        }
    }
    return false;
}
// One out-of-line instance of coll_rect per (T, policy): both trees call it,
// so sharing it halves the code the instruction cache has to hold.  The
// policy state travels by value (decision, smallest margin).
template <typename T, typename P>
__host__ __device__ __noinline__ RB coll_rect_call(const Num<T> nm, const T *A, const T *B, T radius, const T *obs,
                                                   int face) {
    P pol;
    const bool v = coll_rect(pol, nm, A, B, radius, obs, face);
    return RB{v, pol.m};
}

// collisionCapsuleToBox (:4-42).  r_new = radius * sqrt(3) / 3 comes
// precomputed per link with the reference's rounding.  The face tests of
// :19-40 run as one loop over the axes (x, then y, then z), stopping at the
// first collision.  FLAT inlines the rectangle test: for a kernel that runs
// this tree alone, a nested out-of-line call costs more in saved registers
// than the shared copy saves in instruction cache.
template <typename T, typename P, bool FLAT = false>
RPM_HD bool coll_box(P &pol, const Num<T> &nm, const T *A, const T *B, T radius, T r_new, const T *o) {
    auto inA = P::all6(P::gt(A[0], o[0] - r_new), P::gt(A[1], o[1] - r_new), P::gt(A[2], o[2] - r_new),
                       P::lt(A[0], o[3] + r_new), P::lt(A[1], o[4] + r_new), P::lt(A[2], o[5] + r_new));
    auto inB = P::all6(P::gt(B[0], o[0] - r_new), P::gt(B[1], o[1] - r_new), P::gt(B[2], o[2] - r_new),
                       P::lt(B[0], o[3] + r_new), P::lt(B[1], o[4] + r_new), P::lt(B[2], o[5] + r_new));
    if (RPM_TAKE(pol, P::any(inA, inB))) return true;
    auto slab = P::any6(P::all(P::lt(A[0], o[0] - radius), P::lt(B[0], o[0] - radius)),
                        P::all(P::gt(A[0], o[3] + radius), P::gt(B[0], o[3] + radius)),
                        P::all(P::lt(A[1], o[1] - radius), P::lt(B[1], o[1] - radius)),
                        P::all(P::gt(A[1], o[4] + radius), P::gt(B[1], o[4] + radius)),
                        P::all(P::lt(A[2], o[2] - radius), P::lt(B[2], o[2] - radius)),
                        P::all(P::gt(A[2], o[5] + radius), P::gt(B[2], o[5] + radius)));
    if (RPM_TAKE(pol, slab)) return false;
#pragma unroll 1
    for (int ax = 0; ax < 3; ++ax) {
        const T a = sel3(A, ax);
        int face = -1;
        if (RPM_TAKE(pol, P::lt(a, sel6(o, ax)))) face = ax;
        else if (RPM_TAKE(pol, P::gt(a, sel6(o, ax + 3)))) face = ax + 3;
        if (face >= 0) {
            if constexpr (FLAT) {
                if (coll_rect(pol, nm, A, B, radius, o, face)) return true;
            } else {
                const RB rr = coll_rect_call<T, P>(nm, A, B, radius, o, face);
                RPM_NOTE(pol, rr.m);
                if (rr.v) return true;
            }
        }
    }
    return false;
}

// Edge sources of CapsuleToBox's distance phase, all as box-corner pairs
// (corner bit 0 = x max, bit 1 = y max, bit 2 = z max).
enum EdgeKind { kEdgesNone = 0, kEdgesList = 1, kEdgesFaceLoop = 2, kEdgesAll12 = 3 };

// The k-th edge of a source.  List: up to 4 packed (c0 | c1 << 3) entries.
// Face loop (checkOtherCases, one axis outside): the face's corners in the
// reference's order (u, v) = (0,0), (1,0), (1,1), (0,1).  All 12 (:747-750):
// bottom loop, top loop, then the four vertical edges.
RPM_HD void edge_of(int kind, uint32_t list, int base, int u, int v, int k, int &c0, int &c1) {
    if (kind == kEdgesList) {
        const uint32_t e = (list >> (6 * k)) & 63u;
        c0 = (int)(e & 7u);
        c1 = (int)(e >> 3);
    } else if (kind == kEdgesFaceLoop) {
        const int g0 = gray2(k), g1 = gray2((k + 1) & 3);
        c0 = base | ((g0 & 1) << u) | ((g0 >> 1) << v);
        c1 = base | ((g1 & 1) << u) | ((g1 >> 1) << v);
    } else {
        if (k < 8) {
            const int b = k & 4, kk = k & 3;
            c0 = b | gray2(kk);
            c1 = b | gray2((kk + 1) & 3);
        } else {
            c0 = gray2(k - 8);
            c1 = c0 | 4;
        }
    }
}

// CapsuleToBox::compute (:409-448) with projectionLineSegOnSide (:450-474),
// checkEdges/getLineSegments (:476-574), distanceToMoreLineSegments (:576-595)
// and checkOtherCases (:597-755).  Returns d_c after the radius is subtracted
// (or 0 when an endpoint is inside the box).
template <typename T, typename P>
RPM_HD Val<T> capsule_box(P &pol, const Num<T> &nm, const T *A, const T *B, T radius, const T *o) {
    // ---- projections of A and B on the six faces
    unsigned projA = 0u, projB = 0u;
    T distA = nm.maxd, distB = nm.maxd;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const int u = (c == 0) ? 1 : 0, v = (c == 2) ? 1 : 2;
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const T *X = i ? B : A;
            auto inr = P::all(P::ge(X[u], o[u]), P::le(X[u], o[3 + u]), P::ge(X[v], o[v]), P::le(X[v], o[3 + v]));
            if (RPM_TAKE(pol, inr)) {
                if (RPM_TAKE(pol, P::all(P::gt(X[c], o[c]), P::lt(X[c], o[3 + c])))) return Val<T>{T(0), 1.f};
                unsigned &pj = i ? projB : projA;
                T &dj = i ? distB : distA;
                if (RPM_TAKE(pol, P::le(X[c], o[c]))) { pj |= 1u << c; dj = o[c] - X[c]; }
                else if (RPM_TAKE(pol, P::ge(X[c], o[3 + c]))) { pj |= 1u << (3 + c); dj = X[c] - o[3 + c]; }
            }
        }
    }
    // ---- what to evaluate
    T d = nm.maxd;
    int rect_face = -1;      // 0..5: checkEdges' rectangle test; 6: all six faces (checkOtherCases)
    int kind = kEdgesNone, ne = 0, base = 0, fu = 0, fv = 0, point = -1;
    bool direct = false;     // a single edge whose distance replaces d_c (tie(...) in checkOtherCases)
    int ip = 0, ce_face = -1;
    if (projA | projB) {
        ip = RPM_TAKE(pol, P::lt(distA, distB)) ? 0 : 1;
        d = (distB < distA) ? distB : distA;
        if ((projA & projB) == 0u) {   // num_proj == 1: checkEdges with the other point
            const unsigned pm = ip ? projB : projA;
            ce_face = (pm & 1u) ? 0 : (pm & 8u) ? 3 : (pm & 2u) ? 1 : (pm & 16u) ? 4 : (pm & 4u) ? 2 : (pm & 32u) ? 5 : -1;
            rect_face = ce_face;
        }
    } else {
        int rg[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (RPM_TAKE(pol, P::all(P::lt(A[c], o[c]), P::lt(B[c], o[c])))) rg[c] = 0;
            else if (RPM_TAKE(pol, P::all(P::gt(A[c], o[3 + c]), P::gt(B[c], o[3 + c])))) rg[c] = 2;
            else rg[c] = 1;
        }
        const int mids = (rg[0] == 1) + (rg[1] == 1) + (rg[2] == 1);
        base = (rg[0] == 2 ? 1 : 0) | (rg[1] == 2 ? 2 : 0) | (rg[2] == 2 ? 4 : 0);
        if (mids == 0) {
            point = base;
        } else if (mids == 1) {
            const int k = (rg[0] == 1) ? 0 : (rg[1] == 1 ? 1 : 2);
            kind = kEdgesList; ne = 1; direct = true;
            const uint32_t c0 = (uint32_t)base, c1 = (uint32_t)(base | (1 << k));
            fu = (int)(c0 | (c1 << 3));
        } else if (mids == 2) {
            const int f = (rg[0] != 1) ? 0 : (rg[1] != 1 ? 1 : 2);
            kind = kEdgesFaceLoop; ne = 4;
            fu = (f == 0) ? 1 : 0;
            fv = (f == 2) ? 1 : 2;
        } else {
            rect_face = 6;
            kind = kEdgesAll12; ne = 12;
        }
    }
    uint32_t list = (kind == kEdgesList) ? (uint32_t)fu : 0u;
    // ---- rectangle tests (radius 0)
    bool crossed = false;
    if (rect_face >= 0) {
        const int f0 = rect_face == 6 ? 0 : rect_face, f1 = rect_face == 6 ? 6 : rect_face + 1;
#pragma unroll 1
        for (int f = f0; f < f1; ++f) {
            const RB rr = coll_rect_call<T, P>(nm, A, B, T(0), o, f);
            RPM_NOTE(pol, rr.m);
            if (rr.v) { crossed = true; break; }
        }
        if (crossed) {
            d = T(0);
            kind = kEdgesNone; ne = 0;
        } else if (ce_face >= 0) {
            // getLineSegments (:542-574): edges of the projected face facing the other point
            const T *Q = ip ? A : B;
            const int c = ce_face > 2 ? ce_face - 3 : ce_face;
            const int u = (c == 0) ? 1 : 0, v = (c == 2) ? 1 : 2;
            const int fb = (ce_face > 2 ? 1 : 0) << c;
            const T qu = sel3(Q, u), qv = sel3(Q, v);
            kind = kEdgesList; ne = 0; list = 0u;
            int us = -1, vs = -1;
            if (RPM_TAKE(pol, P::lt(qu, sel6(o, u)))) us = 0;
            else if (RPM_TAKE(pol, P::gt(qu, sel6(o, u + 3)))) us = 1;
            if (RPM_TAKE(pol, P::lt(qv, sel6(o, v)))) vs = 0;
            else if (RPM_TAKE(pol, P::gt(qv, sel6(o, v + 3)))) vs = 1;
            if (us >= 0) {   // u fixed, v from min to max
                const uint32_t c0 = (uint32_t)(fb | (us << u)), c1 = c0 | (1u << v);
                list |= (c0 | (c1 << 3)) << (6 * ne);
                ++ne;
            }
            if (vs >= 0) {   // v fixed, u from min to max
                const uint32_t c0 = (uint32_t)(fb | (vs << v)), c1 = c0 | (1u << u);
                list |= (c0 | (c1 << 3)) << (6 * ne);
                ++ne;
            }
            // no edge leaves the reference's 3x2 matrix uninitialised (undefined);
            // that needs the segment to meet the face exactly on its border
        }
    }
    // ---- point (one axis class per coordinate, no overlap): distanceLineSegToPoint
    if (point >= 0) {
        T Cc[3];
        corner(o, point, Cc);
        d = seg_point(pol, nm, A, B, Cc);
    }
    // ---- box edges
#pragma unroll 1
    for (int k = 0; k < ne; ++k) {
        int c0, c1;
        edge_of(kind, list, base, fu, fv, k, c0, c1);
        T Cc[3], Dd[3];
        corner(o, c0, Cc);
        corner(o, c1, Dd);
        const T dt = seg_seg(pol, nm, A, B, Cc, Dd).v;
        if (direct) { d = dt; break; }
        if (dt <= T(0)) { d = T(0); break; }
        if (dt < d) d = dt;
    }
    return Val<T>{d - radius, 1.f};
}

// Out-of-line instances of the two trees per (T, policy): every drain of a
// kernel calls the same copy, so the instruction cache holds each tree once.
// The policy's smallest margin travels back by value.
template <typename T> struct ValM {
    T v;
    float ia, m;
};

template <typename T, typename P, bool FLAT = false>
__host__ __device__ __noinline__ RB coll_box_call(const Num<T> nm, const T *A, const T *B, T radius, T r_new,
                                                  const T *o) {
    P pol;
    const bool v = coll_box<T, P, FLAT>(pol, nm, A, B, radius, r_new, o);
    return RB{v, pol.m};
}

template <typename T, typename P>
__host__ __device__ __noinline__ ValM<T> capsule_box_call(const Num<T> nm, const T *A, const T *B, T radius,
                                                          const T *o) {
    P pol;
    const Val<T> r = capsule_box(pol, nm, A, B, radius, o);
    return ValM<T>{r.v, r.ia, pol.m};
}

// Lower bound of the segment-box distance: the gap between the box and the
// segment's own bounding box.  Any reference distance of the pair is at least
// this bound minus EQUALITY_THRESHOLD (the snap of :237, :338).
template <typename T> RPM_HD T gap2(const T *A, const T *B, const T *o) {
    T g2 = T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        T lo = A[c] < B[c] ? A[c] : B[c];
        T hi = A[c] < B[c] ? B[c] : A[c];
        T g = o[c] - hi;
        T g2b = lo - o[3 + c];
        g = g > g2b ? g : g2b;
        g = g > T(0) ? g : T(0);
        g2 = g2 + g * g;
    }
    return g2;
}

}  // namespace rpm
