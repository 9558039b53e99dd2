// rpm_dev.cuh -- device data layout, FK and obstacle staging shared by the
// kernels of the GB300 RealVectorSpace engine.
//
// Layout in HBM
//   robot   : DevRobot (one struct per uploaded robot, ~6 KB)
//   scene   : one allocation per obstacle-set version, n padded to n_pad
//             (a multiple of 16) so every row starts 16-byte aligned:
//               float  rows [8][n_pad] : xmin ymin zmin xmax ymax zmax tol ground(0/1)
//               double rows [7][n_pad] : xmin ymin zmin xmax ymax zmax tol (exact widening)
//   configs : float [C][D] row-major (one RealVectorSpaceState coordinate vector per row)
// Each CTA copies its scene into shared memory with one bulk-async (TMA)
// copy per row block and reads obstacles from there as warp-uniform broadcasts.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rpm_gpu.h"

#define RPM_HD __host__ __device__ __forceinline__

namespace rpm {

// Round-to-nearest multiply / add that are never contracted into an FMA.
RPM_HD double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
RPM_HD double dadd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
RPM_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
RPM_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

constexpr int kMaxDof = RPM_MAX_DOF;
constexpr int kMaxObstacles = RPM_MAX_OBSTACLES;   // per scene (the pair-recheck entry keeps 11 bits of index)
constexpr int kFRows = 8;               // float rows per scene
constexpr int kDRows = 7;               // double rows per scene
constexpr int kRowTol = 6;
constexpr int kRowGround = 7;
// Scenes of at most this many padded obstacles also get a per-obstacle copy of
// their float rows ([n_pad][8] floats) in the FP32 lane kernel's shared memory.
constexpr int kAosMaxPad = 512;
// FP32 + FP64-recheck thresholds.  The FP32 skeleton differs from the FP64
// one by at most ~2e-7 m on the reference's robots, so an FP32 branch decision
// whose (error-amplification-scaled) margin is at least kDecide = 1e-5 m takes
// the same branch in FP64.  Clearances within the contact band kBand = 1e-4 m
// of zero (or of an obstacle's min_dist_tol) always go to FP64.
constexpr float kDecide = 1e-5f;
constexpr float kBand = 1e-4f;
constexpr unsigned kWaitLimit = 1u << 22;   // bounded spin on an mbarrier

// device status codes (written to the context's status word)
constexpr int kStatusTimeout = 1;

struct DevRobot {
    int32_t kind, D, ground_included, rot_identity_mask;
    int32_t axis[kMaxDof];
    float radius_f[kMaxDof];
    float rnew_f[kMaxDof];       // (float)((double)r * sqrt(3) / 3)  CollisionAndDistance.cpp:7
    double radius_d[kMaxDof];
    double rnew_d[kMaxDof];      // r * sqrt(3) / 3 in double
    double gripper_d;            // (double)gripper_length
    float gripper_f;
    float grip03_f;              // (float)(0.3 * (double)gripper_length)   xArm6.cpp:231
    double oxyz[kMaxDof + 1][3];
    double orot[kMaxDof + 1][9];
    float oxyz_f[kMaxDof + 1][3];
    float orot_f[kMaxDof + 1][9];
};
// The robot is bulk-copied to shared memory ahead of 16-byte aligned rows.
static_assert(sizeof(DevRobot) % 16 == 0, "DevRobot must be a multiple of 16 bytes");

// One contiguous run of configurations checked against one scene.
struct Seg {
    const DevRobot *robot;
    const float *obs_f;      // [8][n_pad]
    const double *obs_d;     // [7][n_pad]
    const float *q;          // [count][D]
    uint8_t *valid;          // nullable
    double *dist;            // nullable
    float *profile;          // nullable, [count][L]
    int64_t count;
    int64_t first_block;     // first CTA of this segment in the launch
    int32_t n, n_pad;
    // spatially sorted copy (warp-per-configuration kernels)
    const float *srt_f;      // [8][ns]: AABB, tol, original index | ground bit (as bits)
    const double *srt_d;     // [7][ns]
    const float *blk;        // [nb][8]: union bounds, max tol, min tol of each block of 32 slots
    int32_t ns, nb;
    // FP32 lane kernel: the order in which configurations are checked (binned
    // by their first joint angles), nullable = index order.  Thread t checks
    // configuration perm[t]; outputs and recheck records use that index.
    const int32_t *perm;
};

struct LaunchCtl {
    const Seg *segs;
    int32_t nseg;
    int32_t pad;
    uint64_t *recheck;       // FP32 pass: (seg << 40 | config) of configs to recompute in FP64
    uint32_t *recheck_count;
    uint32_t recheck_cap;
    int32_t *status;
};

// ------------------------------------------------------------------ sincos --
// Cody-Waite reduction by pi/2 (three-part split; P1, P2 carry 33 significant
// bits) and Taylor series on [-pi/4, pi/4] through r^17 / r^18.  Every
// operation is an IEEE-754 round-to-nearest add or multiply, so with
// contraction disabled the result is bit-identical on any IEEE host.
RPM_HD void taylor_sincos(double x, double *so, double *co) {
    const double kTwoOverPi = 0x1.45f306dc9c883p-1;
    const double kP1 = 0x1.921fb54400000p+0;
    const double kP2 = 0x1.0b4611a600000p-34;
    const double kP3 = 0x1.3198a2e037073p-69;
    double kd = rint(dmul(x, kTwoOverPi));
    double r = dadd(x, -dmul(kd, kP1));
    r = dadd(r, -dmul(kd, kP2));
    r = dadd(r, -dmul(kd, kP3));
    double z = dmul(r, r);
    double ps = 0x1.952c77030ad4ap-49;
    ps = dadd(-0x1.ae7f3e733b81fp-41, dmul(z, ps));
    ps = dadd(0x1.6124613a86d09p-33, dmul(z, ps));
    ps = dadd(-0x1.ae64567f544e4p-26, dmul(z, ps));
    ps = dadd(0x1.71de3a556c734p-19, dmul(z, ps));
    ps = dadd(-0x1.a01a01a01a01ap-13, dmul(z, ps));
    ps = dadd(0x1.1111111111111p-7, dmul(z, ps));
    ps = dadd(-0x1.5555555555555p-3, dmul(z, ps));
    double s = dadd(r, dmul(dmul(r, z), ps));
    double pc = -0x1.6827863b97d97p-53;
    pc = dadd(0x1.ae7f3e733b81fp-45, dmul(z, pc));
    pc = dadd(-0x1.93974a8c07c9dp-37, dmul(z, pc));
    pc = dadd(0x1.1eed8eff8d898p-29, dmul(z, pc));
    pc = dadd(-0x1.27e4fb7789f5cp-22, dmul(z, pc));
    pc = dadd(0x1.a01a01a01a01ap-16, dmul(z, pc));
    pc = dadd(-0x1.6c16c16c16c17p-10, dmul(z, pc));
    pc = dadd(0x1.5555555555555p-5, dmul(z, pc));
    pc = dadd(-0x1.0000000000000p-1, dmul(z, pc));
    double c = dadd(1.0, dmul(z, pc));
    long long k = (long long)kd;
    switch (k & 3) {
        case 0: *so = s; *co = c; break;
        case 1: *so = c; *co = -s; break;
        case 2: *so = -s; *co = -c; break;
        default: *so = -c; *co = s; break;
    }
}

// --------------------------------------------------------------------- FK --
// F <- F * origin_k * Rot(axis_k, q_k) (KDL's root-to-tip composition).
template <typename F> struct Fk {
    F R[9];
    F p[3];
    RPM_HD void init() {
#pragma unroll
        for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0) ? F(1) : F(0);
        p[0] = p[1] = p[2] = F(0);
    }
};

// Right-multiplication of R by a rotation about the joint axis: columns
// (IA, IB) become (a c + b s, b c - a s).
template <int IA, int IB> RPM_HD void rot_cols_d(double *R, double c, double s) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const double a = R[3 * i + IA], b = R[3 * i + IB];
        R[3 * i + IA] = dadd(dmul(a, c), dmul(b, s));
        R[3 * i + IB] = dadd(dmul(b, c), -dmul(a, s));
    }
}
template <int IA, int IB> RPM_HD void rot_cols_f(float *R, float c, float s) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float a = R[3 * i + IA], b = R[3 * i + IB];
        R[3 * i + IA] = a * c + b * s;
        R[3 * i + IB] = b * c - a * s;
    }
}

// sc (nullable): sin / cos of every joint angle, computed ahead (in parallel)
// with taylor_sincos, so the serial chain holds only the rigid transforms.
RPM_HD void fk_step_d(Fk<double> &f, const DevRobot &rb, int k, double q, const double *sc = nullptr) {
    const double *o = rb.oxyz[k];
    double np[3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
        np[i] = dadd(dadd(dadd(dmul(f.R[3 * i + 0], o[0]), dmul(f.R[3 * i + 1], o[1])),
                                    dmul(f.R[3 * i + 2], o[2])),
                          f.p[i]);
#pragma unroll
    for (int i = 0; i < 3; ++i) f.p[i] = np[i];
    if (!((rb.rot_identity_mask >> k) & 1)) {
        const double *M = rb.orot[k];
        double nR[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j)
                nR[3 * i + j] = dadd(dadd(dmul(f.R[3 * i + 0], M[j]), dmul(f.R[3 * i + 1], M[3 + j])),
                                          dmul(f.R[3 * i + 2], M[6 + j]));
#pragma unroll
        for (int i = 0; i < 9; ++i) f.R[i] = nR[i];
    }
    double s, c;
    if (sc) { s = sc[2 * k]; c = sc[2 * k + 1]; }
    else taylor_sincos(q, &s, &c);
    switch (rb.axis[k]) {   // columns (a, b) <- (a c + b s, b c - a s)
        case 0: rot_cols_d<1, 2>(f.R, c, s); break;
        case 1: rot_cols_d<2, 0>(f.R, c, s); break;
        default: rot_cols_d<0, 1>(f.R, c, s); break;
    }
}

RPM_HD void fk_step_f(Fk<float> &f, const DevRobot &rb, int k, float q) {
    const float *o = rb.oxyz_f[k];
    float np[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) np[i] = f.R[3 * i + 0] * o[0] + f.R[3 * i + 1] * o[1] + f.R[3 * i + 2] * o[2] + f.p[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) f.p[i] = np[i];
    if (!((rb.rot_identity_mask >> k) & 1)) {
        const float *M = rb.orot_f[k];
        float nR[9];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) nR[3 * i + j] = f.R[3 * i + 0] * M[j] + f.R[3 * i + 1] * M[3 + j] + f.R[3 * i + 2] * M[6 + j];
#pragma unroll
        for (int i = 0; i < 9; ++i) f.R[i] = nR[i];
    }
    float s, c;
    sincosf(q, &s, &c);
    switch (rb.axis[k]) {
        case 0: rot_cols_f<1, 2>(f.R, c, s); break;
        case 1: rot_cols_f<2, 0>(f.R, c, s); break;
        default: rot_cols_f<0, 1>(f.R, c, s); break;
    }
}

// Walks the skeleton points 0..L of one configuration in order, advancing the
// FK only as far as the next point needs (so an early exit also skips FK).
//   CHAIN : point k = origin of chain segment k; point D = tool
//           (Planar2DOF.cpp:125-126)
//   XARM6 : 0, F1.p, F2.p, F3.p - 0.25 z3, F4.p, F4.p + 0.076 x4,
//           F5.p + g z5 - 0.3 g z5   (xArm6.cpp:130, 215-231)
// MODE 0: FP64 points.  MODE 1: the reference's float skeleton (FP64 FK,
// rounded, line (*) of xArm6.cpp:231 in float).  MODE 2: FP32 FK.
template <int MODE> struct SkelWalker;

template <> struct SkelWalker<0> {
    Fk<double> f;
    const double *sc = nullptr;   // precomputed joint sin / cos (nullable)
    RPM_HD void begin() { f.init(); }
    RPM_HD void point(const DevRobot &rb, const float *q, int k, double *out) {
        if (rb.kind != RPM_ROBOT_XARM6) {
            if (k < rb.D) {
                fk_step_d(f, rb, k, (double)q[k], sc);
                out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2];
            } else {
                const double *o = rb.oxyz[rb.D];
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    out[i] = dadd(dadd(dadd(dmul(f.R[3 * i], o[0]), dmul(f.R[3 * i + 1], o[1])),
                                                 dmul(f.R[3 * i + 2], o[2])),
                                       f.p[i]);
            }
            return;
        }
        switch (k) {
            case 0: out[0] = out[1] = out[2] = 0.0; break;
            case 1: fk_step_d(f, rb, 0, (double)q[0], sc); fk_step_d(f, rb, 1, (double)q[1], sc);
                    out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2]; break;
            case 2: fk_step_d(f, rb, 2, (double)q[2], sc); out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2]; break;
            case 3: fk_step_d(f, rb, 3, (double)q[3], sc);
#pragma unroll
                    for (int i = 0; i < 3; ++i) out[i] = dadd(f.p[i], -dmul(f.R[3 * i + 2], 0.25));
                    break;
            case 4: fk_step_d(f, rb, 4, (double)q[4], sc); out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2]; break;
            case 5:
#pragma unroll
                    for (int i = 0; i < 3; ++i) out[i] = dadd(f.p[i], dmul(f.R[3 * i + 0], 0.076));
                    break;
            default: {
                fk_step_d(f, rb, 5, (double)q[5], sc);
                const double g = rb.gripper_d, g3 = dmul(0.3, rb.gripper_d);
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    double z = f.R[3 * i + 2];
                    double ps = dadd(f.p[i], dmul(g, z));
                    out[i] = dadd(ps, -dmul(g3, z));
                }
            }
        }
    }
};

template <> struct SkelWalker<1> {
    SkelWalker<0> w;
    RPM_HD void begin() { w.begin(); }
    RPM_HD void point(const DevRobot &rb, const float *q, int k, float *out) {
        if (rb.kind == RPM_ROBOT_XARM6 && k == 6) {
            fk_step_d(w.f, rb, 5, (double)q[5], w.sc);
            const double g = rb.gripper_d;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                double z = w.f.R[3 * i + 2];
                float ps = (float)dadd(w.f.p[i], dmul(g, z));
                out[i] = fadd(ps, -fmul(rb.grip03_f, (float)z));
            }
            return;
        }
        double d[3];
        w.point(rb, q, k, d);
        out[0] = (float)d[0]; out[1] = (float)d[1]; out[2] = (float)d[2];
    }
};

template <> struct SkelWalker<2> {
    Fk<float> f;
    RPM_HD void begin() { f.init(); }
    RPM_HD void point(const DevRobot &rb, const float *q, int k, float *out) {
        if (rb.kind != RPM_ROBOT_XARM6) {
            if (k < rb.D) {
                fk_step_f(f, rb, k, q[k]);
                out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2];
            } else {
                const float *o = rb.oxyz_f[rb.D];
#pragma unroll
                for (int i = 0; i < 3; ++i) out[i] = f.R[3 * i] * o[0] + f.R[3 * i + 1] * o[1] + f.R[3 * i + 2] * o[2] + f.p[i];
            }
            return;
        }
        switch (k) {
            case 0: out[0] = out[1] = out[2] = 0.f; break;
            case 1: fk_step_f(f, rb, 0, q[0]); fk_step_f(f, rb, 1, q[1]);
                    out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2]; break;
            case 2: fk_step_f(f, rb, 2, q[2]); out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2]; break;
            case 3: fk_step_f(f, rb, 3, q[3]);
#pragma unroll
                    for (int i = 0; i < 3; ++i) out[i] = f.p[i] - f.R[3 * i + 2] * 0.25f;
                    break;
            case 4: fk_step_f(f, rb, 4, q[4]); out[0] = f.p[0]; out[1] = f.p[1]; out[2] = f.p[2]; break;
            case 5:
#pragma unroll
                    for (int i = 0; i < 3; ++i) out[i] = f.p[i] + f.R[3 * i + 0] * 0.076f;
                    break;
            default: {
                fk_step_f(f, rb, 5, q[5]);
                const float g7 = 0.7f * rb.gripper_f;
#pragma unroll
                for (int i = 0; i < 3; ++i) out[i] = f.p[i] + g7 * f.R[3 * i + 2];
            }
        }
    }
};

#ifdef __CUDACC__
// ---------------------------------------------------------- warp sincos --
// The sines and cosines of q[0..D-1] into sc (sin, cos per joint): the values
// taylor_sincos computes, with one warp.  Lane j evaluates joint j's sine and
// lane 16 + j its cosine.  The two polynomials run as one instruction stream:
// the sine's starts one Horner step earlier from 0 (z * 0 + c0 is c0), and
// the coefficients and the final factor are selected per lane.  The quadrant
// swap then trades the two values across the half-warps.  Each value comes
// from taylor_sincos's operations in their order.  On this part a warp's FP64
// instruction occupies the FP64 pipe for its whole width, so the cost goes
// with the number of instructions issued, not with the lanes that need them.
// Every lane calls it; more than 16 joints take one lane per joint.
__device__ __forceinline__ void warp_sincos(const float *q, int D, double *sc) {
    const int lane = threadIdx.x & 31;
    if (D > 16) {
        if (lane < D) taylor_sincos((double)q[lane], &sc[2 * lane], &sc[2 * lane + 1]);
        return;
    }
    const int j = lane & 15;
    const bool is_sin = lane < 16;
    const double x = j < D ? (double)q[j] : 0.0;
    const double kTwoOverPi = 0x1.45f306dc9c883p-1;
    const double kP1 = 0x1.921fb54400000p+0;
    const double kP2 = 0x1.0b4611a600000p-34;
    const double kP3 = 0x1.3198a2e037073p-69;
    const double kd = rint(dmul(x, kTwoOverPi));
    double r = dadd(x, -dmul(kd, kP1));
    r = dadd(r, -dmul(kd, kP2));
    r = dadd(r, -dmul(kd, kP3));
    const double z = dmul(r, r);
    const double rz = dmul(r, z);
    double p = is_sin ? 0.0 : -0x1.6827863b97d97p-53;
    p = dadd(is_sin ? 0x1.952c77030ad4ap-49 : 0x1.ae7f3e733b81fp-45, dmul(z, p));
    p = dadd(is_sin ? -0x1.ae7f3e733b81fp-41 : -0x1.93974a8c07c9dp-37, dmul(z, p));
    p = dadd(is_sin ? 0x1.6124613a86d09p-33 : 0x1.1eed8eff8d898p-29, dmul(z, p));
    p = dadd(is_sin ? -0x1.ae64567f544e4p-26 : -0x1.27e4fb7789f5cp-22, dmul(z, p));
    p = dadd(is_sin ? 0x1.71de3a556c734p-19 : 0x1.a01a01a01a01ap-16, dmul(z, p));
    p = dadd(is_sin ? -0x1.a01a01a01a01ap-13 : -0x1.6c16c16c16c17p-10, dmul(z, p));
    p = dadd(is_sin ? 0x1.1111111111111p-7 : 0x1.5555555555555p-5, dmul(z, p));
    p = dadd(is_sin ? -0x1.5555555555555p-3 : -0x1.0000000000000p-1, dmul(z, p));
    // sine: r + (r z) ps; cosine: 1 + z pc
    const double v = dadd(is_sin ? r : 1.0, dmul(is_sin ? rz : z, p));
    const double o = __shfl_xor_sync(0xffffffffu, v, 16);   // the other value of the same joint
    const int qd = (int)((long long)kd & 3);
    // quadrant 0..3: sin = s, c, -s, -c and cos = c, -s, -c, s
    const double base = (qd & 1) ? o : v;
    const bool neg = is_sin ? (qd & 2) != 0 : (qd == 1 || qd == 2);
    if (j < D) sc[2 * j + (is_sin ? 0 : 1)] = neg ? -base : base;
}

// ------------------------------------------------ warp forward kinematics --
// The FP64 chain of SkelWalker<MODE> (MODE 0: FP64 points; MODE 1: the
// reference's float skeleton) run by a whole warp: lane e < 9 holds R[e]
// (row e / 3, column e % 3), lanes 9-11 hold p[lane - 9].  Each element is
// computed with the operations fk_step_d and SkelWalker use, in their order,
// so the points are the same bits; the serial chain per joint is a few
// shuffles and three products instead of about eighty FP64 operations.
// Every lane of the warp calls it; sc holds the joints' sines and cosines
// (taylor_sincos or warp_sincos, computed ahead); lanes 9-11 write the D + 1 points to out.
template <int MODE, typename TO>
__device__ void skel_coop(const DevRobot &rb, const double *sc, TO *out) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool is_r = lane < 9, is_p = lane >= 9 && lane < 12;
    const int row = is_r ? lane / 3 : (is_p ? lane - 9 : 0);
    const int col = is_r ? lane % 3 : 0;
    double v = (is_r && lane % 4 == 0) ? 1.0 : 0.0;   // R = I, p = 0
    auto rowval = [&](int t) { return __shfl_sync(full, v, 3 * row + t); };
    auto emit = [&](int kp, double x) {
        if (is_p) out[3 * kp + row] = (TO)x;
    };
    // One joint with no divergent FP64 code: every lane issues the same nine
    // FP64 instructions and keeps its own result by a select.  The p lanes
    // take p + R o_k (r0 o0 + r1 o1, + r2 o2, + p); the R lanes R M_k (the
    // same products and sums without the last; skipped for an identity M_k).
    auto step = [&](int k) {
        const double r0 = rowval(0), r1 = rowval(1), r2 = rowval(2);
        const double *X = is_p ? rb.oxyz[k] : rb.orot[k] + col;
        const int sx = is_p ? 1 : 3;
        const double t = dadd(dadd(dmul(r0, X[0]), dmul(r1, X[sx])), dmul(r2, X[2 * sx]));
        const double tp = dadd(t, v);
        const bool rot = is_r && !((rb.rot_identity_mask >> k) & 1);
        v = is_p ? tp : (rot ? t : v);
        // columns (IA, IB) <- (a c + b s, b c - a s), as rot_cols_d; x (-s)
        // is -(x s) exactly
        const int ax = rb.axis[k];
        const int ia = ax == 0 ? 1 : (ax == 1 ? 2 : 0), ib = ax == 0 ? 2 : (ax == 1 ? 0 : 1);
        const double sn = sc[2 * k], cs = sc[2 * k + 1];
        const double x = __shfl_sync(full, v, is_r ? 3 * row + (col == ia ? ib : ia) : lane);
        const bool a = is_r && col == ia, b = is_r && col == ib;
        const double w = dadd(dmul(v, cs), dmul(x, b ? -sn : sn));
        v = (a || b) ? w : v;
    };
    const int D = rb.D;
    if (rb.kind != RPM_ROBOT_XARM6) {
        for (int k = 0; k < D; ++k) {
            step(k);
            emit(k, v);
        }
        const double r0 = rowval(0), r1 = rowval(1), r2 = rowval(2);
        const double *o = rb.oxyz[D];
        emit(D, dadd(dadd(dadd(dmul(r0, o[0]), dmul(r1, o[1])), dmul(r2, o[2])), v));
        return;
    }
    emit(0, 0.0);
    step(0);
    step(1);
    emit(1, v);
    step(2);
    emit(2, v);
    step(3);
    {
        const double z = rowval(2);
        emit(3, dadd(v, -dmul(z, 0.25)));
    }
    step(4);
    emit(4, v);
    {
        const double x = rowval(0);
        emit(5, dadd(v, dmul(x, 0.076)));
    }
    step(5);
    const double z = rowval(2);
    if constexpr (MODE == 0) {
        const double g = rb.gripper_d, g3 = dmul(0.3, rb.gripper_d);
        emit(6, dadd(dadd(v, dmul(g, z)), -dmul(g3, z)));
    } else if (is_p) {
        const float ps = (float)dadd(v, dmul(rb.gripper_d, z));
        out[18 + row] = (TO)fadd(ps, -fmul(rb.grip03_f, (float)z));
    }
}
#endif

// --------------------------------------------------- shared-memory staging --
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bulk-async (TMA) copies global -> shared completed on an mbarrier.  Sizes
// are multiples of 16 bytes and both addresses 16-byte aligned.  Thread 0
// arms the barrier with the total byte count and issues the copies; every
// thread then waits with a bounded spin, which on expiry records
// kStatusTimeout and returns false instead of hanging.
__device__ __forceinline__ void bulk_init(uint64_t *bar) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}

__device__ __forceinline__ void bulk_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy(uint64_t *bar, void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool bulk_wait(uint64_t *bar, uint32_t parity, int32_t *status,
                                          unsigned limit = kWaitLimit) {
    uint32_t done = 0;
    for (unsigned it = 0; it < limit; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    if (status) atomicCAS(status, 0, kStatusTimeout);
    return false;
}

}  // namespace rpm
