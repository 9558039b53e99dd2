// rpm_spine.cuh -- the bubble and spine steps of the RBT planners on the
// device, in the reference's float numerics (the FP32_REF skeleton and plain
// IEEE float operations; compiled without contracted multiply-adds):
//   computeEnclosingRadii   xArm6.cpp:237-275, Spatial10DOF.cpp:11-30,
//                           Planar2DOF.cpp:132-148
//   extendSpine             RBTConnect.cpp:85-150 (self-collision checking off)
//   computeReachedState     DRGBT.cpp:475-495 = extendGenSpine
//                           (RGBTConnect.cpp:73-93) from the current state with
//                           computeDistanceUnderestimation after each layer.
// Sums over dynamic-size Eigen expressions (a skeleton column,
// R->col(i).dot(delta_q)) run in index order; fixed-size 3-vector reductions
// as x0 + (x1 + x2).
#pragma once
#include "rpm_dev.cuh"
#include "rpm_check.cuh"

namespace rpm {

enum { kStNone = 0, kStAdvanced = 1, kStTrapped = 2, kStReached = 3 };   // base::State::Status (State.h:22)

struct SpineParams {
    const DevRobot *robot;
    const float *q;          // [C][D] spine starts (extendSpine)
    const float *qe;         // [C][D] spine targets (the horizon for reached states)
    const float *dist;       // [C] d_c of each start (extendSpine)
    const float *profile;    // [C][L] its profile (extendSpine)
    int64_t C;
    int32_t num_iter;        // NUM_ITER_SPINE
    int32_t expanded;        // USE_EXPANDED_BUBBLE
    int32_t num_layers;      // NUM_LAYERS (reached states)
    float d_crit;            // RBTConnectConfig::D_CRIT (reached states)
    float *q_new;            // [C][D] output
    int32_t *status;         // [C] output
    float *radii;            // [C][D][D + 1] (enclosing radii)
    // reached states: the current state's computeDistance (reference float numerics)
    const float *q_cur;      // [D]
    const double *cur_dist;  // [1]
    const float *cur_prof;   // [L]
    const float *cur_near;   // [n][6][L]
    const float *cur_skel;   // [3 (D + 1)] its float skeleton, when the nearest-point kernel wrote it (nullable)
    int32_t n;
    float maxd;              // MAX_DISTANCE
    int32_t L;               // reached states: links (sizes the plane table below)
    int32_t planes;          // reached states: 1 = the CTA keeps the underestimation planes in shared memory
};

#ifdef __CUDACC__
__device__ __forceinline__ float max_std(float a, float b) { return (a < b) ? b : a; }   // std::max
__device__ __forceinline__ float min_std(float a, float b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ float dot3f(const float *a, const float *b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

// |a - b| over dynamic 3-element columns, summed in index order.
__device__ __forceinline__ float col_dist(const float *a, const float *b) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float d = a[k] - b[k];
        s = s + d * d;
    }
    return sqrtf(s);
}

// The reference's float skeleton (D + 1 points).
__device__ __forceinline__ void skel_ref(const DevRobot &rb, const float *q, float *sk) {
    SkelWalker<1> sw;
    sw.begin();
    for (int k = 0; k <= rb.D; ++k) sw.point(rb, q, k, sk + 3 * k);
}

// The same skeleton with the whole warp (every lane passes the same q): the
// warp computes the joints' sines and cosines (warp_sincos: the values the
// chain would compute itself) and every lane then runs the chain.  sc:
// 2 * kMaxDof doubles of the warp's shared memory.
__device__ __forceinline__ void skel_ref_warp(const DevRobot &rb, const float *q, float *sk, double *sc) {
    __syncwarp();
    warp_sincos(q, rb.D, sc);
    __syncwarp();
    SkelWalker<1> sw;
    sw.begin();
    sw.w.sc = sc;
    for (int k = 0; k <= rb.D; ++k) sw.point(rb, q, k, sk + 3 * k);
}

// Row i (D + 1 entries) of computeEnclosingRadii from the float skeleton.
static __device__ void enclosing_row(const DevRobot &rb, const float *sk, int i, float *row) {
    const int D = rb.D;
    for (int j = 0; j <= D; ++j) row[j] = 0.f;
    if (rb.kind == RPM_ROBOT_XARM6) {
        if (i >= D - 1) return;
        for (int j = i + 1; j <= D; ++j) {
            const float rn = j - 1 < D - 1 ? max_std(rb.radius_f[j - 1], rb.radius_f[j]) : rb.radius_f[D - 1];
            const float *pj = sk + 3 * j;
            if (i == 0) {
                if (j >= 2) row[j] = max_std(row[j - 1], sqrtf(pj[0] * pj[0] + pj[1] * pj[1]) + rn);
            } else if (i == 3) {
                if (j >= 5) {
                    const float *p3 = sk + 9, *p4 = sk + 12;
                    float AB[3], v[3], proj[3], w[3];
#pragma unroll
                    for (int k = 0; k < 3; ++k) { AB[k] = p4[k] - p3[k]; v[k] = pj[k] - p3[k]; }
                    const float t = dot3f(v, AB) / dot3f(AB, AB);
#pragma unroll
                    for (int k = 0; k < 3; ++k) { proj[k] = p3[k] + t * AB[k]; w[k] = pj[k] - proj[k]; }
                    row[j] = max_std(row[j - 1], sqrtf(dot3f(w, w)) + rn);
                }
            } else {
                row[j] = max_std(row[j - 1], col_dist(pj, sk + 3 * i) + rn);
            }
        }
        return;
    }
    const bool spatial = rb.kind == RPM_ROBOT_SPATIAL;
    for (int j = i + 1; j <= D; ++j) {
        const float *pj = sk + 3 * j;
        const float v = (i == 0 && spatial) ? sqrtf(pj[0] * pj[0] + pj[1] * pj[1]) : col_dist(pj, sk + 3 * i);
        row[j] = max_std(row[j - 1], v + rb.radius_f[j - 1]);
    }
}

// The term enclosing_row adds at column j of row i (0 where it adds none).
static __device__ __forceinline__ float enclosing_term(const DevRobot &rb, const float *sk, int i, int j) {
    const int D = rb.D;
    if (j <= i) return 0.f;
    const float *pj = sk + 3 * j;
    if (rb.kind == RPM_ROBOT_XARM6) {
        if (i >= D - 1) return 0.f;
        const float rn = j - 1 < D - 1 ? max_std(rb.radius_f[j - 1], rb.radius_f[j]) : rb.radius_f[D - 1];
        if (i == 0) return j >= 2 ? sqrtf(pj[0] * pj[0] + pj[1] * pj[1]) + rn : 0.f;
        if (i == 3) {
            if (j < 5) return 0.f;
            const float *p3 = sk + 9, *p4 = sk + 12;
            float AB[3], v[3], proj[3], w[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) { AB[k] = p4[k] - p3[k]; v[k] = pj[k] - p3[k]; }
            const float t = dot3f(v, AB) / dot3f(AB, AB);
#pragma unroll
            for (int k = 0; k < 3; ++k) { proj[k] = p3[k] + t * AB[k]; w[k] = pj[k] - proj[k]; }
            return sqrtf(dot3f(w, w)) + rn;
        }
        return col_dist(pj, sk + 3 * i) + rn;
    }
    const bool spatial = rb.kind == RPM_ROBOT_SPATIAL;
    const float v = (i == 0 && spatial) ? sqrtf(pj[0] * pj[0] + pj[1] * pj[1]) : col_dist(pj, sk + 3 * i);
    return v + rb.radius_f[j - 1];
}

// enclosing_row of every joint with the whole warp: each (i, j) term on a
// lane of its own, then each row's running maximum by lane i.  The terms are
// non-negative and max is exact, so the rows are enclosing_row's, bit for bit.
static __device__ void enclosing_rows_warp(const DevRobot &rb, const float *sk, float (*rows)[kMaxDof + 1]) {
    const int lane = threadIdx.x & 31;
    const int D = rb.D, W = D + 1;
    for (int e = lane; e < D * W; e += 32) {
        const int i = e / W, j = e - i * W;
        rows[i][j] = enclosing_term(rb, sk, i, j);
    }
    __syncwarp();
    if (lane < D) {
        float r = 0.f;
        for (int j = 0; j <= D; ++j) {
            r = max_std(r, rows[lane][j]);
            rows[lane][j] = r;
        }
    }
}

// extendSpine from q (its skeleton sk_q, distance d, profile prof) towards
// qe; q_new gets the end and sk_new its skeleton.  Each iteration computes
// one forward kinematics, of its new state: the skeleton of the state an
// iteration starts from is the previous iteration's (or sk_q).
// sc: the warp's shared sincos scratch when the whole warp runs this spine
// (every lane the same arguments), null for one spine per lane.
static __device__ int extend_spine(const DevRobot &rb, const float *q, const float *sk_q, float d, const float *prof,
                                   const float *qe, int num_iter, bool expanded, float *q_new, float *sk_new,
                                   double *sc = nullptr) {
    const int D = rb.D, L = D, NP = 3 * (D + 1);
    if (d <= 0.f) {
        for (int k = 0; k < D; ++k) q_new[k] = q[k];
        for (int k = 0; k < NP; ++k) sk_new[k] = sk_q[k];
        return kStTrapped;
    }
    float skt[3 * (kMaxDof + 1)];
    float qt[kMaxDof], dq[kMaxDof], rho_profile[kMaxDof], col[kMaxDof + 1], row[kMaxDof + 1];
    float rho = 0.f;
    for (int k = 0; k < NP; ++k) skt[k] = sk_q[k];
    for (int k = 0; k < D; ++k) { qt[k] = q[k]; rho_profile[k] = 0.f; }
    int status = kStAdvanced, counter = 0;
    for (;;) {
        for (int k = 0; k < D; ++k) dq[k] = fabsf(qe[k] - qt[k]);
        // R->col(j).dot(delta_q) for every column j, rows in index order
        for (int j = 0; j <= D; ++j) col[j] = 0.f;
        for (int i = 0; i < D; ++i) {
            enclosing_row(rb, skt, i, row);
            for (int j = 0; j <= D; ++j) col[j] = col[j] + row[j] * dq[i];
        }
        float step;
        if (expanded) {
            step = INFINITY;
            for (int i = 0; i < D; ++i) step = min_std(step, (prof[i] - rho_profile[i]) / col[i + 1]);
        } else {
            step = (d - rho) / col[D];
        }
        if (step > 1.f) {
            for (int k = 0; k < D; ++k) q_new[k] = qe[k];
            status = kStReached;
        } else {
            for (int k = 0; k < D; ++k) q_new[k] = qt[k] + step * (qe[k] - qt[k]);
        }
        if (sc) skel_ref_warp(rb, q_new, sk_new, sc);
        else skel_ref(rb, q_new, sk_new);
        if (++counter == num_iter || status != kStAdvanced) return status;
        float rk_prev = 0.f;
        for (int k = 1; k <= L; ++k) {
            const float rk = col_dist(sk_q + 3 * k, sk_new + 3 * k);
            rho_profile[k - 1] = max_std(rk_prev, rk);
            rk_prev = rk;
            rho = max_std(rho, rk);
        }
        for (int k = 0; k < D; ++k) qt[k] = q_new[k];
        for (int k = 0; k < NP; ++k) skt[k] = sk_new[k];
    }
}

// ---------------------------------------------------------------------------
// One spine with the whole warp (DRGBT's horizon: one warp per state).  The
// state lives in shared memory and the work is spread over the lanes: the
// enclosing-radius rows one per lane, the column sums R->col(j).dot(delta_q)
// one per lane (rows in index order), the joints one per lane; the step, the
// start's radii and rho in lane 0, in index order.  Every float operation is
// the one extend_spine performs, in its order, so the results are the same
// bits.
struct SpineWarp {
    float qn[kMaxDof], pn[kMaxDof], qe[kMaxDof];   // state, its profile, the target
    float qt[kMaxDof], qs[kMaxDof], dq[kMaxDof], rho_prof[kMaxDof], p[kMaxDof];
    float rk[kMaxDof + 1];
    float skn[3 * (kMaxDof + 1)], skt[3 * (kMaxDof + 1)], sk[3 * (kMaxDof + 1)];
    float rows[kMaxDof][kMaxDof + 1];
    float col[kMaxDof + 1];
    double sc[2 * kMaxDof];
};

// The reference's float skeleton of q (shared memory) into sk (shared
// memory): joint sines in parallel, then the chain spread over the warp.
__device__ __forceinline__ void skel_ref_shared(const DevRobot &rb, const float *q, float *sk, double *sc) {
    __syncwarp();
    warp_sincos(q, rb.D, sc);
    __syncwarp();
    skel_coop<1, float>(rb, sc, sk);
    __syncwarp();
}

// extendSpine from w.qn (skeleton w.skn, distance d, profile w.pn) towards
// w.qe; the end goes to w.qs and its skeleton to w.sk.  Returns the status
// (the same in every lane).
static __device__ int extend_spine_warp(const DevRobot &rb, SpineWarp &w, float d, int num_iter, bool expanded) {
    const int lane = threadIdx.x & 31;
    const int D = rb.D, L = D, NP = 3 * (D + 1);
    __syncwarp();
    if (d <= 0.f) {
        if (lane < D) w.qs[lane] = w.qn[lane];
        for (int k = lane; k < NP; k += 32) w.sk[k] = w.skn[k];
        __syncwarp();
        return kStTrapped;
    }
    for (int k = lane; k < NP; k += 32) w.skt[k] = w.skn[k];
    if (lane < D) { w.qt[lane] = w.qn[lane]; w.rho_prof[lane] = 0.f; }
    float rho = 0.f;   // lane 0's copy is the one used
    int counter = 0;
    __syncwarp();
    for (;;) {
        if (lane < D) w.dq[lane] = fabsf(w.qe[lane] - w.qt[lane]);
        enclosing_rows_warp(rb, w.skt, w.rows);
        __syncwarp();
        if (lane <= D) {
            float c = 0.f;
            for (int i = 0; i < D; ++i) c = c + w.rows[i][lane] * w.dq[i];
            w.col[lane] = c;
        }
        __syncwarp();
        float step = 0.f;
        if (expanded) {
            // the min over the joints of (p_i - rho_i) / col_{i+1}, a quotient
            // per lane: the serial min keeps the first of equal values and
            // passes over NaN, so the tree takes the lower joint on a tie and
            // NaN as +inf
            float x = INFINITY;
            if (lane < D) {
                x = (w.pn[lane] - w.rho_prof[lane]) / w.col[lane + 1];
                if (x != x) x = INFINITY;
            }
            int at = lane;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float y = __shfl_xor_sync(0xffffffffu, x, off);
                const int ay = __shfl_xor_sync(0xffffffffu, at, off);
                if (y < x || (y == x && ay < at)) { x = y; at = ay; }
            }
            step = x;
        } else {
            if (lane == 0) step = (d - rho) / w.col[D];
            step = __shfl_sync(0xffffffffu, step, 0);
        }
        const bool reached = step > 1.f;
        if (lane < D) w.qs[lane] = reached ? w.qe[lane] : w.qt[lane] + step * (w.qe[lane] - w.qt[lane]);
        skel_ref_shared(rb, w.qs, w.sk, w.sc);
        if (++counter == num_iter || reached) return reached ? kStReached : kStAdvanced;
        if (lane >= 1 && lane <= L) w.rk[lane] = col_dist(w.skn + 3 * lane, w.sk + 3 * lane);
        __syncwarp();
        if (lane == 0) {
            float rk_prev = 0.f;
            for (int k = 1; k <= L; ++k) {
                const float rk = w.rk[k];
                w.rho_prof[k - 1] = max_std(rk_prev, rk);
                rk_prev = rk;
                rho = max_std(rho, rk);
            }
        }
        for (int k = lane; k < NP; k += 32) w.skt[k] = w.sk[k];
        if (lane < D) w.qt[lane] = w.qs[lane];
        __syncwarp();
    }
}
#endif

cudaError_t launch_enclosing_radii(const SpineParams &p, cudaStream_t st);
cudaError_t launch_extend_spines(const SpineParams &p, cudaStream_t st);
cudaError_t launch_reached_states(const SpineParams &p, cudaStream_t st);

}  // namespace rpm

namespace rpm {

// MotionValidity::check for a batch of motions (rpm_motion_validity).
struct MotionParams {
    const DevRobot *robot;
    const float *obs_f;      // [8][n_pad] scene rows (float), ground row
    const double *obs_d;     // [7][n_pad]
    int32_t n, n_pad;
    const float *q_prev, *q_cur;   // [M][D]
    int64_t M;
    int32_t N;               // checks per motion
    int32_t n_mov;           // moving boxes
    float max_iter_time;
    const uint8_t *moving;   // [n] 1 = a moving box (its stored AABB is replaced)
    const int32_t *mov_idx;  // [n_mov] obstacle index
    const float *mov_aabb;   // [N][n_mov][6] AABB of each moving box before check k
    Num<double> nmd;
    Num<float> nmf;
    uint8_t *valid;
    int32_t *checks;
};

cudaError_t launch_motion_validity(int mode, const MotionParams &p, cudaStream_t st);

}  // namespace rpm
