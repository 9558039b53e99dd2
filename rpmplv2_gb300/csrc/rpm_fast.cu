// rpm_fast.cu -- the FP32 bulk pass of the FP32 + FP64-recheck form.  Every
// decision of both trees carries a margin; pairs whose decisions fell within
// kBand of a boundary are listed and re-evaluated in FP64 by the pair recheck
// (rpm_exact.cu), or, when the lists are full, their configurations are
// recomputed whole by k_recheck.
#include <algorithm>

#include "rpm_check.cuh"
#include "rpm_edges.cuh"
#include "rpm_launch.cuh"
#include "rpm_wide.cuh"

namespace rpm {

// KIND: 1 = every segment of the launch is isValid only, 2 = distance /
// profile only, 3 = distance only, 0 = mixed (the body compiled for the
// launch's outputs).
template <int KIND>
__global__ void __launch_bounds__(kThreads, 5) k_check_fp32(const __grid_constant__ KParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ WarpShared<float> wsh[kThreads / 32];
    int s = 0;
    while (s + 1 < P.nseg && P.segs[s + 1].first_block <= (int64_t)blockIdx.x) ++s;
    const Seg &sg = P.segs[s];
    bulk_init(&bar);
    if (threadIdx.x == 0) {
        const uint32_t rb = (uint32_t)sizeof(DevRobot);
        const uint32_t rows = (uint32_t)(kFRows * sg.n_pad * sizeof(float));
        bulk_expect(&bar, rb + rows);
        bulk_copy(&bar, smem, sg.robot, rb);
        bulk_copy(&bar, smem + rb, sg.obs_f, rows);
    }
    if (!bulk_wait(&bar, 0, P.status)) return;
    const DevRobot &rb = *reinterpret_cast<const DevRobot *>(smem);
    const float *rows = reinterpret_cast<const float *>(smem + sizeof(DevRobot));
    // The obstacle loop reads each obstacle's rows as two 16-byte words.
    float4 *aos = nullptr;
    if (sg.n_pad <= kAosMaxPad) {
        aos = reinterpret_cast<float4 *>(smem + sizeof(DevRobot) + (size_t)kFRows * sg.n_pad * sizeof(float));
        for (int t = threadIdx.x; t < sg.n; t += kThreads) {
            const int np = sg.n_pad;
            aos[2 * t] = make_float4(rows[t], rows[np + t], rows[2 * np + t], rows[3 * np + t]);
            aos[2 * t + 1] = make_float4(rows[4 * np + t], rows[5 * np + t], rows[kRowTol * np + t],
                                         rows[kRowGround * np + t]);
        }
        __syncthreads();
    }
    const int64_t t = (int64_t)(blockIdx.x - sg.first_block) * kThreads + threadIdx.x;
    const int64_t warp0 = t - (threadIdx.x & 31);
    if (warp0 >= sg.count) return;   // whole warp idle
    const bool active = t < sg.count;
    const int64_t c = (active && sg.perm) ? (int64_t)sg.perm[t] : t;   // the configuration this thread checks
    ObsView<float> ob{rows, rows + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
    ob.aos = aos;
    const Want w{sg.valid != nullptr, sg.dist != nullptr, sg.profile != nullptr};
    const int D = rb.D;
    int hl = -1, hj = 0x7fffffff, slot = -1;
    uint8_t *vo = (w.valid && active) ? sg.valid + c : nullptr;
    double *dout = (w.dist && active) ? sg.dist + c : nullptr;
    float *po = (w.profile && active) ? sg.profile + c * D : nullptr;
    int st;
    if constexpr (KIND == 1 || KIND == 3) {
        // the order-free kinds: the skeleton buffer follows the rows and their per-obstacle copy
        float *skel = reinterpret_cast<float *>(smem + sizeof(DevRobot) + (size_t)kFRows * sg.n_pad * sizeof(float) +
                                                (aos ? (size_t)sg.n_pad * kFRows * sizeof(float) : 0));
        st = warp_check_any<KIND, kThreads>(wsh[threadIdx.x >> 5], skel, rb, ob, sg.q + c * D, active, P.nmf, vo, dout,
                                            &P.ps, &slot);
    } else {
        st = warp_check<2, float, KIND>(wsh[threadIdx.x >> 5], rb, ob, sg.q + c * D, active, P.nmf, w, vo, dout, po,
                                        &P.ps, &slot, &hl, &hj);
    }
    if (active) {
        complete_record(&P.ps, slot, st, s, c, hl, hj);
        if (st == kFull) recheck_whole(P, s, c);
    }
}

// ------------------------------------------------------------ check order --
// A large batch is checked in an order that puts configurations with similar
// first joint angles into the same warp (the first three joints place most of
// the arm), so a warp's skeletons span a small part of the workspace: the
// obstacle culling of warp_check_any then skips most obstacles for the whole
// warp, and the warp's pairs take similar branches of the trees.  A counting
// sort over 16^3 bins; the order within a bin is whatever the atomics give,
// which changes no output (every configuration's result depends on itself
// alone).
__device__ __forceinline__ int config_bin(const float *q, int D) {
    int key = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int b = 0;
        if (k < D) {
            const float x = (q[k] + 3.14159265f) * (16.f / 6.28318531f);
            b = x > 0.f ? (x < 15.f ? (int)x : 15) : 0;   // clamped; NaN -> 0
        }
        key = key * 16 + b;
    }
    return key;
}

__global__ void __launch_bounds__(1024) k_bin_count(const float *q, int64_t C, int D, int32_t *bins) {
    __shared__ int32_t h[kConfigBins];
    for (int k = threadIdx.x; k < kConfigBins; k += blockDim.x) h[k] = 0;
    __syncthreads();
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[config_bin(q + c * D, D)], 1);
    __syncthreads();
    for (int k = threadIdx.x; k < kConfigBins; k += blockDim.x)
        if (h[k]) atomicAdd(&bins[k], h[k]);
}

// Exclusive scan of the counts into bins[kConfigBins..] (one CTA of 1024 threads, 4 bins each).
__global__ void __launch_bounds__(1024) k_bin_scan(int32_t *bins) {
    __shared__ int32_t part[1024];
    const int t = threadIdx.x;
    int32_t v[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[k] = bins[4 * t + k]; sum += v[k]; }
    part[t] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int32_t x = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    int32_t run = part[t] - sum;
#pragma unroll
    for (int k = 0; k < 4; ++k) { bins[kConfigBins + 4 * t + k] = run; run += v[k]; }
}

__global__ void k_bin_scatter(const float *q, int64_t C, int D, int32_t *bins, int32_t *perm) {
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
        const int32_t pos = atomicAdd(&bins[kConfigBins + config_bin(q + c * D, D)], 1);
        perm[pos] = (int32_t)c;
    }
}

// A small batch in one CTA: count, scan and scatter in shared memory, one launch.
__global__ void __launch_bounds__(1024) k_bin_small(const float *q, int32_t C, int D, int32_t *perm) {
    __shared__ int32_t h[kConfigBins];
    __shared__ int32_t part[1024];
    const int t = threadIdx.x;
    for (int k = t; k < kConfigBins; k += 1024) h[k] = 0;
    __syncthreads();
    for (int c = t; c < C; c += 1024) atomicAdd(&h[config_bin(q + (int64_t)c * D, D)], 1);
    __syncthreads();
    int32_t v[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) { v[k] = h[4 * t + k]; sum += v[k]; }
    part[t] = sum;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int32_t x = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    int32_t run = part[t] - sum;
#pragma unroll
    for (int k = 0; k < 4; ++k) { h[4 * t + k] = run; run += v[k]; }
    __syncthreads();
    for (int c = t; c < C; c += 1024) perm[atomicAdd(&h[config_bin(q + (int64_t)c * D, D)], 1)] = c;
}

cudaError_t launch_bin_configs(const float *q, int64_t C, int D, int32_t *bins, int32_t *perm, cudaStream_t st) {
    static_assert(kConfigBins == 4 * 1024, "k_bin_scan scans 4 bins per thread");
    if (C <= 0) return cudaSuccess;
    if (C <= kBinSmallConfigs) {
        k_bin_small<<<1, 1024, 0, st>>>(q, (int32_t)C, D, perm);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(bins, 0, kConfigBins * sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    const unsigned grid = (unsigned)std::min<int64_t>((C + 1023) / 1024, 256);
    k_bin_count<<<grid, 1024, 0, st>>>(q, C, D, bins);
    k_bin_scan<<<1, 1024, 0, st>>>(bins);
    k_bin_scatter<<<(unsigned)std::min<int64_t>((C + 255) / 256, 4096), 256, 0, st>>>(q, C, D, bins, perm);
    return cudaGetLastError();
}

// FP32 pass of the warp-per-configuration form; unsettled configurations go
// to the same recheck list as k_check_fp32's.
__global__ void __launch_bounds__(kWideThreads, 2) k_check_wide_fp32(const __grid_constant__ KParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ MultiState<float> ms[kWideWarps];
    int s = 0;
    while (s + 1 < P.nseg && P.segs[s + 1].first_block <= (int64_t)blockIdx.x) ++s;
    bulk_init(&bar);
    wide_kernel_body<2>(P, smem, &bar, ms, s);
}

cudaError_t launch_check_wide_fp32(const KParams &p, int64_t blocks, size_t smem, cudaStream_t st) {
    static std::atomic<uint64_t> attr{0};
    ensure_smem_limit(k_check_wide_fp32, 200 * 1024, attr);
    k_check_wide_fp32<<<(unsigned)blocks, kWideThreads, smem, st>>>(p);
    return cudaGetLastError();
}

// FP32 pass of the warp-per-check edge form (MULTI: several segments).
template <bool MULTI>
__global__ void __launch_bounds__(kWideThreads, 2) k_edges_wide_fp32(const __grid_constant__ EdgeParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ MultiState<float> ms[kWideWarps];
    bulk_init(&bar);
    edge_wide_body<2, MULTI>(P, smem, &bar, ms);
}

cudaError_t launch_edges_wide_fp32(const EdgeParams &p, int grid, size_t smem, cudaStream_t st) {
    static std::atomic<uint64_t> attr[2] = {{0}, {0}};
    if (p.nseg - p.nseg_lane > 1) {
        ensure_smem_limit(k_edges_wide_fp32<true>, 200 * 1024, attr[1]);
        k_edges_wide_fp32<true><<<grid, kWideThreads, smem, st>>>(p);
    } else {
        ensure_smem_limit(k_edges_wide_fp32<false>, 200 * 1024, attr[0]);
        k_edges_wide_fp32<false><<<grid, kWideThreads, smem, st>>>(p);
    }
    return cudaGetLastError();
}

// FP32 pass of the edge checks (unsettled checks go to the pair recheck or k_edge_recheck).
// MULTI: several lane-layout segments, robots and scenes read from global
// memory; otherwise one segment staged in shared memory.  Two instances, so
// each holds one copy of the check code (the pass is fetch-bound on it).
template <bool MULTI>
__global__ void __launch_bounds__(kThreads) k_edges_fp32(const __grid_constant__ EdgeParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ WarpShared<float> wsh[kThreads / 32];
    __shared__ float qbuf[kThreads / 32][32 * kMaxDof];
    if constexpr (MULTI) {
        edge_warps<2, float>(P, nullptr, nullptr, P.nmf, wsh[threadIdx.x >> 5], qbuf[threadIdx.x >> 5],
                             reinterpret_cast<float *>(smem));
        return;
    }
    const Seg &sg = P.segs[0].seg;
    bulk_init(&bar);
    if (threadIdx.x == 0) {
        const uint32_t rb = (uint32_t)sizeof(DevRobot);
        const uint32_t rows = (uint32_t)(kFRows * sg.n_pad * sizeof(float));
        bulk_expect(&bar, rb + rows);
        bulk_copy(&bar, smem, sg.robot, rb);
        bulk_copy(&bar, smem + rb, sg.obs_f, rows);
    }
    if (!bulk_wait(&bar, 0, P.status)) return;
    const DevRobot &rb = *reinterpret_cast<const DevRobot *>(smem);
    const float *rows = reinterpret_cast<const float *>(smem + sizeof(DevRobot));
    ObsView<float> ob{rows, rows + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
    if (sg.n_pad <= kAosMaxPad) {   // the per-obstacle copy of the rows (room reserved by the launcher)
        float4 *aos = reinterpret_cast<float4 *>(smem + sizeof(DevRobot) + (size_t)kFRows * sg.n_pad * sizeof(float));
        for (int t = threadIdx.x; t < sg.n; t += kThreads) {
            const int np = sg.n_pad;
            aos[2 * t] = make_float4(rows[t], rows[np + t], rows[2 * np + t], rows[3 * np + t]);
            aos[2 * t + 1] = make_float4(rows[4 * np + t], rows[5 * np + t], rows[kRowTol * np + t],
                                         rows[kRowGround * np + t]);
        }
        __syncthreads();
        ob.aos = aos;
    }
    // the skeleton buffer follows the robot, the rows and their per-obstacle copy
    float *skel = reinterpret_cast<float *>(smem + sizeof(DevRobot) + (size_t)kFRows * sg.n_pad * sizeof(float) +
                                            (sg.n_pad <= kAosMaxPad ? (size_t)sg.n_pad * kFRows * sizeof(float) : 0));
    edge_warps<2, float>(P, &rb, &ob, P.nmf, wsh[threadIdx.x >> 5], qbuf[threadIdx.x >> 5], skel);
}

cudaError_t launch_edges_fp32(const EdgeParams &p, int grid, size_t smem, cudaStream_t st) {
    if (p.nseg_lane == 1 && p.segs[0].seg.n_pad <= kAosMaxPad) smem += (size_t)p.segs[0].seg.n_pad * kFRows * sizeof(float);
    int dmax = 1;   // the skeleton buffer of the order-free driver
    for (int k = 0; k < p.nseg_lane; ++k) dmax = std::max(dmax, (int)p.segs[k].D);
    smem += (size_t)kThreads * 3 * (dmax + 1) * sizeof(float);
    static std::atomic<uint64_t> attr[2] = {{0}, {0}};
    if (p.nseg_lane != 1) {
        ensure_smem_limit(k_edges_fp32<true>, 160 * 1024, attr[1]);
        k_edges_fp32<true><<<grid, kThreads, smem, st>>>(p);
    } else {
        ensure_smem_limit(k_edges_fp32<false>, 160 * 1024, attr[0]);
        k_edges_fp32<false><<<grid, kThreads, smem, st>>>(p);
    }
    return cudaGetLastError();
}

// Failure-detection probe: the staging wait of a CTA whose copy is never
// issued.  Thread 0 announces 16 bytes that no copy delivers, so the bounded
// wait runs out after 'limit' polls, records the timeout in *status and the
// kernel returns; nothing is left in flight.
__global__ void k_wait_probe(int32_t *status, unsigned limit) {
    __shared__ uint64_t bar;
    bulk_init(&bar);
    if (threadIdx.x == 0) bulk_expect(&bar, 16);
    bulk_wait(&bar, 0, status, limit);
}

cudaError_t launch_wait_probe(int32_t *status, unsigned limit, cudaStream_t st) {
    k_wait_probe<<<1, 32, 0, st>>>(status, limit);
    return cudaGetLastError();
}

// Peak FP32 issue rate of this GPU: independent FMA chains, no memory traffic.
__global__ void k_ffma_probe(float *out, int iters) {
    float a[kProbeChains];
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) a[k] = (float)(threadIdx.x + k);
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kProbeChains; ++k) a[k] = fmaf(a[k], m, c);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t launch_ffma_probe(float *out, int blocks, int threads, int iters, cudaStream_t st) {
    k_ffma_probe<<<blocks, threads, 0, st>>>(out, iters);
    return cudaGetLastError();
}

template <int KIND> static cudaError_t launch_fp32_kind(const KParams &p, int64_t blocks, size_t smem, cudaStream_t st) {
    static std::atomic<uint64_t> attr{0};
    ensure_smem_limit(k_check_fp32<KIND>, 200 * 1024, attr);
    k_check_fp32<KIND><<<(unsigned)blocks, kThreads, smem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_check_fp32(const KParams &p, int64_t blocks, size_t smem, cudaStream_t st) {
    bool any_b = false, any_d = false, any_p = false;
    int aos_pad = 0;   // room for the per-obstacle copy of the largest scene that gets one
    for (int k = 0; k < p.nseg; ++k) {
        any_b = any_b || p.segs[k].valid;
        any_d = any_d || p.segs[k].dist;
        any_p = any_p || p.segs[k].profile;
        if (p.segs[k].n_pad <= kAosMaxPad) aos_pad = std::max(aos_pad, p.segs[k].n_pad);
    }
    smem += (size_t)aos_pad * kFRows * sizeof(float);
    const size_t skel = (size_t)kThreads * 3 * p.skel_pts * sizeof(float);   // order-free kinds
    if (!any_d && !any_p) return launch_fp32_kind<1>(p, blocks, smem + skel, st);
    if (!any_b && !any_p) return launch_fp32_kind<3>(p, blocks, smem + skel, st);
    if (!any_b) return launch_fp32_kind<2>(p, blocks, smem, st);
    return launch_fp32_kind<0>(p, blocks, smem, st);
}

// ------------------------------------------------------------- primitive probe --
// The FP32 pass's decisions on single cases: the value in FP32 and whether the
// pass would settle it (every decision margin at least kDecide, and for
// distances the contact-band rule of pair_distance with min_dist_tol =
// MAX_DISTANCE).  Unsettled cases are left to the FP64 recheck.
__global__ void k_probe_fp32(const __grid_constant__ ProbeParams P) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const Num<float> nm = P.nmf;
    float A[3], B[3], X[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) { A[k] = P.a[3 * i + k]; B[k] = P.b[3 * i + k]; }
#pragma unroll
    for (int k = 0; k < 6; ++k) X[k] = P.x[6 * i + k];
    const float r = P.r[i];
    const float rn = (float)((double)r * sqrt(3.0) / 3);
    const int kind = P.kind[i];
    double v;
    uint8_t settled;
    if (kind == 0) {
        // the inlined (isValid-only kernels) and out-of-line rectangle tests must agree
        const RB flat = coll_box_call<float, RobustPol, true>(nm, A, B, r, rn, X);
        const RB call = coll_box_call<float, RobustPol, false>(nm, A, B, r, rn, X);
        v = flat.v ? 1.0 : 0.0;
        settled = (flat.v != call.v || flat.m != call.m) ? 2 : (flat.m >= kDecide ? 1 : 0);
    } else if (kind == 1) {
        const ValM<float> dv = capsule_box_call<float, RobustPol>(nm, A, B, r, X);
        const float tol = nm.maxd;
        float d = dv.v, m = dv.m;
        const float band = dv.ia * (kDecide / kBand);
        m = fminf(m, fabsf(d - tol) * band);
        if (d != 0.f) m = fminf(m, fabsf(d > tol ? nm.maxd : d) * band);
        if (d > tol) d = nm.maxd;
        v = (double)d;
        settled = m >= kDecide ? 1 : 0;
    } else {
        RobustPol pol;
        v = (double)seg_seg(pol, nm, A, B, X, X + 3).v;
        settled = pol.m >= kDecide ? 1 : 0;
    }
    P.value[i] = v;
    P.settled[i] = settled;
}

cudaError_t launch_probe_fp32(const ProbeParams &p, cudaStream_t st) {
    const unsigned grid = (unsigned)((p.n + 127) / 128);
    if (grid == 0) return cudaSuccess;
    k_probe_fp32<<<grid, 128, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace rpm
