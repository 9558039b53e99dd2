// rpm_exact.cu -- exact forms: FP64 ("plain form"), the reference's own FP32
// numerics, and the FP64 recheck of configurations the FP32 pass could not
// settle.  Built with --fmad=false: no multiply-add is contracted, so every
// operation rounds as the CPU restatement's does.
#include <type_traits>

#include "rpm_check.cuh"
#include "rpm_launch.cuh"

namespace rpm {

size_t smem_bytes(int mode, int n_pad) {
    size_t rb = sizeof(DevRobot);
    if (mode == RPM_PREC_FP64) return rb + (size_t)kDRows * n_pad * sizeof(double) + (size_t)n_pad * sizeof(float);
    return rb + (size_t)kFRows * n_pad * sizeof(float);
}

// Stage the segment's robot and obstacle rows in shared memory (bulk async
// copies on one mbarrier).  Returns false if the bounded wait gave up.
template <int MODE>
__device__ __forceinline__ bool stage(const Seg &sg, unsigned char *smem, uint64_t *bar, int32_t *status) {
    if (threadIdx.x == 0) {
        const uint32_t rb = (uint32_t)sizeof(DevRobot);
        if (MODE == 0) {
            const uint32_t rows = (uint32_t)(kDRows * sg.n_pad * sizeof(double));
            const uint32_t gnd = (uint32_t)(sg.n_pad * sizeof(float));
            bulk_expect(bar, rb + rows + gnd);
            bulk_copy(bar, smem, sg.robot, rb);
            bulk_copy(bar, smem + rb, sg.obs_d, rows);
            bulk_copy(bar, smem + rb + rows, sg.obs_f + (size_t)kRowGround * sg.n_pad, gnd);
        } else {
            const uint32_t rows = (uint32_t)(kFRows * sg.n_pad * sizeof(float));
            bulk_expect(bar, rb + rows);
            bulk_copy(bar, smem, sg.robot, rb);
            bulk_copy(bar, smem + rb, sg.obs_f, rows);
        }
    }
    return bulk_wait(bar, 0, status);
}

__device__ __forceinline__ int find_seg(const KParams &P) {
    int k = 0;
    while (k + 1 < P.nseg && P.segs[k + 1].first_block <= (int64_t)blockIdx.x) ++k;
    return k;
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_check_exact(const __grid_constant__ KParams P) {
    typedef typename std::conditional<MODE == 0, double, float>::type T;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    __shared__ WarpShared<T> wsh[kThreads / 32];
    const int s = find_seg(P);
    const Seg &sg = P.segs[s];
    bulk_init(&bar);
    if (!stage<MODE>(sg, smem, &bar, P.status)) return;
    const DevRobot &rb = *reinterpret_cast<const DevRobot *>(smem);
    const T *rows = reinterpret_cast<const T *>(smem + sizeof(DevRobot));
    const float *ground = (MODE == 0) ? reinterpret_cast<const float *>(smem + sizeof(DevRobot) + kDRows * sg.n_pad * sizeof(double))
                                      : reinterpret_cast<const float *>(rows) + (size_t)kRowGround * sg.n_pad;
    const int64_t c = (int64_t)(blockIdx.x - sg.first_block) * kThreads + threadIdx.x;
    const int64_t warp0 = c - (threadIdx.x & 31);
    if (warp0 >= sg.count) return;   // whole warp idle
    const bool active = c < sg.count;
    ObsView<T> ob{rows, ground, sg.n, sg.n_pad};
    const Want w{sg.valid != nullptr, sg.dist != nullptr, sg.profile != nullptr};
    const int D = rb.D;
    Num<T> nm;
    if (MODE == 0) { nm.eq = (T)P.nmd.eq; nm.maxd = (T)P.nmd.maxd; }
    else { nm.eq = (T)P.nmf.eq; nm.maxd = (T)P.nmf.maxd; }
    warp_check<MODE, T>(wsh[threadIdx.x >> 5], rb, ob, sg.q + c * D, active, nm, w,
                        (w.valid && active) ? sg.valid + c : nullptr, (w.dist && active) ? sg.dist + c : nullptr,
                        (w.profile && active) ? sg.profile + c * D : nullptr);
}

// FP64 recomputation of the configurations listed by the FP32 pass, one warp
// per configuration.  Reads robot and obstacles from global memory (the list
// mixes segments).
__global__ void __launch_bounds__(kThreads) k_recheck(const __grid_constant__ KParams P) {
    const uint32_t n = *P.recheck_count;
    const uint32_t warps = gridDim.x * (blockDim.x / 32);
    for (uint32_t k = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); k < n; k += warps) {
        const uint64_t e = P.recheck[k];
        const int s = (int)(e >> 40);
        const int64_t c = (int64_t)(e & ((1ull << 40) - 1));
        if (s >= P.nseg) continue;
        const Seg &sg = P.segs[s];
        if (c >= sg.count) continue;
        ObsView<double> ob{sg.obs_d, sg.obs_f + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
        const Want w{sg.valid != nullptr, sg.dist != nullptr, sg.profile != nullptr};
        const int D = sg.robot->D;
        config_exact_warp<0, double>(*sg.robot, ob, sg.q + c * D, P.nmd, w, w.valid ? sg.valid + c : nullptr,
                                     w.dist ? sg.dist + c : nullptr, w.profile ? sg.profile + c * D : nullptr);
    }
}

// Skeleton points of each configuration (computeSkeleton), widened to double:
// MODE 0 FP64, MODE 1 the reference's float skeleton, MODE 2 the FP32 FK of
// the FP32 bulk pass.
template <int MODE>
__global__ void k_skeleton(const DevRobot *rbp, const float *q, int64_t C, double *out) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const DevRobot &rb = *rbp;
    const int D = rb.D;
    SkelWalker<MODE> sw;
    sw.begin();
    for (int k = 0; k <= D; ++k) {
        if constexpr (MODE == 0) {
            double p[3];
            sw.point(rb, q + c * D, k, p);
            for (int i = 0; i < 3; ++i) out[(c * (D + 1) + k) * 3 + i] = p[i];
        } else {
            float p[3];
            sw.point(rb, q + c * D, k, p);
            for (int i = 0; i < 3; ++i) out[(c * (D + 1) + k) * 3 + i] = (double)p[i];
        }
    }
}

cudaError_t launch_check_exact(int mode, const KParams &p, int64_t blocks, size_t smem, cudaStream_t st) {
    if (mode == RPM_PREC_FP64) {
        static bool attr = false;
        if (!attr) { cudaFuncSetAttribute(k_check_exact<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); attr = true; }
        k_check_exact<0><<<(unsigned)blocks, kThreads, smem, st>>>(p);
    } else {
        static bool attr = false;
        if (!attr) { cudaFuncSetAttribute(k_check_exact<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); attr = true; }
        k_check_exact<1><<<(unsigned)blocks, kThreads, smem, st>>>(p);
    }
    return cudaGetLastError();
}

cudaError_t launch_recheck(const KParams &p, int grid, cudaStream_t st) {
    k_recheck<<<grid, kThreads, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_skeleton(int mode, const DevRobot *rb, int D, const float *q, int64_t C, double *out, cudaStream_t st) {
    (void)D;
    const unsigned grid = (unsigned)((C + 127) / 128);
    if (grid == 0) return cudaSuccess;
    if (mode == RPM_PREC_FP64) k_skeleton<0><<<grid, 128, 0, st>>>(rb, q, C, out);
    else if (mode == RPM_PREC_FP32_REF) k_skeleton<1><<<grid, 128, 0, st>>>(rb, q, C, out);
    else k_skeleton<2><<<grid, 128, 0, st>>>(rb, q, C, out);
    return cudaGetLastError();
}

}  // namespace rpm
