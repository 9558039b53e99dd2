// rpm_fast.cu -- the FP32 bulk pass of the FP32 + FP64-recheck form.  Every
// decision of both trees carries a margin; configurations whose outputs
// depended on a decision within kBand of its boundary are appended to the
// recheck list and recomputed in FP64 by k_recheck (rpm_exact.cu).
#include "rpm_check.cuh"
#include "rpm_launch.cuh"

namespace rpm {

__global__ void __launch_bounds__(kThreads) k_check_fp32(const __grid_constant__ KParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
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
    const int64_t c = (int64_t)(blockIdx.x - sg.first_block) * kThreads + threadIdx.x;
    if (c >= sg.count) return;
    ObsView<float> ob{rows, rows + (size_t)kRowGround * sg.n_pad, sg.n, sg.n_pad};
    const Want w{sg.valid != nullptr, sg.dist != nullptr, sg.profile != nullptr};
    const int D = rb.D;
    const bool ok = config_fp32(rb, ob, sg.q + c * D, P.nmf, w, w.valid ? sg.valid + c : nullptr,
                                w.dist ? sg.dist + c : nullptr, w.profile ? sg.profile + c * D : nullptr);
    if (!ok) {
        const uint32_t slot = atomicAdd(P.recheck_count, 1u);
        P.recheck[slot] = ((uint64_t)s << 40) | (uint64_t)c;
    }
}

cudaError_t launch_check_fp32(const KParams &p, int64_t blocks, size_t smem, cudaStream_t st) {
    static bool attr = false;
    if (!attr) { cudaFuncSetAttribute(k_check_fp32, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); attr = true; }
    k_check_fp32<<<(unsigned)blocks, kThreads, smem, st>>>(p);
    return cudaGetLastError();
}

}  // namespace rpm
