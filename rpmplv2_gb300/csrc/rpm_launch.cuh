// rpm_launch.cuh -- kernel parameter block and host-side launchers.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

#include "rpm_dev.cuh"
#include "rpm_check.cuh"
#include "rpm_tree.cuh"

namespace rpm {

constexpr int kThreads = 128;     // configurations per CTA
constexpr int kMaxSegs = 32;      // segments per launch (passed by value)

// Raise a kernel's dynamic shared-memory limit once per device.  'done'
// holds one bit per device (the attribute belongs to the device's context);
// concurrent callers may both set it, which is harmless.
template <typename K>
inline void ensure_smem_limit(K kernel, int bytes, std::atomic<uint64_t> &done) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    const uint64_t bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess)
        done.fetch_or(bit, std::memory_order_acq_rel);
}

struct KParams {
    Seg segs[kMaxSegs];
    int32_t nseg;
    int32_t wide_g;             // warp-per-configuration kernels: configurations per warp
    int32_t skel_pts;           // FP32 lane kernels: the most skeleton points (D + 1) of the launch's robots
    int32_t pad;
    Num<double> nmd;
    Num<float> nmf;
    uint64_t *recheck;          // FP32 pass -> whole-configuration FP64 recheck: (segment << 40) | config
    uint32_t *recheck_count;
    int32_t *status;
    PairSink ps;                // FP32 pass -> pair-level FP64 recheck
};

#ifdef __CUDACC__
// A configuration the FP32 pass could not settle through the pair recheck:
// recompute it whole in FP64 (the list holds every configuration of a launch).
__device__ __forceinline__ void recheck_whole(const KParams &P, int seg, int64_t c) {
    const uint32_t r = atomicAdd(P.recheck_count, 1u);
    P.recheck[r] = ((uint64_t)(seg + P.ps.seg_base) << 40) | (uint64_t)c;
}
#endif

// Host helpers shared by the C ABI translation units (rpm_api.cu).
int build_dev_robot(const rpm_robot_desc &d, DevRobot &r);   // RPM_OK or an error code (message set)
int set_error(int code, const char *msg);                     // records the thread's error string

// Dynamic shared memory of one CTA: robot + obstacle rows of its scene.
size_t smem_bytes(int mode, int n_pad);

cudaError_t launch_check_exact(int mode, const KParams &p, int64_t blocks, size_t smem, cudaStream_t st);
cudaError_t launch_check_fp32(const KParams &p, int64_t blocks, size_t smem, cudaStream_t st);
// Check order of a large batch for the FP32 lane kernel: configurations binned
// by their first three joint angles (16 bins each over [-pi, pi]) with a
// counting sort; bins needs 2 * kConfigBins ints, perm C ints.
constexpr int kConfigBins = 4096;
constexpr int64_t kBinMinConfigs = 2048;      // smaller batches keep the index order
constexpr int64_t kBinSmallConfigs = 16384;   // up to this many: one CTA sorts them (one launch)
cudaError_t launch_bin_configs(const float *q, int64_t C, int D, int32_t *bins, int32_t *perm, cudaStream_t st);
cudaError_t launch_recheck(const KParams &p, int grid, cudaStream_t st);
// Pair-level FP64 recheck: FK of the recorded configurations, their listed
// pairs, and the fold into the outputs.
cudaError_t launch_pair_recheck(const KParams &p, int grid, cudaStream_t st);
// Warp-per-configuration form over the sorted scene copy (rpm_wide.cuh).
size_t wide_smem_bytes(int mode, int ns, int nb);
cudaError_t launch_check_wide(int mode, const KParams &p, int64_t blocks, size_t smem, cudaStream_t st);
cudaError_t launch_check_wide_fp32(const KParams &p, int64_t blocks, size_t smem, cudaStream_t st);
// FP32 FFMA throughput probe: kProbeChains independent FMA chains per thread.
constexpr int kProbeChains = 8;
cudaError_t launch_ffma_probe(float *out, int blocks, int threads, int iters, cudaStream_t st);
cudaError_t launch_skeleton(int mode, const DevRobot *rb, int D, const float *q, int64_t C, double *out, cudaStream_t st);

cudaError_t launch_wait_probe(int32_t *status, unsigned limit, cudaStream_t st);

// Primitive probe: the device trees on single (segment, box) or (segment,
// segment) cases.  kind[i]: 0 collisionCapsuleToBox, 1 distanceCapsuleToBox,
// 2 distanceLineSegToLineSeg.  x holds the AABB (kinds 0, 1) or C, D (kind 2).
struct ProbeParams {
    const int32_t *kind;
    const float *a, *b, *x, *r;
    int64_t n;
    Num<double> nmd;
    Num<float> nmf;
    double *value;
    uint8_t *settled;   // FP32 pass: 1 settled, 0 left to the FP64 recheck, 2 tree variants disagree
};
// MODE 0: FP64 trees (with only_unsettled, only where settled[i] == 0, as
// the FP64 recheck does); MODE 1: the reference's FP32 numerics.
cudaError_t launch_probe_exact(int mode, const ProbeParams &p, bool only_unsettled, cudaStream_t st);
// The FP32 pass's trees with margins (contracted multiply-adds, as the bulk
// kernels are compiled).
cudaError_t launch_probe_fp32(const ProbeParams &p, cudaStream_t st);

}  // namespace rpm
