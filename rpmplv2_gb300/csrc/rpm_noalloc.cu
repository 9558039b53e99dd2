// rpm_noalloc.cu -- rpm_check_configs_noalloc: the FP32 + FP64-recheck check
// for callers that must not allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- a real-time
// control loop that forbids allocator calls (and their implicit
// synchronisation) after start-up, or a host framework that owns all device
// memory itself and hands out only the buffers it manages.  Such a caller
// already holds its inputs and outputs in device memory; this entry point
// needs nothing else.
//
// Scratch: the FP32 pass lists the configurations it could not settle for the
// FP64 recheck.  Here that list lives in a file-scope static __device__ array
// (g_noalloc_scratch, 65,536 entries plus a counter, about 512 KB), which
// every GPU that loads this library holds until the process exits.  Host code
// cannot use the array's name as a device address, so the first call on each
// device looks the address up with cudaGetSymbolAddress (with that device
// current) and caches it with the device's current context; a call that finds
// another context current (after cudaDeviceReset, or under a context the
// caller made current through the driver API) looks it up again.  Make the
// first call on a device before any stream capture.  Every call shares the one
// array and clears its counter first, so calls that overlap on the GPU
// (different streams, or host threads) race on it and must be serialised by
// the caller.
//
// This translation unit is built with --fmad=false like rpm_exact.cu, so its
// FP64 recheck rounds exactly as the FP64 form does.
#include <cuda.h>   // CUcontext / CUresult types only; the driver is reached through the runtime

#include <mutex>

#include "rpm_check.cuh"
#include "rpm_launch.cuh"

namespace rpm {

constexpr int64_t kNoAllocMaxConfigs = 1 << 16;   // configurations per call
constexpr int kNoAllocMaxDevices = 64;

// [0, kNoAllocMaxConfigs): recheck list; [kNoAllocMaxConfigs]: counter.
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocMaxConfigs + 1];

struct NoAllocParams {
    DevRobot rb;
    const float *aabb;         // [n][6] caller's device array
    const float *tol;          // [n] or nullptr
    const uint8_t *flags;      // [n] or nullptr
    int32_t n, n_pad;
    const float *q;
    int64_t count;
    uint8_t *valid;
    double *dist;
    float *profile;
    Num<float> nmf;
    Num<double> nmd;
    uint64_t *scratch;         // device address of g_noalloc_scratch
};

// Copy the caller's obstacles into shared-memory rows ([8][n_pad] floats, or
// [7][n_pad] doubles plus a float ground row).
template <typename T>
__device__ void stage_rows(const NoAllocParams &P, T *rows, float *ground, float maxd) {
    for (int j = threadIdx.x; j < P.n_pad; j += blockDim.x) {
        const bool in = j < P.n;
#pragma unroll
        for (int k = 0; k < 6; ++k) rows[k * P.n_pad + j] = in ? (T)P.aabb[6 * j + k] : T(0);
        rows[kRowTol * P.n_pad + j] = in ? (T)(P.tol ? P.tol[j] : maxd) : T(0);
        ground[j] = (in && P.flags && (P.flags[j] & RPM_OBS_GROUND)) ? 1.f : 0.f;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kThreads) k_noalloc_fp32(const __grid_constant__ NoAllocParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ WarpShared<float> wsh[kThreads / 32];
    float *rows = reinterpret_cast<float *>(smem);
    stage_rows<float>(P, rows, rows + (size_t)kRowGround * P.n_pad, P.nmf.maxd);
    const int64_t c = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    if (c - (threadIdx.x & 31) >= P.count) return;
    const bool active = c < P.count;
    ObsView<float> ob{rows, rows + (size_t)kRowGround * P.n_pad, P.n, P.n_pad};
    const Want w{P.valid != nullptr, P.dist != nullptr, P.profile != nullptr};
    const int D = P.rb.D;
    const bool ok = warp_check<2, float>(wsh[threadIdx.x >> 5], P.rb, ob, P.q + c * D, active, P.nmf, w,
                                         (w.valid && active) ? P.valid + c : nullptr,
                                         (w.dist && active) ? P.dist + c : nullptr,
                                         (w.profile && active) ? P.profile + c * D : nullptr) == kSettled;
    if (active && !ok) {
        unsigned long long *cnt = reinterpret_cast<unsigned long long *>(&P.scratch[kNoAllocMaxConfigs]);
        const unsigned long long slot = atomicAdd(cnt, 1ull);
        if (slot < (unsigned long long)kNoAllocMaxConfigs) P.scratch[slot] = (uint64_t)c;
    }
}

__global__ void __launch_bounds__(kThreads) k_noalloc_recheck(const __grid_constant__ NoAllocParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    double *rows = reinterpret_cast<double *>(smem);
    float *ground = reinterpret_cast<float *>(smem + (size_t)kDRows * P.n_pad * sizeof(double));
    stage_rows<double>(P, rows, ground, P.nmf.maxd);
    const uint64_t n = P.scratch[kNoAllocMaxConfigs];
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x / 32);
    ObsView<double> ob{rows, ground, P.n, P.n_pad};
    const Want w{P.valid != nullptr, P.dist != nullptr, P.profile != nullptr};
    const int D = P.rb.D;
    for (uint64_t k = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); k < n; k += warps) {
        const int64_t c = (int64_t)P.scratch[k];
        if (c >= P.count) continue;
        config_exact_warp<0, double>(P.rb, ob, P.q + c * D, P.nmd, w, w.valid ? P.valid + c : nullptr,
                                     w.dist ? P.dist + c : nullptr, w.profile ? P.profile + c * D : nullptr);
    }
}

// The calling thread's current driver context (nullptr if none is bound yet),
// through the runtime's driver entry point so the library needs no link
// against the driver.
static void *current_context() {
    typedef CUresult (*CtxGetCurrent)(CUcontext *);
    static std::once_flag once;
    static CtxGetCurrent fn = nullptr;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrent>(f);
    });
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

}  // namespace rpm

using namespace rpm;

extern "C" int rpm_check_configs_noalloc(const rpm_robot_desc *robot, const float *aabb_dev, const float *min_dist_tol_dev,
                                         const uint8_t *flags_dev, int32_t n, const rpm_params *params,
                                         const float *q_dev, int64_t num_configs, uint8_t *valid_dev,
                                         double *dist_dev, float *profile_dev, void *stream) {
    if (!robot || !params) return set_error(RPM_ERR_INVALID, "robot and params are required");
    if (n < 0 || (n > 0 && !aabb_dev)) return set_error(RPM_ERR_INVALID, "bad obstacle array");
    if (num_configs < 0 || (num_configs > 0 && !q_dev)) return set_error(RPM_ERR_INVALID, "bad configuration array");
    if (num_configs > kNoAllocMaxConfigs)
        return set_error(RPM_ERR_RANGE, "rpm_check_configs_noalloc: more than 65536 configurations in one call "
                                        "(its static recheck list holds 65536); split the batch");
    if (n > kMaxObstacles) return set_error(RPM_ERR_RANGE, "rpm_check_configs_noalloc: more than 2048 obstacles");
    NoAllocParams P;
    memset(&P, 0, sizeof P);
    int rc = build_dev_robot(*robot, P.rb);
    if (rc) return rc;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
        return set_error(RPM_ERR_CUDA, "rpm_check_configs_noalloc: no usable current device");
    // once per device (and again if the device's current context changed),
    // with that device current: the array's device address
    static std::mutex mu;
    static uint64_t *addr[kNoAllocMaxDevices] = {nullptr};
    static void *addr_ctx[kNoAllocMaxDevices] = {nullptr};
    {
        std::lock_guard<std::mutex> lk(mu);
        void *cur = current_context();
        if (!addr[dev] || !cur || cur != addr_ctx[dev]) {
            void *p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return set_error(RPM_ERR_CUDA, cudaGetErrorString(e));
            addr[dev] = static_cast<uint64_t *>(p);
            addr_ctx[dev] = current_context();   // bound by the lookup if it was not before
        }
    }
    P.scratch = addr[dev];
    P.aabb = aabb_dev;
    P.tol = min_dist_tol_dev;
    P.flags = flags_dev;
    P.n = n;
    P.n_pad = n < 16 ? 16 : (n + 15) / 16 * 16;
    P.q = q_dev;
    P.count = num_configs;
    P.valid = valid_dev;
    P.dist = dist_dev;
    P.profile = profile_dev;
    P.nmf.eq = (float)params->equality_threshold;
    P.nmf.maxd = (float)params->max_distance;
    P.nmd.eq = params->equality_threshold;
    P.nmd.maxd = params->max_distance;
    cudaStream_t st = (cudaStream_t)stream;
    // the shared array keeps the previous call's contents: clear the counter
    if (cudaMemsetAsync(P.scratch + kNoAllocMaxConfigs, 0, sizeof(uint64_t), st) != cudaSuccess)
        return set_error(RPM_ERR_CUDA, "rpm_check_configs_noalloc: clearing the scratch counter failed");
    if (num_configs == 0) return RPM_OK;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return set_error(RPM_ERR_CUDA, "rpm_check_configs_noalloc: device query failed");
    const size_t smem32 = (size_t)kFRows * P.n_pad * sizeof(float);
    const size_t smem64 = (size_t)kDRows * P.n_pad * sizeof(double) + (size_t)P.n_pad * sizeof(float);
    static std::atomic<uint64_t> attr32{0}, attr64{0};
    ensure_smem_limit(k_noalloc_fp32, 200 * 1024, attr32);
    ensure_smem_limit(k_noalloc_recheck, 200 * 1024, attr64);
    const unsigned blocks = (unsigned)((num_configs + kThreads - 1) / kThreads);
    k_noalloc_fp32<<<blocks, kThreads, smem32, st>>>(P);
    k_noalloc_recheck<<<sms * 2, kThreads, smem64, st>>>(P);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(RPM_ERR_CUDA, cudaGetErrorString(e));
    return RPM_OK;
}
