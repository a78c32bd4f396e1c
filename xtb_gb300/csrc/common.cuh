// Shared device helpers for the GB300 GFN2-xTB engine (sm_103a, FP64 path).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <set>
#include <stdexcept>
#include <string>
#include <utility>

namespace xg {

struct CudaError : std::runtime_error {
    explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

#define XG_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            throw ::xg::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));     \
    } while (0)

// Allow `kernel` the device's largest opt-in dynamic shared memory, once per device.  The
// limit is a process-wide property of the function: setting it before each launch to that
// launch's own size races with host threads that launch the same kernel with a larger size
// (a launch that falls between the other thread's two calls fails), so every launcher sets
// the same, largest value.
inline void allow_max_dynamic_smem(const void* kernel) {
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    XG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (done.count({kernel, dev})) return;
    int mx = 0;
    XG_CUDA(cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    XG_CUDA(cudaFuncGetAttributes(&fa, kernel));
    XG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - (int)fa.sharedSizeBytes));
    done.insert({kernel, dev});
}

// kernel launches issued by this thread (every launch is followed by XG_LAUNCH_CHECK)
long long& launch_counter();
#define XG_LAUNCH_CHECK()                    \
    do {                                     \
        ++::xg::launch_counter();            \
        XG_CUDA(cudaGetLastError());         \
    } while (0)

// physical constants of the reference (src/mctc/convert.f90:25-29, src/mctc/mctc_constants.f90:22-34)
constexpr double AUTOAA = 0.52917726;
constexpr double AUTOEV = 27.21138505;
constexpr double EVTOAU = 1.0 / AUTOEV;
constexpr double KB_AU = 3.166808578545117e-06;
constexpr double PI = 3.1415926535897932384626433832795029;

#if defined(__CUDACC__)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum; every thread receives the result.  `red` needs blockDim.x/32 doubles.
// 1/x from the FP32 reciprocal and one third-order Newton step for the reciprocal,
// y = y0 (1 + e + e^2) with e = 1 - x y0: a seed of relative error d leaves d^3 + rounding,
// and d <= 2^-23 here, so the result is within about one ulp of 1/x at roughly a third of
// the dependent latency of an FP64 division.  Outside [2^-120, 2^120] the FP32 seed would
// leave the normal range, so the division is used there.
__device__ __forceinline__ double rcp_fast(double x) {
    const int ex = (__double2hiint(x) >> 20) & 0x7ff;
    if (ex > 1023 - 120 && ex < 1023 + 120) {
        const double y0 = (double)__frcp_rn((float)x);
        const double e = fma(-x, y0, 1.0);
        return fma(y0, fma(e, e, e), y0);
    }
    return 1.0 / x;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double t = 0.0;
    for (int k = 0; k < nw; ++k) t += red[k];
    return t;
}

#endif  // __CUDACC__

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

}  // namespace xg
