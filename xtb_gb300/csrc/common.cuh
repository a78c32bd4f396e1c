// Shared device helpers for the GB300 GFN2-xTB engine (sm_103a, FP64 path).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

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
