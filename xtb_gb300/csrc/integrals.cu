// GFN2-xTB multipole integrals and their fused gradient contraction (FP64, sm_103a).
//
// Split from the other GFN2 kernels so that the heavily unrolled per-(l_i, l_j)
// templates compile in their own translation unit.
#include <algorithm>
#include <cmath>

#include "gfn2_kernels.h"
#include "integrals_device.cuh"

namespace xg {


template <int LI, int LJ>
__global__ void k_sdqh0(DevMol m, const double* __restrict__ se, double intcut, long npairs,
                                               double* __restrict__ S, double* __restrict__ D, double* __restrict__ Q,
                                               double* __restrict__ H0) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= class_pairs<LI, LJ>(m)) return;
    d_sdqh0<LI, LJ>(m, se, intcut, npairs, S, D, Q, H0, t);
}


// one warp per shell pair (classes with many Cartesian component pairs)
constexpr int WI_WARPS = 4;
constexpr int WI_MAX_BLOCKS = 4096;

template <int LI, int LJ>
__global__ void __launch_bounds__(32 * WI_WARPS) k_sdqh0_w(DevMol m, const double* __restrict__ se, double intcut,
                                                          long npairs, double* __restrict__ S, double* __restrict__ D,
                                                          double* __restrict__ Q, double* __restrict__ H0) {
    __shared__ double sm[WI_WARPS][WarpInt<LI, LJ>::SMEM];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long np = class_pairs<LI, LJ>(m);
    for (long t = (long)blockIdx.x * WI_WARPS + w; t < np; t += (long)gridDim.x * WI_WARPS)
        d_sdqh0_warp<LI, LJ>(m, se, intcut, S, D, Q, H0, t, lane, sm[w]);
}

template <int LI, int LJ>
__global__ void __launch_bounds__(32 * WI_WARPS) k_grad_sdqh0_w(DevMol m, const double* __restrict__ se, double intcut,
                                                               long npairs, const double* __restrict__ P,
                                                               const double* __restrict__ Pew,
                                                               const double* __restrict__ shift,
                                                               const double* __restrict__ vs,
                                                               const double* __restrict__ vd,
                                                               const double* __restrict__ vq, double* __restrict__ grad,
                                                               double* __restrict__ dhdcn) {
    __shared__ double sm[WI_WARPS][WarpInt<LI, LJ>::SMEM];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long np = class_pairs<LI, LJ>(m);
    for (long t = (long)blockIdx.x * WI_WARPS + w; t < np; t += (long)gridDim.x * WI_WARPS)
        d_grad_sdqh0_warp<LI, LJ>(m, se, intcut, P, Pew, shift, vs, vd, vq, grad, dhdcn, t, lane, sm[w]);
}

void build_sdqh0(cudaStream_t st, const DevMol& m, const double* se, Thresholds th, double* S, double* D, double* Q,
                 double* H0) {
    const size_t nn = (size_t)m.nao * m.nao;
    XG_CUDA(cudaMemsetAsync(S, 0, nn * sizeof(double), st));
    XG_CUDA(cudaMemsetAsync(H0, 0, nn * sizeof(double), st));
    XG_CUDA(cudaMemsetAsync(D, 0, 3 * nn * sizeof(double), st));
    XG_CUDA(cudaMemsetAsync(Q, 0, 6 * nn * sizeof(double), st));
    const long np = (long)m.nsh * (m.nsh + 1) / 2;
    // s-s and p-s pairs: one thread per pair; the others: one warp per pair; each class walks
    // only its own pairs
    auto nb = [](long c) { return ceil_div(c, 128); };
    auto nw = [](long c) { return (int)std::min<long>(WI_MAX_BLOCKS, ceil_div(c, WI_WARPS)); };
    long c;
    if ((c = class_pairs<0, 0>(m)) > 0) { k_sdqh0<0, 0><<<nb(c), 128, 0, st>>>(m, se, th.intcut, np, S, D, Q, H0); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<1, 0>(m)) > 0) { k_sdqh0<1, 0><<<nb(c), 128, 0, st>>>(m, se, th.intcut, np, S, D, Q, H0); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<1, 1>(m)) > 0) { k_sdqh0_w<1, 1><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, S, D, Q, H0); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<2, 0>(m)) > 0) { k_sdqh0_w<2, 0><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, S, D, Q, H0); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<2, 1>(m)) > 0) { k_sdqh0_w<2, 1><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, S, D, Q, H0); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<2, 2>(m)) > 0) { k_sdqh0_w<2, 2><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, S, D, Q, H0); XG_LAUNCH_CHECK(); }
}


template <int LI, int LJ>
__global__ void k_grad_sdqh0(DevMol m, const double* __restrict__ se, double intcut, long npairs,
                                                    const double* __restrict__ P, const double* __restrict__ Pew,
                                                    const double* __restrict__ shift, const double* __restrict__ vs,
                                                    const double* __restrict__ vd, const double* __restrict__ vq,
                                                    double* __restrict__ grad, double* __restrict__ dhdcn) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= class_pairs<LI, LJ>(m)) return;
    d_grad_sdqh0<LI, LJ>(m, se, intcut, npairs, P, Pew, shift, vs, vd, vq, grad, dhdcn, t);
}


void grad_sdqh0(cudaStream_t st, const DevMol& m, Thresholds th, const double* se, const double* P, const double* Pew,
                const double* shift, const double* vs, const double* vd, const double* vq, double* grad,
                double* dhdcn) {
    const long np = (long)m.nsh * (m.nsh + 1) / 2;
    auto nb = [](long c) { return ceil_div(c, 128); };
    auto nw = [](long c) { return (int)std::min<long>(WI_MAX_BLOCKS, ceil_div(c, WI_WARPS)); };
    long c;
    if ((c = class_pairs<0, 0>(m)) > 0) { k_grad_sdqh0<0, 0><<<nb(c), 128, 0, st>>>(m, se, th.intcut, np, P, Pew, shift, vs, vd, vq, grad, dhdcn); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<1, 0>(m)) > 0) { k_grad_sdqh0<1, 0><<<nb(c), 128, 0, st>>>(m, se, th.intcut, np, P, Pew, shift, vs, vd, vq, grad, dhdcn); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<1, 1>(m)) > 0) { k_grad_sdqh0_w<1, 1><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, P, Pew, shift, vs, vd, vq, grad, dhdcn); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<2, 0>(m)) > 0) { k_grad_sdqh0_w<2, 0><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, P, Pew, shift, vs, vd, vq, grad, dhdcn); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<2, 1>(m)) > 0) { k_grad_sdqh0_w<2, 1><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, P, Pew, shift, vs, vd, vq, grad, dhdcn); XG_LAUNCH_CHECK(); }
    if ((c = class_pairs<2, 2>(m)) > 0) { k_grad_sdqh0_w<2, 2><<<nw(c), 32 * WI_WARPS, 0, st>>>(m, se, th.intcut, np, P, Pew, shift, vs, vd, vq, grad, dhdcn); XG_LAUNCH_CHECK(); }
}


}  // namespace xg
