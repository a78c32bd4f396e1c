// Multipole integrals and their gradient contraction over a batch of molecules.
//
// Same device bodies as the per-molecule kernels (build_SDQH0 and
// build_dSDQH0_noreset, src/xtb/hamiltonian.F90:146-371, 575-792); grid row y is
// molecule y, and the blocks of a row stride over that molecule's shell pairs.
// Kept in their own translation unit: the per-(l_i, l_j) templates dominate
// compile time.
#include <algorithm>

#include "batch.h"
#include "integrals_device.cuh"

namespace xg {

namespace {

constexpr int BI_THREADS = 128;
constexpr int BI_MAX_BLOCKS = 64;   // blocks per molecule row (grid-stride beyond)

template <int LI, int LJ>
__global__ void __launch_bounds__(BI_THREADS) k_batch_sdqh0(BatchMol* __restrict__ mols, int nmol, double intcut) {
    const int mi = blockIdx.y;
    if (mi >= nmol) return;
    BatchMol* b = mols + mi;
    if (b->stage != BS_SETUP) return;
    const long np = class_pairs<LI, LJ>(b->m);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < np; t += (long)gridDim.x * blockDim.x)
        d_sdqh0<LI, LJ>(b->m, b->se, intcut, np, b->S, b->D, b->Q, b->H0, t);
}

template <int LI, int LJ>
__global__ void __launch_bounds__(BI_THREADS) k_batch_grad_sdqh0(BatchMol* __restrict__ mols, int nmol,
                                                                  double intcut) {
    const int mi = blockIdx.y;
    if (mi >= nmol) return;
    BatchMol* b = mols + mi;
    if (b->stage != BS_GRAD || !b->want_grad) return;
    const long np = class_pairs<LI, LJ>(b->m);
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < np; t += (long)gridDim.x * blockDim.x)
        d_grad_sdqh0<LI, LJ>(b->m, b->se, intcut, np, b->P, b->W, b->shift, b->vs, b->vd, b->vq, b->grad, b->dhdcn,
                             t);
}

// one warp per shell pair for the classes with many Cartesian component pairs
template <int LI, int LJ>
__global__ void __launch_bounds__(BI_THREADS) k_batch_sdqh0_w(BatchMol* __restrict__ mols, int nmol, double intcut) {
    constexpr int NW = BI_THREADS / 32;
    __shared__ double sm[NW][WarpInt<LI, LJ>::SMEM];
    const int mi = blockIdx.y;
    if (mi >= nmol) return;
    BatchMol* b = mols + mi;
    if (b->stage != BS_SETUP) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long np = class_pairs<LI, LJ>(b->m);
    for (long t = (long)blockIdx.x * NW + w; t < np; t += (long)gridDim.x * NW)
        d_sdqh0_warp<LI, LJ>(b->m, b->se, intcut, b->S, b->D, b->Q, b->H0, t, lane, sm[w]);
}

template <int LI, int LJ>
__global__ void __launch_bounds__(BI_THREADS) k_batch_grad_sdqh0_w(BatchMol* __restrict__ mols, int nmol,
                                                                    double intcut) {
    constexpr int NW = BI_THREADS / 32;
    __shared__ double sm[NW][WarpInt<LI, LJ>::SMEM];
    const int mi = blockIdx.y;
    if (mi >= nmol) return;
    BatchMol* b = mols + mi;
    if (b->stage != BS_GRAD || !b->want_grad) return;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long np = class_pairs<LI, LJ>(b->m);
    for (long t = (long)blockIdx.x * NW + w; t < np; t += (long)gridDim.x * NW)
        d_grad_sdqh0_warp<LI, LJ>(b->m, b->se, intcut, b->P, b->W, b->shift, b->vs, b->vd, b->vq, b->grad, b->dhdcn, t,
                                  lane, sm[w]);
}

dim3 batch_grid(int nmol, int max_nsh) {
    const long np = (long)max_nsh * (max_nsh + 1) / 2;
    const int bx = (int)std::min<long>(BI_MAX_BLOCKS, std::max<long>(1, (np + BI_THREADS - 1) / BI_THREADS));
    return dim3(bx, nmol);
}

// blocks per molecule row for the warp-per-pair kernels (a warp takes a pair)
dim3 batch_grid_warps(int nmol, int max_nsh) {
    const long np = (long)max_nsh * (max_nsh + 1) / 2;
    const int bx = (int)std::min<long>(BI_MAX_BLOCKS, std::max<long>(1, (np + BI_THREADS / 32 - 1) / (BI_THREADS / 32)));
    return dim3(bx, nmol);
}

}  // namespace

void batch_integrals(cudaStream_t st, BatchMol* mols, int nmol, int max_nsh, double intcut) {
    if (nmol <= 0) return;
    if (nmol > 65535) throw CudaError("batch_integrals: too many molecules for one grid");
    const dim3 g = batch_grid(nmol, max_nsh), gw = batch_grid_warps(nmol, max_nsh);
    k_batch_sdqh0<0, 0><<<g, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_sdqh0<1, 0><<<g, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_sdqh0_w<1, 1><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_sdqh0_w<2, 0><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_sdqh0_w<2, 1><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_sdqh0_w<2, 2><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
}

void batch_integral_gradient(cudaStream_t st, BatchMol* mols, int nmol, int max_nsh, double intcut) {
    if (nmol <= 0) return;
    if (nmol > 65535) throw CudaError("batch_integral_gradient: too many molecules for one grid");
    const dim3 g = batch_grid(nmol, max_nsh), gw = batch_grid_warps(nmol, max_nsh);
    k_batch_grad_sdqh0<0, 0><<<g, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_grad_sdqh0<1, 0><<<g, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_grad_sdqh0_w<1, 1><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_grad_sdqh0_w<2, 0><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_grad_sdqh0_w<2, 1><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
    k_batch_grad_sdqh0_w<2, 2><<<gw, BI_THREADS, 0, st>>>(mols, nmol, intcut);
    XG_LAUNCH_CHECK();
}

}  // namespace xg
