// Allocation-free repulsion energy and gradient (device-resident inputs and outputs).
//
// A variant of the per-molecule repulsion kernel (repulsionEnGrad_latp,
// src/xtb/repulsion.F90:41-158) whose scratch -- the per-atom energies and the
// completion counter of the in-kernel reduction -- lives in one file-scope
// static device array instead of the engine's workspace.  The element tables
// travel as a by-value kernel argument, so a call needs no device allocation and
// no host<->device copy: one cudaMemsetAsync of the counter and one launch on the
// caller's stream.  The first call on each device looks up the scratch address
// with cudaGetSymbolAddress (which also loads the module); that first call should
// come before any stream capture.  Calls that overlap in time (on different
// streams or host threads) share the scratch and race.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace xg {
namespace {

#include "gfn2_params.inc"

constexpr int NOALLOC_MAX_ATOMS = 8192;   // scratch bound: 64 KiB of per-atom energies
constexpr int NOALLOC_BLOCK = 512;        // same width as the engine's energy reduction
constexpr int MAX_DEVICES = 64;

struct RepScratch {
    double e_atom[NOALLOC_MAX_ATOMS];
    unsigned int done;                    // blocks finished; must be 0 at launch
};

static __device__ __align__(256) RepScratch g_rep_scratch;

struct RepTables {
    double alpha[86];
    double zeff[86];
};

RepTables make_tables() {
    RepTables t;
    for (int i = 0; i < 86; ++i) {
        t.alpha[i] = k_repAlpha[i];
        t.zeff[i] = k_repZeff[i];
    }
    return t;
}

// Thread per atom (the engine's kernel runs a warp per atom with a warp reduction and forms
// r^1.5 as r sqrt(r); this one loops over the pairs serially and calls pow), so the two agree to
// rounding, not bit for bit.  The last block to finish sums the per-atom energies in atom order.
__global__ void __launch_bounds__(NOALLOC_BLOCK)
    k_repulsion_noalloc(int nat, const int* __restrict__ Z, const double* __restrict__ xyz, RepTables tab,
                        RepScratch* __restrict__ sc, double* __restrict__ energy, double* __restrict__ grad) {
    __shared__ double red[32];
    __shared__ bool last;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < nat) {
        const int za = Z[a];
        const bool ok_a = za >= 1 && za <= 86;
        double e = 0.0, g[3] = {0.0, 0.0, 0.0};
        for (int b = 0; b < nat && ok_a; ++b) {
            if (b == a) continue;
            const int zb = Z[b];
            if (zb < 1 || zb > 86) { e = nan(""); break; }
            const double rij[3] = {xyz[3 * a] - xyz[3 * b], xyz[3 * a + 1] - xyz[3 * b + 1],
                                   xyz[3 * a + 2] - xyz[3 * b + 2]};
            const double r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
            if (r2 > 1600.0 || r2 < 1e-8) continue;
            const double r1 = sqrt(r2);
            const double alpha = sqrt(tab.alpha[za - 1] * tab.alpha[zb - 1]);
            const double zeff = tab.zeff[za - 1] * tab.zeff[zb - 1];
            const double kexp = (za > 2 || zb > 2) ? 1.5 : 1.0;
            const double t16 = pow(r1, kexp);
            const double t26 = exp(-alpha * t16);
            const double dE = zeff * t26 / r1;
            const double f = -(alpha * t16 * kexp + 1.0) * dE / r2;
            e += 0.5 * dE;
            for (int k = 0; k < 3; ++k) g[k] += f * rij[k];
        }
        if (!ok_a) e = nan("");
        sc->e_atom[a] = e;
        for (int k = 0; k < 3; ++k) grad[3 * a + k] = g[k];
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&sc->done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    for (int i = threadIdx.x; i < nat; i += blockDim.x) s += __ldcg(&sc->e_atom[i]);
    s = block_sum(s, red);
    if (threadIdx.x == 0) {
        *energy = s;
        sc->done = 0u;
    }
}

std::mutex g_setup_mutex;
RepScratch* g_scratch_ptr[MAX_DEVICES] = {};

int report(char* errbuf, int errlen, int code, const char* msg) {
    if (errbuf && errlen > 0) {
        std::strncpy(errbuf, msg, (size_t)errlen - 1);
        errbuf[errlen - 1] = '\0';
    }
    return code;
}

}  // namespace
}  // namespace xg

extern "C" int xtbgb_repulsionNoAlloc(int natoms, const int* numbers, const double* positions, double* energy,
                                      double* gradient, void* stream, char* errbuf, int errlen) {
    using namespace xg;
    if (errbuf && errlen > 0) errbuf[0] = '\0';
    if (natoms < 1 || natoms > NOALLOC_MAX_ATOMS) {
        char msg[128];
        std::snprintf(msg, sizeof msg, "xtbgb_repulsionNoAlloc: natoms = %d outside 1..%d (static scratch bound)",
                      natoms, NOALLOC_MAX_ATOMS);
        return report(errbuf, errlen, 1, msg);
    }
    if (!numbers || !positions || !energy || !gradient)
        return report(errbuf, errlen, 2, "xtbgb_repulsionNoAlloc: null device pointer");
    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) return report(errbuf, errlen, 3, cudaGetErrorString(rc));
    if (dev < 0 || dev >= MAX_DEVICES) return report(errbuf, errlen, 3, "xtbgb_repulsionNoAlloc: device index");
    RepScratch* sc;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            rc = cudaGetSymbolAddress(&p, g_rep_scratch);
            if (rc != cudaSuccess) return report(errbuf, errlen, 3, cudaGetErrorString(rc));
            g_scratch_ptr[dev] = static_cast<RepScratch*>(p);
        }
        sc = g_scratch_ptr[dev];
    }
    static const RepTables tables = make_tables();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rc = cudaMemsetAsync(&sc->done, 0, sizeof(unsigned int), st);
    if (rc != cudaSuccess) return report(errbuf, errlen, 3, cudaGetErrorString(rc));
    const int blocks = (natoms + NOALLOC_BLOCK - 1) / NOALLOC_BLOCK;
    k_repulsion_noalloc<<<blocks, NOALLOC_BLOCK, 0, st>>>(natoms, numbers, positions, tables, sc, energy, gradient);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) return report(errbuf, errlen, 3, cudaGetErrorString(rc));
    return 0;
}
