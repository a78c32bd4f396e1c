// The engine's autotuner: measures on the current device where the two size-dependent kernel
// choices of the single point cross over (see tune.h), with CUDA events on a private stream.
#include "tune.h"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>

#include "linalg.h"
#include "splitgemm.h"

namespace xg {

namespace {

constexpr int TUNE_MAXDEV = 16;
Tuned g_tuned[TUNE_MAXDEV];
std::mutex g_tune_mu;

int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= TUNE_MAXDEV) return 0;
    return d;
}

// symmetric n x n matrix (row stride n) with pseudo-random entries in (-1, 1)
__global__ void k_tune_sym(int n, unsigned seed, double* __restrict__ A) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)n * n) return;
    int i = (int)(t / n), j = (int)(t % n);
    const int a = max(i, j), b = min(i, j);
    unsigned long long h = ((unsigned long long)a * 0x9E3779B97F4A7C15ull) ^ ((unsigned long long)b << 21) ^ seed;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    A[t] = (double)(h >> 11) * 0x1p-52 - 1.0;
}

// best of `reps` timed runs of f after one warm-up (ms)
template <typename F>
double best_ms(cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, int reps, F&& f) {
    f();
    double best = 1e30;
    for (int r = 0; r < reps; ++r) {
        XG_CUDA(cudaEventRecord(e0, st));
        f();
        XG_CUDA(cudaEventRecord(e1, st));
        XG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        XG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = std::min(best, (double)ms);
    }
    return best;
}

// out[0] = max |A - B|, out[1] = max |A| over rows < n, columns < nc (row stride n); non-negative
// doubles order like their bit patterns
__global__ void k_tune_maxdiff(int n, int nc, const double* __restrict__ A, const double* __restrict__ B,
                               unsigned long long* __restrict__ out) {
    double md = 0.0, ma = 0.0;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < (long)n * nc; t += (long)gridDim.x * blockDim.x) {
        const size_t o = (size_t)(t / nc) * n + (size_t)(t % nc);
        md = fmax(md, fabs(A[o] - B[o]));
        ma = fmax(ma, fabs(A[o]));
    }
    atomicMax(&out[0], (unsigned long long)__double_as_longlong(md));
    atomicMax(&out[1], (unsigned long long)__double_as_longlong(ma));
}

// smallest tested size from which `fast` wins at every larger tested size (INT_MAX: never)
int crossover(const std::vector<int>& sizes, const std::vector<bool>& wins) {
    int at = 1 << 30;
    for (int k = (int)sizes.size() - 1; k >= 0 && wins[k]; --k) at = sizes[k];
    return at;
}

}  // namespace

Tuned tuned() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tuned[current_device()];
}

int tuned_blocked_min(int precision) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const Tuned& t = g_tuned[current_device()];
    return precision == 1 ? t.blocked_min_split : t.blocked_min_fp64;
}

int tuned_sytrd_sym_min() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return g_tuned[current_device()].sytrd_sym_min;
}

void set_tuned(int sytrd_sym_min, int blocked_min_fp64, int blocked_min_split) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    Tuned& t = g_tuned[current_device()];
    t.sytrd_sym_min = sytrd_sym_min;
    t.blocked_min_fp64 = blocked_min_fp64;
    t.blocked_min_split = blocked_min_split;
    t.level = std::max(t.level, 1);
}

double time_sytrd(int n, int form, int max_blocks, int reps) {
    if (n < 3 || n > 8192) throw std::runtime_error("time_sytrd: n must lie in 3..8192");
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    XG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    XG_CUDA(cudaEventCreate(&e0));
    XG_CUDA(cudaEventCreate(&e1));
    const size_t nn = (size_t)n * n;
    const size_t doubles = 3 * nn + 3 * (size_t)n + sytrd_workspace(n);
    double* A0 = nullptr;
    double ms = 0.0;
    XG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&A0), doubles * sizeof(double), st));
    try {
        double* A = A0 + nn;
        double* V = A + nn;
        double* tau = V + nn;
        double* d = tau + n;
        double* e = d + n;
        double* p = e + n;
        k_tune_sym<<<ceil_div((long)n * n, 256), 256, 0, st>>>(n, 17u + n, A0);
        XG_LAUNCH_CHECK();
        ms = best_ms(st, e0, e1, std::max(1, reps), [&] {
            XG_CUDA(cudaMemcpyAsync(A, A0, sizeof(double) * nn, cudaMemcpyDeviceToDevice, st));
            sytrd_form(st, n, A, n, V, tau, d, e, p, form, max_blocks);
        });
    } catch (...) {
        cudaFreeAsync(A0, st);
        cudaStreamSynchronize(st);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaStreamDestroy(st);
        throw;
    }
    XG_CUDA(cudaFreeAsync(A0, st));
    XG_CUDA(cudaStreamSynchronize(st));
    XG_CUDA(cudaEventDestroy(e0));
    XG_CUDA(cudaEventDestroy(e1));
    XG_CUDA(cudaStreamDestroy(st));
    return ms;
}

void check_backtransform(int n, int ncol, int slices, double* out) {
    if (n < 3 || n > 8192 || ncol < 1 || ncol > n || slices < 0 || slices > 8)
        throw std::runtime_error("check_backtransform: n must lie in 3..8192, ncol in 1..n, slices in 0..8");
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    XG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    XG_CUDA(cudaEventCreate(&e0));
    XG_CUDA(cudaEventCreate(&e1));
    const size_t nn = (size_t)n * n;
    const size_t split_ws = slices ? (split_gemm_workspace(n, n, n, slices) + 255) / 256 * 256 : 0;
    const size_t doubles = 5 * nn + 3 * (size_t)n + sytrd_workspace(n) + ormtr_workspace(n) + 64;
    char* buf = nullptr;
    XG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&buf), doubles * sizeof(double) + split_ws + 512, st));
    try {
        char* sgw = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(buf) + 255) / 256 * 256);
        double* A = reinterpret_cast<double*>(sgw + split_ws);
        double* V = A + nn;
        double* Y0 = V + nn;
        double* Y1 = Y0 + nn;
        double* Y2 = Y1 + nn;
        double* tau = Y2 + nn;
        double* d = tau + n;
        double* e = d + n;
        double* p = e + n;
        double* ormw = p + sytrd_workspace(n);
        int* dcol = reinterpret_cast<int*>(ormw + ormtr_workspace(n));
        unsigned long long* mx = reinterpret_cast<unsigned long long*>(dcol + 16);
        k_tune_sym<<<ceil_div((long)nn, 256), 256, 0, st>>>(n, 91u + n, A);
        k_tune_sym<<<ceil_div((long)nn, 256), 256, 0, st>>>(n, 7u + n, Y0);
        XG_LAUNCH_CHECK();
        sytrd_form(st, n, A, n, V, tau, d, e, p, -1);
        XG_CUDA(cudaMemcpyAsync(dcol, &ncol, sizeof(int), cudaMemcpyHostToDevice, st));
        XG_CUDA(cudaMemsetAsync(mx, 0, 2 * sizeof(unsigned long long), st));
        auto warp = [&](double* Y) { ormtr_inplace(st, n, V, tau, Y, dcol); };
        auto blocked = [&](double* Y) { ormtr_blocked(st, n, V, tau, Y, dcol, ormw, slices, slices ? sgw : nullptr); };
        float ms[2] = {0.0f, 0.0f};
        double* dst[2] = {Y1, Y2};
        for (int f = 0; f < 2; ++f) {
            XG_CUDA(cudaMemcpyAsync(dst[f], Y0, nn * sizeof(double), cudaMemcpyDeviceToDevice, st));
            f ? blocked(dst[f]) : warp(dst[f]);   // warm-up
            XG_CUDA(cudaMemcpyAsync(dst[f], Y0, nn * sizeof(double), cudaMemcpyDeviceToDevice, st));
            XG_CUDA(cudaEventRecord(e0, st));
            f ? blocked(dst[f]) : warp(dst[f]);
            XG_CUDA(cudaEventRecord(e1, st));
            XG_CUDA(cudaEventSynchronize(e1));
            XG_CUDA(cudaEventElapsedTime(&ms[f], e0, e1));
        }
        k_tune_maxdiff<<<304, 256, 0, st>>>(n, ncol, Y1, Y2, mx);
        XG_LAUNCH_CHECK();
        unsigned long long h[2];
        XG_CUDA(cudaMemcpyAsync(h, mx, sizeof(h), cudaMemcpyDeviceToHost, st));
        XG_CUDA(cudaStreamSynchronize(st));
        double md, ma;
        std::memcpy(&md, &h[0], sizeof(double));
        std::memcpy(&ma, &h[1], sizeof(double));
        out[0] = ma > 0.0 ? md / ma : md;
        out[1] = ms[0];
        out[2] = ms[1];
    } catch (...) {
        cudaFreeAsync(buf, st);
        cudaStreamSynchronize(st);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaStreamDestroy(st);
        throw;
    }
    XG_CUDA(cudaFreeAsync(buf, st));
    XG_CUDA(cudaStreamSynchronize(st));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
}

Tuned autotune() {
    const int dev = current_device();
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (g_tuned[dev].level >= 1) return g_tuned[dev];
    }
    const auto t0 = std::chrono::steady_clock::now();
    Tuned t;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    XG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    XG_CUDA(cudaEventCreate(&e0));
    XG_CUDA(cudaEventCreate(&e1));
    const int nmax = 3072;
    const size_t nn = (size_t)nmax * nmax;
    const size_t split_ws = (split_gemm_workspace(nmax, nmax, nmax, 5) + 255) / 256 * 256;
    const size_t doubles = 4 * nn + 3 * (size_t)nmax + sytrd_workspace(nmax) + ormtr_workspace(nmax) + 64;
    char* buf = nullptr;
    XG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&buf), doubles * sizeof(double) + split_ws + 512, st));
    char* sgw = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(buf) + 255) / 256 * 256);
    double* A0 = reinterpret_cast<double*>(sgw + split_ws);
    double* A = A0 + nn;
    double* V = A + nn;
    double* Y = V + nn;
    double* tau = Y + nn;
    double* d = tau + nmax;
    double* e = d + nmax;
    double* p = e + nmax;
    double* ormw = p + sytrd_workspace(nmax);
    int* ncol = reinterpret_cast<int*>(ormw + ormtr_workspace(nmax));
    try {
        // 1. tridiagonalisation: row form against the upper-triangle form
        const std::vector<int> tsz = {192, 256, 384, 512, 768, 1024, 1536, 2048, 2560, 3072};
        std::vector<bool> sym_wins;
        for (int n : tsz) {
            k_tune_sym<<<ceil_div((long)n * n, 256), 256, 0, st>>>(n, 17u + n, A0);
            XG_LAUNCH_CHECK();
            double ms[2];
            for (int form = 0; form < 2; ++form)
                ms[form] = best_ms(st, e0, e1, 3, [&] {
                    XG_CUDA(cudaMemcpyAsync(A, A0, sizeof(double) * n * n, cudaMemcpyDeviceToDevice, st));
                    sytrd_form(st, n, A, n, V, tau, d, e, p, form);
                });
            // the copy is inside the timing of both forms alike
            t.sytrd_rows.insert(t.sytrd_rows.end(), {(double)n, ms[0], ms[1]});
            sym_wins.push_back(ms[1] < ms[0]);
        }
        t.sytrd_sym_min = crossover(tsz, sym_wins);
        // 2. back-transformation of n / 2 vectors: one warp per vector against the compact-WY form
        //    (FP64: column strips in one launch; split: the GEMM chain on the tensor cores)
        const std::vector<int> bsz = {300, 450, 600, 900, 1200, 1500, 1800, 2400};
        std::vector<bool> fp64_wins, split_wins;
        for (int n : bsz) {
            k_tune_sym<<<ceil_div((long)n * n, 256), 256, 0, st>>>(n, 91u + n, A);
            k_tune_sym<<<ceil_div((long)n * n, 256), 256, 0, st>>>(n, 7u + n, Y);
            XG_LAUNCH_CHECK();
            sytrd_form(st, n, A, n, V, tau, d, e, p, -1);
            const int k = n / 2;
            XG_CUDA(cudaMemcpyAsync(ncol, &k, sizeof(int), cudaMemcpyHostToDevice, st));
            const double w = best_ms(st, e0, e1, 2, [&] { ormtr_inplace(st, n, V, tau, Y, ncol); });
            const double b = best_ms(st, e0, e1, 2, [&] { ormtr_blocked(st, n, V, tau, Y, ncol, ormw, 0, nullptr); });
            const double s = best_ms(st, e0, e1, 2, [&] { ormtr_blocked(st, n, V, tau, Y, ncol, ormw, 5, sgw); });
            t.backtr_rows.insert(t.backtr_rows.end(), {(double)n, w, b, s});
            fp64_wins.push_back(b < w);
            split_wins.push_back(s < std::min(w, b));   // split mode runs the faster FP64 form below
        }
        t.blocked_min_fp64 = crossover(bsz, fp64_wins);
        t.blocked_min_split = crossover(bsz, split_wins);
    } catch (...) {
        cudaFreeAsync(buf, st);
        cudaStreamSynchronize(st);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaStreamDestroy(st);
        throw;
    }
    XG_CUDA(cudaFreeAsync(buf, st));
    XG_CUDA(cudaStreamSynchronize(st));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    t.level = 1;
    t.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tuned[dev] = t;
    return t;
}

}  // namespace xg
