// Split-precision GEMM on the BF16 tensor cores with FP64-level results.
//
// C = alpha op(A) op(B) + beta C for FP64 operands, computed from fixed-point slices:
// every row of op(A) (column of op(B)) is scaled by a power of two s_i (t_j) so that
// |x| < 1, and cut into S digits of 8 bits, x / s = sum_{p=1..S} d_p 2^(-8p) with integer
// d_p in [-256, 256] -- exactly representable in BF16 (the cut rounds x / s 2^(8S) to a 64-bit
// integer and takes its balanced base-256 digits with integer arithmetic).  A digit product d_p e_q is exact in
// FP32 (16 bits).  Products are grouped by level p + q (levels beyond S - 1 carry less than
// 2^(-8S) of the result and are dropped); the two leading levels are summed exactly over K
// chunks and recombined as integers, the others in FP32 (see the kernel), and the result is
// scaled back in FP64 with the weights 2^(-8(p+q)).  The errors are the truncation to S digits
// and the FP32 sums of the lower levels: with S = 5 about 2^-40 relative per product term.
//
// The products run on the tcgen05 tensor cores (BF16 in, FP32 accumulate in tensor memory);
// S(S+1)/2 tensor-core products replace one FP64 product.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "linalg.h"
#include "splitgemm.h"

namespace xg {

namespace {

constexpr int SG_KT = 32;               // K is padded to a multiple of this (one pipeline stage)

// 2^(8S - e) for scaling an element of a row with maximum magnitude in [2^(e-1), 2^e) to S
// digits, or 0 when that power of two is not a normal double (rows of subnormal magnitude)
template <int S>
__device__ __forceinline__ double digit_scale(int e) {
    const int sh = 8 * S - e;
    return sh <= 1023 ? ldexp(1.0, sh) : 0.0;
}

// The S balanced base-256 digits of y = x 2^(8S - e), |x| < 2^e: v = round(y) as a 64-bit
// integer (|v| <= 2^(8S) <= 2^56, and y itself is x with a shifted exponent), then the digits
// from the least significant one, each in [-128, 127], the leading one taking the rest (in
// [-256, 256]).  sum_p d_p 2^(8(S-1-p)) = v, so x 2^-e = sum_p d_p 2^(-8(p+1)) up to the rounding
// of the last digit -- the representation the products need, with one FP64 multiply and one
// conversion per element; the digit arithmetic is integer.
template <int S>
__device__ __forceinline__ void cut_digits(double x, double sc, int e, __nv_bfloat16 (&d)[S]) {
    const double y = sc != 0.0 ? x * sc : ldexp(x, 8 * S - e);
    long long v = __double2ll_rn(y);
#pragma unroll
    for (int p = S - 1; p > 0; --p) {
        const long long t = ((v + 128) & 255) - 128;
        d[p] = __float2bfloat16_rn((float)t);
        v = (v - t) >> 8;
    }
    d[0] = __float2bfloat16_rn((float)v);
}

// Digits of row r of X (element k = trans ? X[k*ldx + r] : X[r*ldx + k]), k < K (and k < *dK),
// zero beyond; out[p][r][k] for k < Kp.  One warp per row.
template <int S>
__global__ void k_split_rows(int R, int K, int Kp, const double* __restrict__ X, int ldx, int trans,
                             const int* __restrict__ dK, __nv_bfloat16* __restrict__ out, double* __restrict__ scale) {
    const int r = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (r >= R) return;
    const int kmax = dK ? min(K, *dK) : K;
    auto at = [&](int k) { return trans ? X[(size_t)k * ldx + r] : X[(size_t)r * ldx + k]; };
    double mx = 0.0;
    for (int k = lane; k < kmax; k += 32) mx = fmax(mx, fabs(at(k)));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if (mx > 0.0) {
        frexp(mx, &e);                 // mx = f 2^e, f in [0.5, 1): |x| / 2^e < 1
    }
    if (lane == 0) scale[r] = (mx > 0.0) ? ldexp(1.0, e) : 1.0;
    const size_t plane = (size_t)R * Kp;
    const double sc = digit_scale<S>(e);
    for (int k = lane; k < Kp; k += 32) {
        __nv_bfloat16 d[S];
        cut_digits<S>((k < kmax && mx > 0.0) ? at(k) : 0.0, sc, e, d);
#pragma unroll
        for (int p = 0; p < S; ++p) out[p * plane + (size_t)r * Kp + k] = d[p];
    }
}

// The same digits for the transposed case (element k of row r is X[k*ldx + r]), in two passes
// that read X along its rows: k_col_max takes the largest magnitude of each column over one
// 256-long K block (integer max on the magnitude bits, so the result does not depend on the
// order of the blocks), and k_col_digits cuts one 32 x 32 (r, k) tile per block, read with the
// lanes along r and written through shared memory with the lanes along k.
__global__ void __launch_bounds__(256) k_col_max(int R, int K, const double* __restrict__ X, int ldx,
                                                 const int* __restrict__ dK, unsigned long long* __restrict__ mbits) {
    __shared__ unsigned long long red[8][32];
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int r = blockIdx.x * 32 + l;
    const int kmax = dK ? min(K, *dK) : K;
    const int k0 = blockIdx.y * 256, k1 = min(kmax, k0 + 256);
    unsigned long long m = 0;
    if (r < R)
        for (int k = k0 + w; k < k1; k += 8) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(X[(size_t)k * ldx + r]) &
                                         0x7fffffffffffffffULL;
            m = b > m ? b : m;
        }
    red[w][l] = m;
    __syncthreads();
    if (w == 0 && r < R) {
        for (int q = 1; q < 8; ++q) m = red[q][l] > m ? red[q][l] : m;
        if (m) atomicMax(&mbits[r], m);
    }
}

template <int S>
__global__ void __launch_bounds__(256) k_col_digits(int R, int K, int Kp, const double* __restrict__ X, int ldx,
                                                    const int* __restrict__ dK,
                                                    const unsigned long long* __restrict__ mbits,
                                                    __nv_bfloat16* __restrict__ out, double* __restrict__ scale) {
    constexpr int LD = 34;   // bf16 per staged row: 17 words, so the 32 lanes hit 32 banks
    __shared__ __align__(16) __nv_bfloat16 dig[S][32][LD];
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    const int r = r0 + l;
    const int kmax = dK ? min(K, *dK) : K;
    const double mx = r < R ? __longlong_as_double((long long)mbits[r]) : 0.0;
    int e = 0;
    if (mx > 0.0) frexp(mx, &e);
    if (blockIdx.y == 0 && w == 0 && r < R) scale[r] = (mx > 0.0) ? ldexp(1.0, e) : 1.0;
    const double sc = digit_scale<S>(e);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int kk = w + 8 * j, k = k0 + kk;
        __nv_bfloat16 d[S];
        cut_digits<S>((r < R && k < kmax && mx > 0.0) ? X[(size_t)k * ldx + r] : 0.0, sc, e, d);
#pragma unroll
        for (int p = 0; p < S; ++p) dig[p][l][kk] = d[p];
    }
    __syncthreads();
    const size_t plane = (size_t)R * Kp;
    for (int idx = threadIdx.x; idx < S * 32 * 16; idx += 256) {
        const int p = idx / 512, row = (idx / 16) % 32, wd = idx % 16;
        if (r0 + row >= R) continue;
        const uint32_t v = *reinterpret_cast<const uint32_t*>(&dig[p][row][2 * wd]);
        *reinterpret_cast<uint32_t*>(out + p * plane + (size_t)(r0 + row) * Kp + k0 + 2 * wd) = v;
    }
}

}  // namespace

namespace {

// ------------------------------------------------------------------ tcgen05 form
// The same digit products on the 5th-generation tensor cores: tcgen05.mma (M = 128, N = 64,
// K = 16, BF16 in, FP32 accumulate) with the accumulators in tensor memory (TMEM) and the digit
// planes staged by TMA (cp.async.bulk.tensor, one 3-D box = all S planes of a 32-long K slice,
// 64-byte swizzle) through a TC_STAGES-deep mbarrier pipeline.  Warp roles: warp 0 issues the
// TMA loads, one thread of warp 1 issues the MMAs (warp 1 also owns the TMEM allocation),
// warps 2..5 run the epilogue, one TMEM lane (= one output row) per thread.
//
// Exactness: digits are integers with |d| <= 256 (first) and <= 128 (later), so over a K chunk
// of 256 the level-0 sum (at most 256 * 2^16) and the level-1 sum (at most 2 * 256 * 2^15)
// are integers of at most 2^24 -- exact in FP32.  These two levels are reset every chunk and
// folded by the epilogue into 64-bit integer accumulators (F2I and integer adds, no FP64
// work: the FP64 pipe would otherwise bound the product), while the TMEM holds the next chunk's
// sums (two buffers).  Levels 2 .. S-1 carry at most 2^-16 of the result; they accumulate over
// the whole K in FP32 (rounding below 2^-40 of the result) and are added once at the end.
constexpr int TC_BM = 128, TC_BN = 64, TC_BK = 32, TC_KC = 256;
constexpr int TC_THREADS = 192;
constexpr int TC_GROUP = 8;              // row tiles per group of the tile order (8 x 19 = 152 CTAs)
constexpr unsigned TC_SPIN = 1u << 25;   // iteration limit of every mbarrier wait

template <int S>
struct TcCfg {
    static constexpr int A_BYTES = S * TC_BM * TC_BK * 2;   // one stage of A: [S][128][32] bf16
    static constexpr int B_BYTES = S * TC_BN * TC_BK * 2;   // one stage of B: [S][64][32] bf16
    static constexpr int STAGE = A_BYTES + B_BYTES;         // a multiple of 1024
    static constexpr int STAGES = (3 * STAGE <= 200 * 1024) ? 3 : 2;
    static constexpr int NB = (4 + (S - 2)) * TC_BN <= 512 ? 2 : 1;   // level-0/1 buffers in TMEM
    static constexpr int SMEM = STAGES * STAGE + 1024 /* alignment */ + 256 /* barriers */;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// wait for the phase `parity` of an mbarrier; false after TC_SPIN polls or when another role
// raised the abort flag
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag) {
    for (unsigned it = 0; it < TC_SPIN; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & 255u) == 255u && *abort_flag) return false;
    }
    return false;
}

// K-major operand in shared memory, 64-byte swizzle: rows of 64 bytes (32 bf16), groups of 8
// rows 512 bytes apart (SBO); the leading offset is unused for this layout
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;             // LBO (ignored)
    d |= (uint64_t)(512 >> 4) << 32;    // SBO
    d |= (uint64_t)1 << 46;             // descriptor version of this architecture
    d |= (uint64_t)4 << 61;             // SWIZZLE_64B
    return d;
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

template <int S>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_split_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
               int Kp, const double* __restrict__ sA, const double* __restrict__ sB, double alpha, double beta,
               double* __restrict__ C, int ldc, const int* __restrict__ dN, int kchunk, double* __restrict__ P,
               int* __restrict__ err) {
    using Cfg = TcCfg<S>;
    extern __shared__ unsigned char tc_raw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + Cfg::STAGES * Cfg::STAGE);
    uint64_t* full = bars;                        // [STAGES]: TMA landed
    uint64_t* empty = bars + Cfg::STAGES;         // [STAGES]: MMAs done reading
    uint64_t* cfull = bars + 2 * Cfg::STAGES;     // [NB]: a chunk's level-0/1 sums complete
    uint64_t* cempty = cfull + 2;                 // [NB]: the epilogue has read them
    uint64_t* done = cempty + 2;                  // every MMA complete
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // grouped tile order: TC_GROUP row tiles share each column tile in turn, so that the A and
    // B tiles of the CTAs in flight together stay in L2
    int tm, tn;
    {
        const int npm = (M + TC_BM - 1) / TC_BM, npn = (N + TC_BN - 1) / TC_BN;
        const int pid = blockIdx.x, group = TC_GROUP * npn;
        const int first = (pid / group) * TC_GROUP, gsz = min(npm - first, TC_GROUP);
        tm = first + (pid % group) % gsz;
        tn = (pid % group) / gsz;
    }
    const int i0 = tm * TC_BM, j0 = tn * TC_BN;
    const int Nl = dN ? min(N, *dN) : N;
    if (j0 >= Nl) return;
    const int kb = P ? (int)blockIdx.z * kchunk : 0;
    const int ke = P ? min(Kp, kb + kchunk) : Kp;
    const int nstage = (ke - kb) / TC_BK;
    const int nchunk = (ke - kb + TC_KC - 1) / TC_KC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < Cfg::STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&empty[s])));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&cfull[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;\n" ::"r"(smem_u32(&cempty[b])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(done)));
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    volatile int* abort_v = abort_flag;

    if (warp == 0) {
        // ---- TMA producer
        if (lane == 0) {
            // B tiles are read by the group's row tiles together and then not again for the
            // group: evict-first keeps the group's A tiles in L2 across its column tiles (DRAM
            // reads at 4096^3: 1.34 -> 1.07 GB; groups of 6, 10, 12 or 16 rows read more)
            uint64_t pol_b;
            asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(pol_b));
            int issued = 0;
            for (int ks = 0; ks < nstage; ++ks) {
                const int s = ks % Cfg::STAGES;
                if (ks >= Cfg::STAGES && !tc_wait(smem_u32(&empty[s]), ((ks / Cfg::STAGES) - 1) & 1, abort_v)) {
                    *abort_v = 1;
                    break;
                }
                unsigned char* sa = base + s * Cfg::STAGE;
                unsigned char* sb = sa + Cfg::A_BYTES;
                const uint32_t fb = smem_u32(&full[s]);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(fb), "r"(Cfg::STAGE)
                             : "memory");
                const int kx = kb + ks * TC_BK;
                asm volatile(
                    "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
                    "%3, %4}], [%5];\n" ::"r"(smem_u32(sa)),
                    "l"(reinterpret_cast<uint64_t>(&tmA)), "r"(kx), "r"(i0), "r"(0), "r"(fb)
                    : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint "
                    "[%0], [%1, {%2, %3, %4}], [%5], %6;\n" ::"r"(smem_u32(sb)),
                    "l"(reinterpret_cast<uint64_t>(&tmB)), "r"(kx), "r"(j0), "r"(0), "r"(fb), "l"(pol_b)
                    : "memory");
                ++issued;
            }
            // on an abort, the copies in flight still land: wait for them (bounded) before leaving
            if (*abort_v)
                for (int ks = max(0, issued - Cfg::STAGES); ks < issued; ++ks) {
                    volatile int never = 0;
                    tc_wait(smem_u32(&full[ks % Cfg::STAGES]), (ks / Cfg::STAGES) & 1, &never);
                }
        }
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = tc_idesc(TC_BM, TC_BN);
            const uint32_t low0 = tmem + Cfg::NB * 2 * TC_BN;   // levels 2.. S-1
            for (int ks = 0; ks < nstage; ++ks) {
                const int s = ks % Cfg::STAGES;
                const int c = (ks * TC_BK) / TC_KC, buf = c % Cfg::NB;
                const bool cfirst = (ks * TC_BK) % TC_KC == 0;
                const bool clast = ((ks + 1) * TC_BK) % TC_KC == 0 || ks + 1 == nstage;
                if (cfirst && c >= Cfg::NB && !tc_wait(smem_u32(&cempty[buf]), ((c / Cfg::NB) - 1) & 1, abort_v)) {
                    *abort_v = 1;
                    break;
                }
                if (!tc_wait(smem_u32(&full[s]), (ks / Cfg::STAGES) & 1, abort_v)) {
                    *abort_v = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                const uint32_t sa = smem_u32(base + s * Cfg::STAGE);
                const uint32_t sb = sa + Cfg::A_BYTES;
#pragma unroll
                for (int kk = 0; kk < TC_BK / 16; ++kk) {
                    uint32_t started = 0;   // bit l: level l has had its first product of this k-step
#pragma unroll
                    for (int p = 0; p < S; ++p)
#pragma unroll
                        for (int q = 0; q < S - p; ++q) {
                            const int l = p + q;
                            const uint32_t d = l <= 1 ? tmem + buf * 2 * TC_BN + l * TC_BN : low0 + (l - 2) * TC_BN;
                            // the first product of a level overwrites: levels 0/1 at the start of
                            // their chunk, levels >= 2 at the very start
                            const bool fresh = !(started >> l & 1u) && kk == 0 && (l <= 1 ? cfirst : ks == 0);
                            started |= 1u << l;
                            const uint64_t ad = tc_desc(sa + p * (TC_BM * TC_BK * 2) + kk * 32);
                            const uint64_t bd = tc_desc(sb + q * (TC_BN * TC_BK * 2) + kk * 32);
                            const uint32_t acc = fresh ? 0u : 1u;
                            asm volatile(
                                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                        }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 smem_u32(&empty[s]))
                             : "memory");
                if (clast)
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                     smem_u32(&cfull[buf]))
                                 : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             smem_u32(done))
                         : "memory");
            if (*abort_v) {   // the MMAs issued so far must finish before the TMEM is freed
                volatile int never = 0;
                tc_wait(smem_u32(done), 0, &never);
            }
        }
    } else {
        // ---- epilogue: TMEM lane (32 (warp % 4) + lane) = output row
        const int quarter = warp & 3;
        const uint32_t lrow = (uint32_t)(32 * quarter) << 16;
        const int i = i0 + 32 * quarter + lane;
        long long ex[TC_BN];
#pragma unroll
        for (int j = 0; j < TC_BN; ++j) ex[j] = 0;
        bool ok = true;
        for (int c = 0; c < nchunk && ok; ++c) {
            const int buf = c % Cfg::NB;
            if (!tc_wait(smem_u32(&cfull[buf]), (c / Cfg::NB) & 1, abort_v)) {
                *abort_v = 1;
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int cb = 0; cb < TC_BN / 16; ++cb) {
                float l0[16], l1[16];
                tc_ld16(tmem + lrow + buf * 2 * TC_BN + cb * 16, l0);
                tc_ld16(tmem + lrow + buf * 2 * TC_BN + TC_BN + cb * 16, l1);
#pragma unroll
                for (int k = 0; k < 16; ++k)
                    ex[cb * 16 + k] += 256LL * (long long)__float2int_rn(l0[k]) + (long long)__float2int_rn(l1[k]);
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(&cempty[buf])) : "memory");
        }
        if (ok && !tc_wait(smem_u32(done), 0, abort_v)) {
            *abort_v = 1;
            ok = false;
        }
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t low0 = tmem + lrow + Cfg::NB * 2 * TC_BN;
            const double ra = (i < M) ? alpha * sA[i] : 0.0;
#pragma unroll
            for (int cb = 0; cb < TC_BN / 16; ++cb) {
                double lo[16];
#pragma unroll
                for (int k = 0; k < 16; ++k) lo[k] = 0.0;
#pragma unroll
                for (int l = S - 1; l >= 2; --l) {
                    float v[16];
                    tc_ld16(low0 + (l - 2) * TC_BN + cb * 16, v);
#pragma unroll
                    for (int k = 0; k < 16; ++k) lo[k] = lo[k] * 0x1p-8 + (double)v[k];
                }
#pragma unroll
                for (int k = 0; k < 16; ++k) {
                    const int j = j0 + cb * 16 + k;
                    if (i >= M || j >= Nl) continue;
                    // sum of levels in units of level 0: exact part / 256 + lower levels / 65536
                    const double sum = (double)ex[cb * 16 + k] * 0x1p-8 + lo[k] * 0x1p-16;
                    double r = ra * sB[j] * (sum * 0x1p-16);
                    if (P) {
                        P[((size_t)blockIdx.z * M + i) * N + j] = r;
                        continue;
                    }
                    if (beta != 0.0) r += beta * C[(size_t)i * ldc + j];
                    C[(size_t)i * ldc + j] = r;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && *abort_v) atomicExch(err, 1);
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
    }
}

}  // namespace

// Split K for products with few output tiles (the skinny products of the blocked
// back-transformation): up to SG_KS slices of whole exact chunks, when the tile grid would leave
// SMs idle.  Partials need at most SG_KS x min(M N, SG_SPLIT_ELEMS) doubles.
constexpr int SG_KS = 8;
constexpr long SG_SPLIT_TILES = 304;
constexpr size_t SG_SPLIT_ELEMS = (size_t)SG_SPLIT_TILES * TC_BM * TC_BN;

static int split_k_slices(int M, int N, int Kp) {
    const long tiles = (long)((M + TC_BM - 1) / TC_BM) * ((N + TC_BN - 1) / TC_BN);
    if (tiles >= SG_SPLIT_TILES) return 1;
    const int by_chunks = Kp / (2 * TC_KC);   // at least two exact chunks per slice
    const int want = (int)std::min<long>(SG_KS, std::max<long>(1, SG_SPLIT_TILES / tiles));
    return std::max(1, std::min(want, by_chunks));
}

// cuTensorMapEncodeTiled from the driver (through the runtime, so nothing links libcuda)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (!fn) throw CudaError("split_gemm: cuTensorMapEncodeTiled is not available");
    return fn;
}

// 3-D map of S digit planes [S][rows][Kp] (bf16), boxes of 32 (K) x box_rows x S, 64-byte swizzle
static CUtensorMap plane_map(const __nv_bfloat16* planes, int rows, int Kp, int S, int box_rows) {
    CUtensorMap m;
    const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)S};
    const cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)rows * (cuuint64_t)Kp * 2};
    const cuuint32_t box[3] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows, (cuuint32_t)S};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                                            const_cast<__nv_bfloat16*>(planes), dims, strides, box, es,
                                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw CudaError("split_gemm: tensor map encoding failed");
    return m;
}

// C[i][j] = sum_z P[z][i][j] (in slice order) + beta C[i][j], j < N (and < *dN)
__global__ void k_split_reduce(int M, int N, int KS, const double* __restrict__ P, double beta,
                               double* __restrict__ C, int ldc, const int* __restrict__ dN) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)M * N) return;
    const int i = (int)(t / N), j = (int)(t % N);
    if (dN && j >= *dN) return;
    double r = 0.0;
    for (int z = 0; z < KS; ++z) r += P[((size_t)z * M + i) * N + j];
    if (beta != 0.0) r += beta * C[(size_t)i * ldc + j];
    C[(size_t)i * ldc + j] = r;
}

size_t split_gemm_workspace(int M, int N, int K, int slices) {
    const size_t Kp = (size_t)((K + SG_KT - 1) / SG_KT) * SG_KT;
    const size_t bf = (size_t)slices * ((size_t)M + N) * Kp * sizeof(__nv_bfloat16);
    const size_t split = (size_t)SG_KS * std::min((size_t)M * N, SG_SPLIT_ELEMS);
    return (bf + 255) / 256 * 256 + 2 * ((size_t)M + N) * sizeof(double) + split * sizeof(double) + 768;
}

// the tensor-core kernel's error flag: the last word of the workspace
static int* split_error_flag(void* work, int M, int N, int K, int slices) {
    return reinterpret_cast<int*>(static_cast<char*>(work) + split_gemm_workspace(M, N, K, slices) - sizeof(int));
}

// Digits and scales of the rows of op(X) (R rows, K long): along memory rows when !trans,
// through the column kernels when trans.
template <int S>
static void split_operand(cudaStream_t st, int R, int K, int Kp, const double* X, int ldx, bool trans, const int* dK,
                          __nv_bfloat16* out, double* scale, unsigned long long* mbits) {
    if (!trans) {
        k_split_rows<S><<<ceil_div((long)R * 32, 256), 256, 0, st>>>(R, K, Kp, X, ldx, 0, dK, out, scale);
        XG_LAUNCH_CHECK();
        return;
    }
    XG_CUDA(cudaMemsetAsync(mbits, 0, (size_t)R * sizeof(unsigned long long), st));
    k_col_max<<<dim3(ceil_div(R, 32), std::max(1, ceil_div(K, 256))), 256, 0, st>>>(R, K, X, ldx, dK, mbits);
    XG_LAUNCH_CHECK();
    k_col_digits<S><<<dim3(ceil_div(R, 32), Kp / 32), 256, 0, st>>>(R, K, Kp, X, ldx, dK, mbits, out, scale);
    XG_LAUNCH_CHECK();
}

template <int S>
static void split_gemm_s(cudaStream_t st, bool ta, bool tb, int M, int N, int K, double alpha, const double* A,
                         int lda, const double* B, int ldb, double beta, double* C, int ldc, void* work,
                         const int* dK, const int* dN) {
    const int Kp = ((K + SG_KT - 1) / SG_KT) * SG_KT;
    __nv_bfloat16* As = static_cast<__nv_bfloat16*>(work);
    __nv_bfloat16* Bs = As + (size_t)S * M * Kp;
    const size_t bf = (size_t)S * ((size_t)M + N) * Kp * sizeof(__nv_bfloat16);
    double* sA = reinterpret_cast<double*>(static_cast<char*>(work) + (bf + 255) / 256 * 256);
    double* sB = sA + M;
    unsigned long long* mA = reinterpret_cast<unsigned long long*>(sB + N);
    unsigned long long* mB = mA + M;
    split_operand<S>(st, M, K, Kp, A, lda, ta, dK, As, sA, mA);
    split_operand<S>(st, N, K, Kp, B, ldb, !tb, dK, Bs, sB, mB);
    const CUtensorMap tmA = plane_map(As, M, Kp, S, TC_BM);
    const CUtensorMap tmB = plane_map(Bs, N, Kp, S, TC_BN);
    int* err = split_error_flag(work, M, N, K, S);
    const int smem = TcCfg<S>::SMEM;
    allow_max_dynamic_smem((const void*)k_split_tc<S>);
    const int ks = split_k_slices(M, N, Kp);
    if (ks > 1) {
        const int kchunk = ((Kp / ks + TC_KC - 1) / TC_KC) * TC_KC;
        const int kz = (Kp + kchunk - 1) / kchunk;
        double* P = reinterpret_cast<double*>(
            (reinterpret_cast<uintptr_t>(mB + N) + 255) / 256 * 256);   // after the scales and maxima
        dim3 grid(ceil_div(N, TC_BN) * ceil_div(M, TC_BM), 1, kz);
        k_split_tc<S><<<grid, TC_THREADS, smem, st>>>(tmA, tmB, M, N, Kp, sA, sB, alpha, beta, C, ldc, dN, kchunk,
                                                      P, err);
        XG_LAUNCH_CHECK();
        k_split_reduce<<<ceil_div((long)M * N, 256), 256, 0, st>>>(M, N, kz, P, beta, C, ldc, dN);
        XG_LAUNCH_CHECK();
        return;
    }
    dim3 grid(ceil_div(N, TC_BN) * ceil_div(M, TC_BM));
    k_split_tc<S><<<grid, TC_THREADS, smem, st>>>(tmA, tmB, M, N, Kp, sA, sB, alpha, beta, C, ldc, dN, Kp, nullptr,
                                                  err);
    XG_LAUNCH_CHECK();
}

void split_gemm(cudaStream_t st, bool ta, bool tb, int M, int N, int K, double alpha, const double* A, int lda,
                const double* B, int ldb, double beta, double* C, int ldc, int slices, void* work, const int* dK,
                const int* dN) {
    if (M <= 0 || N <= 0) return;
    if (reinterpret_cast<uintptr_t>(work) % 256 != 0) throw CudaError("split_gemm: workspace must be 256-byte aligned");
    switch (slices) {
        case 4: split_gemm_s<4>(st, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, work, dK, dN); break;
        case 5: split_gemm_s<5>(st, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, work, dK, dN); break;
        case 6: split_gemm_s<6>(st, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, work, dK, dN); break;
        case 7: split_gemm_s<7>(st, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, work, dK, dN); break;
        default: throw CudaError("split_gemm: slices must be 4..7");
    }
}

namespace {
// deterministic pseudo-random fill: uniform(-1, 1) times 2^(e) with e uniform in [-ed, 0]
__global__ void k_fill(size_t n, unsigned seed, int ed, double* __restrict__ x) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long h = (i + 1) * 0x9E3779B97F4A7C15ull ^ ((unsigned long long)seed << 32);
    h ^= h >> 31; h *= 0xBF58476D1CE4E5B9ull; h ^= h >> 27; h *= 0x94D049BB133111EBull; h ^= h >> 31;
    const double u = (double)(h >> 11) * 0x1p-53 * 2.0 - 1.0;
    const int e = ed > 0 ? -(int)((h >> 3) % (unsigned)(ed + 1)) : 0;
    x[i] = ldexp(u, e);
}
__global__ void k_abs(size_t n, const double* __restrict__ x, double* __restrict__ y) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = fabs(x[i]);
}
// out[0] = max |d - r| / b, out[1] = max |d - r| / max |r| (block 0 atomics-free: one block)
__global__ void k_errmax(size_t n, const double* __restrict__ d, const double* __restrict__ r,
                         const double* __restrict__ b, double* __restrict__ out) {
    __shared__ double s0[256], s1[256], s2[256];
    double e0 = 0.0, e1 = 0.0, mr = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double e = fabs(d[i] - r[i]);
        e0 = fmax(e0, b[i] > 0.0 ? e / b[i] : e);
        e1 = fmax(e1, e);
        mr = fmax(mr, fabs(r[i]));
    }
    s0[threadIdx.x] = e0; s1[threadIdx.x] = e1; s2[threadIdx.x] = mr;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)blockDim.x; ++k) { e0 = fmax(e0, s0[k]); e1 = fmax(e1, s1[k]); mr = fmax(mr, s2[k]); }
        out[0] = e0;
        out[1] = mr > 0.0 ? e1 / mr : e1;
    }
}
}  // namespace

void split_gemm_check(int M, int N, int K, int slices, unsigned seed, int exp_range, double* out) {
    cudaStream_t st = nullptr;
    XG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const size_t na = (size_t)M * K, nb = (size_t)K * N, nc = (size_t)M * N;
    const size_t ws = split_gemm_workspace(M, N, K, slices);
    char* buf = nullptr;
    const size_t doubles = 2 * (na + nb) + 3 * nc + 8;
    XG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&buf), doubles * sizeof(double) + 256 + ws, st));
    double* A = reinterpret_cast<double*>(buf);
    double* B = A + na;
    double* Aa = B + nb;
    double* Ba = Aa + na;
    double* Cs = Ba + nb;
    double* Cr = Cs + nc;
    double* Cb = Cr + nc;
    double* res = Cb + nc;
    // the digit planes are read with 16-byte loads: keep the workspace 256-byte aligned
    const size_t off = (((doubles * sizeof(double)) + 255) / 256) * 256;
    void* work = buf + off;
    k_fill<<<ceil_div((long)na, 256), 256, 0, st>>>(na, seed, exp_range, A);
    k_fill<<<ceil_div((long)nb, 256), 256, 0, st>>>(nb, seed + 1, exp_range, B);
    k_abs<<<ceil_div((long)na, 256), 256, 0, st>>>(na, A, Aa);
    k_abs<<<ceil_div((long)nb, 256), 256, 0, st>>>(nb, B, Ba);
    XG_LAUNCH_CHECK();
    int* err = split_error_flag(work, M, N, K, slices);
    XG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    dgemm(st, false, false, M, N, K, 1.0, Aa, K, Ba, N, 0.0, Cb, N);
    cudaEvent_t e0, e1, e2;
    XG_CUDA(cudaEventCreate(&e0));
    XG_CUDA(cudaEventCreate(&e1));
    XG_CUDA(cudaEventCreate(&e2));
    split_gemm(st, false, false, M, N, K, 1.0, A, K, B, N, 0.0, Cs, N, slices, work);   // warm-up
    dgemm(st, false, false, M, N, K, 1.0, A, K, B, N, 0.0, Cr, N);
    XG_CUDA(cudaEventRecord(e0, st));
    split_gemm(st, false, false, M, N, K, 1.0, A, K, B, N, 0.0, Cs, N, slices, work);
    XG_CUDA(cudaEventRecord(e1, st));
    dgemm(st, false, false, M, N, K, 1.0, A, K, B, N, 0.0, Cr, N);
    XG_CUDA(cudaEventRecord(e2, st));
    k_errmax<<<1, 256, 0, st>>>(nc, Cs, Cr, Cb, res);
    XG_LAUNCH_CHECK();
    double h[2];
    int herr = 0;
    XG_CUDA(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    XG_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        cudaFreeAsync(buf, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
        throw CudaError("split_gemm: a pipeline wait of the tensor-core kernel timed out");
    }
    float ms_s = 0.0f, ms_d = 0.0f;
    XG_CUDA(cudaEventElapsedTime(&ms_s, e0, e1));
    XG_CUDA(cudaEventElapsedTime(&ms_d, e1, e2));
    const double flops = 2.0 * M * N * (double)K;
    out[0] = h[0];
    out[1] = h[1];
    out[2] = ms_s;
    out[3] = ms_d;
    out[4] = flops / (ms_s * 1e-3) / 1e12;
    out[5] = flops / (ms_d * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    XG_CUDA(cudaFreeAsync(buf, st));
    XG_CUDA(cudaStreamSynchronize(st));
    cudaStreamDestroy(st);
}

}  // namespace xg
