// Split-precision (Ozaki) products T = X A for tall-skinny FP64 operands on
// the 5th-generation tensor cores: X [rows, K], A [K, ncols <= 16], K <= 4096.
//
// Scheme.  Every row i of X is scaled by 2^-E_i (E_i: smallest power of two
// above max_k |X[i,k]|) and its magnitude rounded to 60 fractional bits,
// which are cut into NSL = 10 signed 6-bit digits d_p (p = 0 most
// significant):
//   X[i,k] ~ 2^E_i sum_p d_p[i,k] 2^-6(p+1),   |d_p| <= 63.
// Columns of A are split the same way with their own exponents F_j.  Each
// digit is an exact BF16.  For every digit pair (p,q) with p + q <= 10 the
// tensor cores form S_pq = sum_k d_p e_q in FP32; |S_pq| <= 63*63*K < 2^24
// for K <= 4096, so these sums are exact and their order does not matter.
// The epilogue recombines
//   T[i,j] = 2^(E_i + F_j - 12) sum_t 2^-6t sum_{p+q=t} S_pq[i,j]
// in integer and FP64 arithmetic.  The error is the rounding to 60 bits
// (2^-61 of the row / column maximum) plus the dropped pairs p + q > 10
// (< 2^-62).
//
// Kernel.  One CTA per SM (persistent over 128-row tiles of up to four
// products), 320 threads: warp 8 streams digit tiles global -> shared with
// 1-D bulk copies (cp.async.bulk, mbarrier transaction counts), warp 9
// issues tcgen05.mma (M = 128, K = 16) into TMEM, warps 0-7 read the
// accumulators back with tcgen05.ld (two warps per TMEM lane quadrant, eight
// output columns each) and recombine.  The 64 digit pairs need 1024
// accumulator columns, so a tile runs four passes over K (slices {0,1,2},
// {3,4,5}, {6,7}, {8,9}), each streaming only its own digit slices; one MMA
// per slice and K step covers all q-slices paired with it.  The epilogue
// copies a pass's sums into integer registers and releases TMEM before the
// FP64 recombination, so the next pass starts at once.  Operand tiles use the
// 128-byte-swizzled K-major layout (one 128-byte swizzle atom per row and
// stage, KC = 64), which the tensor cores read at full shared-memory
// bandwidth; the split kernels write the digits directly in that layout, so
// a pipeline stage (the slices of one pass for 64 columns of K) is one
// contiguous block in HBM.
// Every wait is bounded; a timeout sets the error flag and the kernel winds
// down (waits for its copies in flight, frees TMEM) instead of hanging.
#include <cstdint>

#include "nvpt2_internal.h"
#include "oz_ptx.cuh"
#include "ozaki.cuh"

namespace nvpt {
namespace oz {

__host__ __device__ constexpr int pass_of(int p) {
    int g = 0;
    while (pass_p0(g + 1) <= p) ++g;
    return g;
}
// TMEM column of the (p, q = 0) accumulator within its pass.
__host__ __device__ constexpr int col_off(int p) {
    int c = 0;
    for (int i = pass_p0(pass_of(p)); i < p; ++i) c += NB * nq(i);
    return c;
}
// Lowest and highest t = p + q of a pass.
__host__ __device__ constexpr int pass_tmax(int g) {
    int t = 0;
    for (int p = pass_p0(g); p < pass_p0(g + 1); ++p) t = (p + nq(p) - 1) > t ? (p + nq(p) - 1) : t;
    return t;
}
constexpr int MAX_PASS_T = 11;  // t values a pass can hold (its V registers)
__host__ __device__ constexpr bool passes_fit() {
    for (int g = 0; g < NPASS; ++g) {
        const int last = pass_p0(g + 1) - 1;
        if (col_off(last) + NB * nq(last) > TMEM_COLS) return false;
        if (pass_p0(g + 1) - pass_p0(g) > MAX_PASS_SLICES) return false;
        if (pass_tmax(g) - pass_p0(g) + 1 > MAX_PASS_T) return false;
    }
    return pass_p0(NPASS) == NSL && NB * nq(0) <= 256;  // one MMA (N <= 256) per slice
}
static_assert(passes_fit(), "every pass fits TMEM, one pipeline stage and the epilogue registers");

// ------------------------------------------------------------- the product
constexpr int A_ROW = NSL * A_TILE;  // digit bytes of one (row tile, K chunk) in HBM

// The MMAs of one pipeline stage of pass PASS: for each 32-byte K step of the
// swizzle atom and each slice p of the pass, one MMA over all q-slices paired
// with p.  Descriptors advance by constant offsets (in 16-byte units of the
// start-address field) from the stage bases, so the issuing thread spends a
// few instructions per MMA.  i: the stage's index within the pass (the first
// MMA of a pass overwrites its accumulator).
template <int PASS>
__device__ __forceinline__ void issue_pass(uint64_t dA, uint64_t dB, uint32_t tmem, int i) {
    constexpr int p0 = pass_p0(PASS), p1 = pass_p0(PASS + 1);
#pragma unroll
    for (int kk = 0; kk < KC / 16; ++kk) {  // 32-byte K steps inside the swizzle atom
        const uint32_t acc = (i > 0 || kk > 0) ? 1u : 0u;
#pragma unroll
        for (int p = p0; p < p1; ++p) {
            const uint64_t da = dA + (uint64_t)(((p - p0) * A_TILE + kk * 32) >> 4);
            const uint64_t db = dB + (uint64_t)((kk * 32) >> 4);
            umma(tmem + (uint32_t)col_off(p), da, db, idesc_bf16(NB * nq(p)), acc);
        }
    }
}

// First K chunk of a tile.  Every CTA reads the same B digit tiles; starting
// the tiles at different chunks spreads those reads over L2 instead of
// having all SMs hit the same lines at once.  The digit sums are exact
// integers, so the order over K does not change the result.
__device__ __forceinline__ int kc_start(long long tile, int nkc) { return (int)((tile * 13) % nkc); }

__global__ void __launch_bounds__(THREADS, 1) k_oz_gemm(OzBatch b, int *err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bar_full[STAGES], bar_empty[STAGES], bar_tfull, bar_tempty, bar_done;
    __shared__ uint32_t s_tmem;
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sA0 = su32(smem), sB0 = sA0 + STAGES * A_STAGE;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int PRODUCER = EPI_WARPS, ISSUER = EPI_WARPS + 1;

    long long ntiles = 0;
    for (int j = 0; j < b.njob; ++j) ntiles += b.job[j].nrt;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(su32(&bar_full[s]), 1);
            mbar_init(su32(&bar_empty[s]), 1);
        }
        mbar_init(su32(&bar_tfull), 1);
        mbar_init(su32(&bar_tempty), 32 * EPI_WARPS);
        mbar_init(su32(&bar_done), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_tmem)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = s_tmem;

    auto decode = [&](long long tile, int &j, int &rt) {
        j = 0;
        while (tile >= b.job[j].nrt) {
            tile -= b.job[j].nrt;
            ++j;
        }
        rt = (int)tile;
    };

    if (warp == PRODUCER) {
        // ---------------- producer: digit tiles global -> shared
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                int j, rt;
                decode(tile, j, rt);
                const uint8_t *asrc = b.job[j].ad + (size_t)rt * b.nkc * A_ROW;
                const uint8_t *bsrc = b.job[j].bd;
                const int k0 = kc_start(tile, b.nkc);
                for (int pass = 0; pass < NPASS && ok; ++pass) {
                    const uint32_t abytes = (uint32_t)(pass_p0(pass + 1) - pass_p0(pass)) * A_TILE;
                    // rows of the q-slices this pass pairs with (nq falls with p)
                    const uint32_t bbytes = (uint32_t)nq(pass_p0(pass)) * NB * ROWB;
                    for (int i = 0; i < b.nkc; ++i, ++it) {
                        const int kc = (k0 + i) % b.nkc;
                        const uint32_t s = it % STAGES, ph = (it / STAGES) & 1u;
                        if (!mbar_wait(su32(&bar_empty[s]), ph ^ 1u, err)) {
                            ok = false;
                            break;
                        }
                        mbar_expect_tx(su32(&bar_full[s]), abytes + bbytes);
                        bulk_g2s(sA0 + s * A_STAGE, asrc + (size_t)kc * A_ROW + (size_t)pass_p0(pass) * A_TILE, abytes,
                                 su32(&bar_full[s]));
                        bulk_g2s(sB0 + s * B_STAGE, bsrc + (size_t)kc * B_STAGE, bbytes, su32(&bar_full[s]));
                    }
                }
            }
            // copies still in flight land on the full barriers of the last
            // STAGES iterations: wait for them (bounded) before exiting
            const uint32_t first = it > (uint32_t)STAGES ? it - STAGES : 0u;
            for (uint32_t k = first; k < it; ++k) {
                const uint32_t s = k % STAGES, ph = (k / STAGES) & 1u;
                for (uint32_t i = 0; i < kSpinLimit && !mbar_test(su32(&bar_full[s]), ph); ++i) __nanosleep(100);
            }
        }
    } else if (warp == ISSUER) {
        // ---------------- MMA issuer
        if (lane == 0) {
            uint32_t it = 0, tl = 0;
            bool ok = true;
            for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                for (int pass = 0; pass < NPASS && ok; ++pass, ++tl) {
                    if (!mbar_wait(su32(&bar_tempty), (tl & 1u) ^ 1u, err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    for (int i = 0; i < b.nkc; ++i, ++it) {
                        const uint32_t s = it % STAGES, ph = (it / STAGES) & 1u;
                        if (!mbar_wait(su32(&bar_full[s]), ph, err)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t a0 = sA0 + s * A_STAGE, b0 = sB0 + s * B_STAGE;
                        const uint64_t dA = sdesc_sw128(a0), dB = sdesc_sw128(b0);
                        switch (pass) {  // every offset, N and column a compile-time constant
                        case 0: issue_pass<0>(dA, dB, tmem, i); break;
                        case 1: issue_pass<1>(dA, dB, tmem, i); break;
                        case 2: issue_pass<2>(dA, dB, tmem, i); break;
                        default: issue_pass<3>(dA, dB, tmem, i); break;
                        }
                        umma_commit(su32(&bar_empty[s]));
                    }
                    if (ok) umma_commit(su32(&bar_tfull));
                }
            }
            // every MMA this thread issued has finished before TMEM is freed
            umma_commit(su32(&bar_done));
            for (uint32_t i = 0; i < kSpinLimit && !mbar_test(su32(&bar_done), 0); ++i) __nanosleep(100);
        }
    } else {
        // ---------------- epilogue: warp w reads TMEM lanes 32 (w % 4) ..,
        // output columns 8 (w / 4) .. + 7
        const int quad = warp & 3, half = warp >> 2;
        uint32_t tl = 0;
        bool ok = true;
        for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
            int j, rt;
            decode(tile, j, rt);
            const OzJob &J = b.job[j];
            const long long row = (long long)rt * BM + quad * 32 + lane;
            const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * 8);
            double tot[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) tot[c] = 0.0;
            for (int pass = 0; pass < NPASS; ++pass, ++tl) {
                const bool got = mbar_wait(su32(&bar_tfull), tl & 1u, err);
                if (!__all_sync(0xffffffffu, got)) {  // warp-uniform: tcgen05.ld is .sync.aligned
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int p0 = pass_p0(pass), p1 = pass_p0(pass + 1);
                // V[t - p0][c] = sum_{p+q=t} S_pq[row][c]: exact integers
                int V[MAX_PASS_T][8];
#pragma unroll
                for (int t = 0; t < MAX_PASS_T; ++t)
#pragma unroll
                    for (int c = 0; c < 8; ++c) V[t][c] = 0;
#pragma unroll
                for (int dp = 0; dp < MAX_PASS_SLICES; ++dp) {  // t - p0 = dp + q is known at compile time
                    const int p = p0 + dp;
                    if (p >= p1) break;
#pragma unroll
                    for (int q = 0; q < NSL; ++q) {
                        if (dp + q >= MAX_PASS_T || q >= nq(p)) break;
                        uint32_t r[8];
                        tmem_ld8(tbase + (uint32_t)(col_off(p) + NB * q), r);
                        tmem_wait_ld();
#pragma unroll
                        for (int c = 0; c < 8; ++c) V[dp + q][c] += __float2int_rn(__uint_as_float(r[c]));
                    }
                }
                // the sums are in registers: hand TMEM back to the issuer
                tc_fence_before();
                mbar_arrive(su32(&bar_tempty));
                double acc[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[c] = 0.0;
#pragma unroll
                for (int t = MAX_PASS_T - 1; t >= 0; --t)  // Horner in 2^-6 over t = p0 + index
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[c] = fma(acc[c], 1.0 / 64.0, (double)V[t][c]);
                const double w = pow2(-6 * p0);
#pragma unroll
                for (int c = 0; c < 8; ++c) tot[c] = fma(acc[c], w, tot[c]);
            }
            if (ok && row < J.rows) {
                const int ei = J.rexp[row];
                double *o = J.out + row * b.ldo;
                for (int c = 0; c < 8; ++c) {
                    const int col = half * 8 + c;
                    if (col < b.ncols) o[col] = tot[c] * pow2(ei + J.cexp[col] - 12);
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ------------------------------------------------------------ digit splits
// Integer digits of x / 2^E rounded to 60 fractional bits, |x| < 2^E.
__device__ __forceinline__ void digits(double x, int E, uint16_t (&d)[NSL]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    const unsigned long long man = (bits & ((1ull << 52) - 1)) | (ex ? (1ull << 52) : 0ull);
    const int sh = (ex ? ex : 1) - 1075 + 60 - E;  // x / 2^E * 2^60 = man * 2^sh, sh <= 7
    unsigned long long q;
    if (sh >= 0) q = man << (sh > 7 ? 7 : sh);
    else if (sh < -62) q = 0ull;
    else q = (man + (1ull << (-sh - 1))) >> (-sh);  // round half up in magnitude
    if (q >> 60) q = (1ull << 60) - 1;              // |x| rounds up to 2^E: keep the digits
    const uint32_t sgn = (uint32_t)(bits >> 63) << 15;
#pragma unroll
    for (int p = 0; p < NSL; ++p) {
        const uint32_t v = (uint32_t)(q >> (6 * (NSL - 1 - p))) & 63u;
        const float f = __uint_as_float(0x4B000000u | v) - 8388608.0f;  // exact small integer
        d[p] = (uint16_t)((__float_as_uint(f) >> 16) | (v ? sgn : 0u));
    }
}


// Rows of X (row-major, ld = K) -> digit tiles.  A block of 256 threads
// owns 8 consecutive rows; in each warp lane = (octet phase << 3) | row, and
// the 8 warps take every 8th group of four K octets; each lane stores the
// 16-byte chunk (8 digits) of one row and octet per slice.  nrt * 128 rows
// are written (zeros past `rows`).
__global__ void __launch_bounds__(256) k_oz_split_rows(const double *X, long long rows, int K, int nkc, int nrt,
                                                       uint8_t *ad, int *rexp, const unsigned long long *rmax) {
    __shared__ double smax[8][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, rr = lane & 7, ph = lane >> 3;
    const long long row = (long long)blockIdx.x * 8 + rr;
    if ((long long)blockIdx.x * 8 >= (long long)nrt * BM) return;
    const bool valid = row < rows;
    const double *xr = X + (valid ? row : 0) * (long long)K;
    const int noct = nkc * (KC / 8);
    double mx = 0.0;
    if (rmax) {
        mx = valid ? __longlong_as_double((long long)rmax[row]) : 0.0;
    } else {
        if (valid)
            for (int oct = ph + 4 * warp; oct * 8 < K; oct += 32)
                for (int e = 0; e < 8 && oct * 8 + e < K; ++e) mx = fmax(mx, fabs(xr[oct * 8 + e]));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 8));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
        if (ph == 0) smax[warp][rr] = mx;
        __syncthreads();
        mx = 0.0;
#pragma unroll
        for (int w = 0; w < 8; ++w) mx = fmax(mx, smax[w][rr]);
    }
    const int E = exp_above(mx);
    if (warp == 0 && ph == 0) rexp[row] = E;
    const int rt = (int)(row / BM), r = (int)(row % BM);
    for (int oct = ph + 4 * warp; oct < noct; oct += 32) {
        uint32_t w[NSL][4];
#pragma unroll
        for (int p = 0; p < NSL; ++p) w[p][0] = w[p][1] = w[p][2] = w[p][3] = 0u;
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int k = oct * 8 + e;
            const double x = (valid && k < K) ? xr[k] : 0.0;
            uint16_t d[NSL];
            digits(x, E, d);
#pragma unroll
            for (int p = 0; p < NSL; ++p) w[p][e >> 1] |= (uint32_t)d[p] << (16 * (e & 1));
        }
        const int kc = oct / (KC / 8), kq = oct % (KC / 8);
        uint8_t *base = ad + ((size_t)rt * nkc + kc) * A_ROW + sw128_off(r, kq * 8);
#pragma unroll
        for (int p = 0; p < NSL; ++p)
            *(uint4 *)(base + (size_t)p * A_TILE) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
    }
}

// Columns of A ([K, ncols] row-major, ld = lda) -> digit tiles (one block).
__global__ void __launch_bounds__(256) k_oz_split_cols(const double *A, int K, int ncols, int lda, int nkc,
                                                       uint8_t *bd, int *cexp) {
    __shared__ double smax[256];
    __shared__ int sE[NB];
    const int tid = threadIdx.x, c = tid % NB;
    double mx = 0.0;
    if (c < ncols)
        for (int k = tid / NB; k < K; k += 256 / NB) mx = fmax(mx, fabs(A[(long long)k * lda + c]));
    smax[tid] = mx;
    __syncthreads();
    if (tid < NB) {
        double m = 0.0;
        for (int i = tid; i < 256; i += NB) m = fmax(m, smax[i]);
        sE[tid] = exp_above(m);
        cexp[tid] = sE[tid];
    }
    __syncthreads();
    for (long long i = tid; i < (long long)nkc * KC * NB; i += 256) {
        const int k = (int)(i / NB), col = (int)(i % NB);
        const double x = (col < ncols && k < K) ? A[(long long)k * lda + col] : 0.0;
        uint16_t d[NSL];
        digits(x, sE[col], d);
        const int kc = k / KC;
        for (int q = 0; q < NSL; ++q) {
            const int row = q * NB + col;
            *(uint16_t *)(bd + (size_t)kc * B_STAGE + sw128_off(row, k % KC)) = d[q];
        }
    }
}

// ------------------------------------------------------------------ host
size_t OzPlan::bytes() const {
    const size_t a = (size_t)nrt * nkc * A_ROW, re = (size_t)nrt * BM * sizeof(int);
    const size_t bb = (size_t)nkc * B_STAGE;
    return (size_t)njob * (a + re + bb + 256) + 256;
}

int oz_gemm_skinny(const OzPlan &pl, const double *const *X, const double *const *A, double *const *T, int lda,
                   int ldt, void *work, cudaStream_t st, const unsigned long long *const *rowmax) {
    if (pl.njob < 1 || pl.njob > 4 || pl.K < 1 || pl.K > kMaxK || pl.ncols < 1 || pl.ncols > NB) return 1;
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess)
            return 2;
        attr_set = true;
    }
    uint8_t *w = (uint8_t *)work;
    int *err = (int *)w;
    w += 256;
    OzBatch b{};
    b.njob = pl.njob;
    b.nkc = pl.nkc;
    b.ncols = pl.ncols;
    b.ldo = ldt;
    cudaMemsetAsync(err, 0, sizeof(int), st);
    for (int j = 0; j < pl.njob; ++j) {
        uint8_t *ad = w;
        w += (size_t)pl.nrt * pl.nkc * A_ROW;
        int *rexp = (int *)w;
        w += (size_t)pl.nrt * BM * sizeof(int);
        uint8_t *bd = w;
        w += (size_t)pl.nkc * B_STAGE;
        int *cexp = (int *)w;
        w += 256;
        k_oz_split_rows<<<(unsigned)((long long)pl.nrt * BM / 8), 256, 0, st>>>(X[j], pl.rows, pl.K, pl.nkc, pl.nrt,
                                                                              ad, rexp, rowmax ? rowmax[j] : nullptr);
        k_oz_split_cols<<<1, 256, 0, st>>>(A[j], pl.K, pl.ncols, lda, pl.nkc, bd, cexp);
        g_launches.fetch_add(2, std::memory_order_relaxed);
        b.job[j] = OzJob{ad, rexp, bd, cexp, T[j], pl.rows, pl.nrt};
    }
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (long long)pl.njob * pl.nrt;
    const unsigned grid = (unsigned)(tiles < sms ? tiles : sms);
    // algorithmic bytes: every digit of X and of A once, the FP64 results once
    const long long abytes = (long long)pl.njob * ((long long)pl.nrt * pl.nkc * A_ROW + (long long)pl.nkc * B_STAGE +
                                                   pl.rows * pl.ncols * (long long)sizeof(double));
    ProfSpan span;
    span.begin("oz_gemm", st, abytes);
    k_oz_gemm<<<grid, THREADS, SMEM_BYTES, st>>>(b, err);
    span.end();
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

int oz_check_error(const void *work, cudaStream_t st) {
    int h = 0;
    if (cudaMemcpyAsync(&h, work, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return 3;
    if (cudaStreamSynchronize(st) != cudaSuccess) return 3;
    return h ? 4 : 0;
}

}  // namespace oz
}  // namespace nvpt
