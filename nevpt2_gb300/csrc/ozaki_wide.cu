// Split-precision (Ozaki) general products C = alpha X Y + beta C on the
// 5th-generation tensor cores, for FP64 operands of any shape (the dense
// contractions of the NEVPT2 energy stage in split mode).
//
// Scheme.  Row i of X is scaled by 2^-E_i, E_i one above the smallest power
// of two over max_k |X[i,k]| (so |X[i,k]| < 2^(E_i - 1)), rounded to 60
// fractional bits and written as ten BALANCED base-64 digits,
//   X[i,k] ~ 2^(E_i - 60) sum_p d_p 64^(9-p),   d_p in [-32, 32],
// each an exact BF16; columns of Y likewise with exponents F_j.  For the
// digit pairs with p + q = t <= 10 the tensor cores accumulate in FP32
//   V_t = sum_{p+q=t} sum_k d_p e_q,
// all pairs of one weight t into one TMEM block.  |d_p e_q| <= 2^10 and at
// most ten pairs share a weight, so a block stays an exact integer below
// 2^24 over 1536 columns of K; the epilogue drains the blocks into 64-bit
// integers every 1536 columns (once for K <= 1536):
//   hi = sum_{t<=4} V_t 2^(6(4-t)),  lo = sum_{t>=5} V_t 2^(6(10-t)),
//   C[i,j] = 2^(E_i+F_j-36) hi + 2^(E_i+F_j-72) lo   (+ beta C).
// The error is the rounding of the operands to 60 bits (at most 2^-59 of
// max|X_i| max|Y_j| per term) plus the dropped weights t > 10 (below 2^-64
// per term): at or below the rounding of an FP64 dot product.
//
// Kernel.  Persistent, one CTA per SM, 320 threads.  An output tile is 128
// rows x 32 columns; its 11 weight blocks take 352 TMEM columns.  Warp 8
// streams digit tiles global -> shared with bulk copies (a K chunk of 64:
// the ten 16 KB row-digit slices into an 8-slot ring, the 40 KB of
// column digits into a 2-slot ring); warp 9 issues, per chunk, slice p and
// K step, one tcgen05.mma (M = 128, K = 16) whose B operand is the stack of
// the column slices q paired with p (N = 32 per q, split at N = 256), so
// that pair (p, q) lands in block p + q; warps 0-7 drain the blocks with
// tcgen05.ld and recombine.  Operand tiles are K-major with the 128-byte
// swizzle, written in that layout by the split kernels.  Tiles are
// rastered in groups of 16 row tiles sharing a column tile, so the digit
// tiles in flight stay in L2.  Every wait is bounded: a timeout sets the
// error flag and the kernel winds down.
#include <cstdint>

#include "nvpt2_internal.h"
#include "oz_ptx.cuh"
#include "ozaki.cuh"
#include "tuner.h"

namespace nvpt {
namespace oz {

namespace {

constexpr int NT = 32;                     // output columns per tile
constexpr int B_TILE = NT * ROWB;          // 4 KB: one slice of one K chunk of a column tile
constexpr int B_CHUNK = NSL * B_TILE;      // 40 KB
constexpr int A_SLOTS = 8, B_SLOTS = 2;
constexpr int NWT = TMAX + 1;              // weight blocks t = p + q
constexpr int DRAIN_KC = 24;               // K chunks between drains (1536 columns)
constexpr int GM_DEFAULT = 16;             // row tiles per raster group (tuned per shape)
constexpr int W_THREADS = 32 * (EPI_WARPS + 2);
constexpr int W_SMEM = A_SLOTS * A_TILE + B_SLOTS * B_CHUNK + 1024;
static_assert(NWT * NT <= TMEM_COLS, "weight blocks fit TMEM");
static_assert(10 * 1024 * DRAIN_KC * KC < (1 << 24), "a drained block is an exact FP32 integer");
static_assert(W_SMEM <= 227 * 1024, "shared memory");

// MMA pieces of slice p: (first q, number of q) with N = 32 nq <= 256.  The
// piece that first touches block 10 (p = 1, q = 9) is separate, so that the
// first K step of a drain period can overwrite (not accumulate) exactly the
// blocks each piece initialises: p = 0 covers blocks 0..9, then (1, 9)
// block 10.
__host__ __device__ constexpr int npieces(int p) { return p == 0 ? 2 : p == 1 ? 3 : p == 2 ? 2 : 1; }
__host__ __device__ constexpr int piece_q0(int p, int i) { return p <= 2 ? (i == 0 ? 0 : 8 + (i - 1)) : 0; }
__host__ __device__ constexpr int piece_nq(int p, int i) {
    return p == 0 ? (i == 0 ? 8 : 2) : p == 1 ? (i == 0 ? 8 : 1) : p == 2 ? (i == 0 ? 8 : 1) : nq(p);
}
__host__ __device__ constexpr bool piece_init(int p, int i) { return p == 0 || (p == 1 && i == 2); }
__host__ __device__ constexpr bool pieces_ok() {
    for (int p = 0; p < NSL; ++p) {
        int covered = 0;
        for (int i = 0; i < npieces(p); ++i) {
            if (piece_q0(p, i) != covered) return false;
            if (piece_nq(p, i) * NT > 256 || piece_nq(p, i) < 1) return false;
            covered += piece_nq(p, i);
        }
        if (covered != nq(p)) return false;
    }
    return TMAX == 10 && NSL == 10;
}
static_assert(pieces_ok(), "MMA pieces cover every pair exactly once");

template <int P>
__device__ __forceinline__ void issue_slice(uint64_t dA, uint64_t dB, uint32_t tmem, bool fresh) {
#pragma unroll
    for (int kk = 0; kk < KC / 16; ++kk) {
#pragma unroll
        for (int i = 0; i < npieces(P); ++i) {
            const int q0 = piece_q0(P, i), n = piece_nq(P, i);
            const uint32_t acc = (fresh && kk == 0 && piece_init(P, i)) ? 0u : 1u;
            const uint64_t da = dA + (uint64_t)((kk * 32) >> 4);
            const uint64_t db = dB + (uint64_t)((q0 * B_TILE + kk * 32) >> 4);
            umma(tmem + (uint32_t)(NT * (P + q0)), da, db, idesc_bf16(NT * n), acc);
        }
    }
}

struct WideArgs {
    const uint8_t *ad;  // row digits   [nrt][nkc][NSL][A_TILE]
    const uint8_t *bd;  // column digits [nct][nkc][NSL][B_TILE]
    const int *rexp, *cexp;
    double *C;
    long long ldc, m, n;
    int nrt, nct, nkc, lower, ctrans;
    double beta;
    int gm;  // row tiles per raster group
};

// Tile t -> (row tile, column tile): groups of gm row tiles, column tiles
// outer within a group, so consecutive CTAs share a column tile.
__device__ __forceinline__ void tile_rc(const WideArgs &a, long long t, int &rt, int &ct) {
    const long long per = (long long)a.gm * a.nct;
    const long long g = t / per, r = t % per;
    const int rows_in = (int)min((long long)a.gm, (long long)a.nrt - g * a.gm);
    ct = (int)(r / rows_in);
    rt = (int)(g * a.gm + r % rows_in);
}
// lower: skip tiles entirely above the diagonal (every column > every row)
__device__ __forceinline__ bool tile_skip(const WideArgs &a, int rt, int ct) {
    return a.lower && (long long)ct * NT > (long long)rt * BM + (BM - 1);
}
__device__ __forceinline__ double scale2(double v, int e) {
    return (e >= -1022 && e <= 1023) ? v * pow2(e) : ldexp(v, e);
}
__device__ __forceinline__ int kc_first(long long tile, int nkc) { return (int)((tile * 7) % nkc); }

__global__ void __launch_bounds__(W_THREADS, 1) k_oz_wide(WideArgs a, int *err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t a_full[A_SLOTS], a_empty[A_SLOTS], b_full[B_SLOTS], b_empty[B_SLOTS];
    __shared__ __align__(8) uint64_t t_full, t_empty, done;
    __shared__ uint32_t s_tmem;
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sA0 = su32(smem), sB0 = sA0 + A_SLOTS * A_TILE;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int PRODUCER = EPI_WARPS, ISSUER = EPI_WARPS + 1;
    const long long ntiles = (long long)a.nrt * a.nct;
    const int ndrain = (a.nkc + DRAIN_KC - 1) / DRAIN_KC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < A_SLOTS; ++s) {
            mbar_init(su32(&a_full[s]), 1);
            mbar_init(su32(&a_empty[s]), 1);
        }
        for (int s = 0; s < B_SLOTS; ++s) {
            mbar_init(su32(&b_full[s]), 1);
            mbar_init(su32(&b_empty[s]), 1);
        }
        mbar_init(su32(&t_full), 1);
        mbar_init(su32(&t_empty), 32 * EPI_WARPS);
        mbar_init(su32(&done), 1);
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

    if (warp == PRODUCER) {
        if (lane == 0) {
            uint32_t ia = 0, ib = 0;
            bool ok = true;
            for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                int rt, ct;
                tile_rc(a, tile, rt, ct);
                if (tile_skip(a, rt, ct)) continue;
                const int k0 = kc_first(tile, a.nkc);
                for (int i = 0; i < a.nkc && ok; ++i) {
                    const int kc = (k0 + i) % a.nkc;
                    const uint32_t sb = ib % B_SLOTS, pb = (ib / B_SLOTS) & 1u;
                    if (!mbar_wait(su32(&b_empty[sb]), pb ^ 1u, err)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(su32(&b_full[sb]), B_CHUNK);
                    bulk_g2s(sB0 + sb * B_CHUNK, a.bd + ((size_t)ct * a.nkc + kc) * B_CHUNK, B_CHUNK,
                             su32(&b_full[sb]));
                    ++ib;
                    for (int p = 0; p < NSL; ++p, ++ia) {
                        const uint32_t sa = ia % A_SLOTS, pa = (ia / A_SLOTS) & 1u;
                        if (!mbar_wait(su32(&a_empty[sa]), pa ^ 1u, err)) {
                            ok = false;
                            break;
                        }
                        mbar_expect_tx(su32(&a_full[sa]), A_TILE);
                        bulk_g2s(sA0 + sa * A_TILE, a.ad + (((size_t)rt * a.nkc + kc) * NSL + p) * A_TILE, A_TILE,
                                 su32(&a_full[sa]));
                    }
                }
            }
            // copies still in flight land on the full barriers of the last
            // slots issued: wait for them (bounded) before exiting
            const uint32_t fa = ia > (uint32_t)A_SLOTS ? ia - A_SLOTS : 0u;
            for (uint32_t k = fa; k < ia; ++k)
                for (uint32_t i = 0; i < kSpinLimit && !mbar_test(su32(&a_full[k % A_SLOTS]), (k / A_SLOTS) & 1u); ++i)
                    __nanosleep(100);
            const uint32_t fb = ib > (uint32_t)B_SLOTS ? ib - B_SLOTS : 0u;
            for (uint32_t k = fb; k < ib; ++k)
                for (uint32_t i = 0; i < kSpinLimit && !mbar_test(su32(&b_full[k % B_SLOTS]), (k / B_SLOTS) & 1u); ++i)
                    __nanosleep(100);
        }
    } else if (warp == ISSUER) {
        if (lane == 0) {
            uint32_t ia = 0, ib = 0, nd = 0;
            bool ok = true;
            for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                int rt, ct;
                tile_rc(a, tile, rt, ct);
                if (tile_skip(a, rt, ct)) continue;
                for (int i = 0; i < a.nkc && ok; ++i) {
                    const bool fresh = (i % DRAIN_KC) == 0;
                    if (fresh) {
                        if (!mbar_wait(su32(&t_empty), (nd & 1u) ^ 1u, err)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
                    const uint32_t sb = ib % B_SLOTS, pb = (ib / B_SLOTS) & 1u;
                    if (!mbar_wait(su32(&b_full[sb]), pb, err)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t dB = sdesc_sw128(sB0 + sb * B_CHUNK);
                    for (int p = 0; p < NSL; ++p, ++ia) {
                        const uint32_t sa = ia % A_SLOTS, pa = (ia / A_SLOTS) & 1u;
                        if (!mbar_wait(su32(&a_full[sa]), pa, err)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint64_t dA = sdesc_sw128(sA0 + sa * A_TILE);
                        switch (p) {  // offsets, N and TMEM columns are compile-time constants
                        case 0: issue_slice<0>(dA, dB, tmem, fresh); break;
                        case 1: issue_slice<1>(dA, dB, tmem, fresh); break;
                        case 2: issue_slice<2>(dA, dB, tmem, fresh); break;
                        case 3: issue_slice<3>(dA, dB, tmem, fresh); break;
                        case 4: issue_slice<4>(dA, dB, tmem, fresh); break;
                        case 5: issue_slice<5>(dA, dB, tmem, fresh); break;
                        case 6: issue_slice<6>(dA, dB, tmem, fresh); break;
                        case 7: issue_slice<7>(dA, dB, tmem, fresh); break;
                        case 8: issue_slice<8>(dA, dB, tmem, fresh); break;
                        default: issue_slice<9>(dA, dB, tmem, fresh); break;
                        }
                        umma_commit(su32(&a_empty[sa]));
                    }
                    if (!ok) break;
                    umma_commit(su32(&b_empty[sb]));
                    ++ib;
                    if ((i % DRAIN_KC) == DRAIN_KC - 1 || i == a.nkc - 1) {
                        umma_commit(su32(&t_full));
                        ++nd;
                    }
                }
            }
            umma_commit(su32(&done));
            for (uint32_t i = 0; i < kSpinLimit && !mbar_test(su32(&done), 0); ++i) __nanosleep(100);
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (tile rows),
        // output columns 16 (w / 4) .. + 15 of every weight block
        const int quad = warp & 3, half = warp >> 2;
        uint32_t nd = 0;
        bool ok = true;
        for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
            int rt, ct;
            tile_rc(a, tile, rt, ct);
            if (tile_skip(a, rt, ct)) continue;
            const uint32_t tbase = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * 16);
            long long hi[16], lo[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) hi[c] = lo[c] = 0;
            for (int d = 0; d < ndrain; ++d, ++nd) {
                const bool got = mbar_wait(su32(&t_full), nd & 1u, err);
                if (!__all_sync(0xffffffffu, got)) {  // warp-uniform: tcgen05.ld is .sync.aligned
                    ok = false;
                    break;
                }
                tc_fence_after();
#pragma unroll
                for (int t = 0; t < NWT; ++t) {
                    uint32_t r[16];
                    tmem_ld16(tbase + (uint32_t)(NT * t), r);
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        const long long v = (long long)__float2int_rn(__uint_as_float(r[c]));
                        if (t <= 4) hi[c] += v * (1ll << (6 * (4 - t)));
                        else lo[c] += v * (1ll << (6 * (10 - t)));
                    }
                }
                tc_fence_before();
                mbar_arrive(su32(&t_empty));
            }
            if (!ok) break;
            const long long row = (long long)rt * BM + quad * 32 + lane;
            if (row < a.m) {
                const int ei = a.rexp[row];
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const long long col = (long long)ct * NT + half * 16 + c;
                    if (col < a.n) {
                        const int e = ei + a.cexp[col];
                        double v = scale2((double)hi[c], e - 36) + scale2((double)lo[c], e - 72);
                        double *o = a.ctrans ? a.C + col * a.ldc + row : a.C + row * a.ldc + col;
                        if (a.beta != 0.0) v = fma(a.beta, *o, v);
                        *o = v;
                    }
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
// Balanced base-64 digits of x 2^-E rounded to 60 fractional bits, for
// |x| < 2^(E-1):  x ~ 2^(E-60) sum_p d_p 64^(9-p),  d_p in [-32, 32].
__device__ __forceinline__ void digits_bal(double x, int E, int (&d)[NSL]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    const unsigned long long man = (bits & ((1ull << 52) - 1)) | (ex ? (1ull << 52) : 0ull);
    const int sh = (ex ? ex : 1) - 1075 + 60 - E;  // |x| 2^(60-E) = man 2^sh < 2^59, so sh <= 6
    unsigned long long q;
    if (sh >= 0) q = man << (sh > 6 ? 6 : sh);
    else if (sh < -62) q = 0ull;
    else q = (man + (1ull << (-sh - 1))) >> (-sh);  // round half up in magnitude: q <= 2^59
    long long z = (bits >> 63) ? -(long long)q : (long long)q;
#pragma unroll
    for (int p = NSL - 1; p > 0; --p) {
        int r = (int)(z & 63);
        if (r >= 32) r -= 64;
        d[p] = r;
        z = (z - r) >> 6;
    }
    d[0] = (int)z;  // |z| <= 32: the top digit takes what is left
}
__device__ __forceinline__ uint16_t bf16_of_int(int v) {  // exact for |v| <= 256
    return (uint16_t)(__float_as_uint((float)v) >> 16);
}

// Exponents of the rows of an operand (element (r, k) at src[r sr + k sk]
// times `scale`): ex[r] = E with max_k |x| < 2^(E-1).  32 rows per block.
__global__ void __launch_bounds__(256) k_wide_exp(const double *src, long long sr, long long sk, long long rows, int K,
                                                  double scale, int *ex) {
    __shared__ double sm[8][33];
    const long long r0 = (long long)blockIdx.x * 32;
    const int tid = threadIdx.x;
    double mx = 0.0;
    int r, kl;
    if (sk == 1) {  // k contiguous: a warp sweeps k of four rows
        r = (tid >> 5) * 4;
        kl = tid & 31;
        for (int j = 0; j < 4; ++j) {
            double m = 0.0;
            if (r0 + r + j < rows)
                for (int k = kl; k < K; k += 32) m = fmax(m, fabs(src[(r0 + r + j) * sr + k]));
            for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (kl == 0) sm[0][r + j] = m;
        }
        __syncthreads();
        if (tid < 32 && r0 + tid < rows) ex[r0 + tid] = exp_above(sm[0][tid] * fabs(scale)) + 1;
        return;
    }
    r = tid & 31;
    kl = tid >> 5;
    if (r0 + r < rows)
        for (int k = kl; k < K; k += 8) mx = fmax(mx, fabs(src[(r0 + r) * sr + (long long)k * sk]));
    sm[kl][r] = mx;
    __syncthreads();
    if (tid < 32) {
        double m = 0.0;
        for (int j = 0; j < 8; ++j) m = fmax(m, sm[j][tid]);
        if (r0 + tid < rows) ex[r0 + tid] = exp_above(m * fabs(scale)) + 1;
    }
}

// Digit tiles of an operand: tile (row tile of `tr` rows, K chunk, slice)
// at out + ((rtile * nkc + kc) * NSL + p) * tr * ROWB, 128-byte-swizzled
// K-major; rows and K past the ends are zero.  Block: 32 rows x one K chunk.
__global__ void __launch_bounds__(256) k_wide_split(const double *src, long long sr, long long sk, long long rows,
                                                    int K, double scale, int tr, int nkc, const int *ex, uint8_t *out) {
    __shared__ double t[32][KC + 1];
    const long long r0 = (long long)blockIdx.x * 32;
    const int kc = blockIdx.y, k0 = kc * KC, tid = threadIdx.x;
    for (int i = tid; i < 32 * KC; i += 256) {
        int r, k;
        if (sk == 1) { r = i / KC; k = i % KC; }
        else { r = i % 32; k = i / 32; }
        const long long row = r0 + r;
        t[r][k] = (row < rows && k0 + k < K) ? src[row * sr + (long long)(k0 + k) * sk] * scale : 0.0;
    }
    __syncthreads();
    const int r = tid >> 3, oct = tid & 7;
    const long long row = r0 + r;
    const int E = row < rows ? ex[row] : 0;
    uint32_t w[NSL][4];
#pragma unroll
    for (int p = 0; p < NSL; ++p) w[p][0] = w[p][1] = w[p][2] = w[p][3] = 0u;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        int d[NSL];
        digits_bal(t[r][oct * 8 + e], E, d);
#pragma unroll
        for (int p = 0; p < NSL; ++p) w[p][e >> 1] |= (uint32_t)bf16_of_int(d[p]) << (16 * (e & 1));
    }
    const long long rtile = row / tr;
    const int rr = (int)(row % tr);
    uint8_t *base = out + (((size_t)rtile * nkc + kc) * NSL) * (size_t)tr * ROWB + sw128_off(rr, oct * 8);
#pragma unroll
    for (int p = 0; p < NSL; ++p)
        *(uint4 *)(base + (size_t)p * tr * ROWB) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
}

struct WideLayout {
    int nrt, nct, nkc;
    size_t a_bytes, b_bytes, re_bytes, ce_bytes;
    WideLayout(long long m, long long n, int K)
        : nrt((int)((m + BM - 1) / BM)), nct((int)((n + NT - 1) / NT)), nkc((K + KC - 1) / KC) {
        a_bytes = (size_t)nrt * nkc * NSL * A_TILE;
        b_bytes = (size_t)nct * nkc * B_CHUNK;
        re_bytes = ((size_t)nrt * BM * sizeof(int) + 255) & ~(size_t)255;
        ce_bytes = ((size_t)nct * NT * sizeof(int) + 255) & ~(size_t)255;
    }
    size_t total() const { return a_bytes + b_bytes + re_bytes + ce_bytes; }
};

}  // namespace

size_t oz_wide_bytes(long long m, long long n, int K) { return WideLayout(m, n, K).total(); }

int oz_gemm_wide(const WideGemm &g, void *work, int *err, cudaStream_t st) {
    if (g.m < 0 || g.n < 0 || g.K < 0 || g.K > kWideMaxK || !err) return 1;
    if (g.m == 0 || g.n == 0) return 0;
    if (g.K == 0 || g.alpha == 0.0) return 1;  // callers handle the degenerate products
    {   // alpha = +-2^a exactly
        int e;
        const double f = frexp(fabs(g.alpha), &e);
        if (f != 0.5) return 1;
    }
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(k_oz_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, W_SMEM) != cudaSuccess)
            return 3;
        attr_set = true;
    }
    const WideLayout L(g.m, g.n, g.K);
    uint8_t *w = (uint8_t *)work;
    uint8_t *ad = w, *bd = w + L.a_bytes;
    int *rexp = (int *)(bd + L.b_bytes), *cexp = (int *)((uint8_t *)rexp + L.re_bytes);
    // rows of X; columns of Y carry alpha
    k_wide_exp<<<(unsigned)((g.m + 31) / 32), 256, 0, st>>>(g.A, g.a_r, g.a_k, g.m, g.K, 1.0, rexp);
    k_wide_exp<<<(unsigned)((g.n + 31) / 32), 256, 0, st>>>(g.B, g.b_c, g.b_k, g.n, g.K, g.alpha, cexp);
    k_wide_split<<<dim3((unsigned)((long long)L.nrt * BM / 32), (unsigned)L.nkc), 256, 0, st>>>(
        g.A, g.a_r, g.a_k, g.m, g.K, 1.0, BM, L.nkc, rexp, ad);
    k_wide_split<<<dim3((unsigned)((long long)L.nct * NT / 32), (unsigned)L.nkc), 256, 0, st>>>(
        g.B, g.b_c, g.b_k, g.n, g.K, g.alpha, NT, L.nkc, cexp, bd);
    g_launches.fetch_add(4, std::memory_order_relaxed);
    WideArgs a{ad, bd, rexp, cexp, g.C, g.ldc, g.m, g.n, L.nrt, L.nct, L.nkc, g.lower ? 1 : 0, g.c_trans ? 1 : 0,
               g.beta, GM_DEFAULT};
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (long long)L.nrt * L.nct;
    const unsigned grid = (unsigned)(tiles < sms ? tiles : sms);
    // recorded work: the FP64 flops of the product (2 m n K); the tensor
    // cores run 64 BF16 digit products of that size
    auto run = [&](int gm) {
        a.gm = gm;
        ProfSpan span;
        span.begin("oz_wide", st, 2 * g.m * g.n * (long long)g.K);
        k_oz_wide<<<grid, W_THREADS, W_SMEM, st>>>(a, err);
        span.end();
        g_launches.fetch_add(1, std::memory_order_relaxed);
    };
    // raster group: tuned per shape when the product overwrites C (beta = 0:
    // every trial writes the same result)
    static const int kGm[] = {4, 8, 16, 32};
    const std::string key = "oz_wide.raster_rows/" + std::to_string(L.nrt) + "x" + std::to_string(L.nct) + "x" +
                            std::to_string(L.nkc) + (g.lower ? "L" : "");
    const int cached = tune::lookup(key);
    if (cached >= 0 || g.beta != 0.0) {
        run(cached >= 0 ? cached : GM_DEFAULT);
    } else {
        int used = -1;
        const int gm = tune::choose(key, kGm, 4, GM_DEFAULT, st, [&](int c) { run(c); used = c; });
        if (used < 0) run(gm);  // tuning off: nothing launched yet
    }
    return cudaGetLastError() == cudaSuccess ? 0 : 3;
}

}  // namespace oz
}  // namespace nvpt
