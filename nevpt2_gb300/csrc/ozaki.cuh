// Split-precision tall-skinny products on tcgen05 (ozaki.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace nvpt {
namespace oz {

constexpr int BM = 128;                // rows per tile (UMMA M)
constexpr int KC = 64;                 // K columns per pipeline stage: one 128-byte swizzle atom per row
constexpr int NSL = 10;                // 6-bit digit slices per operand (60 bits)
constexpr int NB = 16;                 // output columns (padded) per slice
constexpr int NBT = NSL * NB;          // B rows per stage (all q-slices)
constexpr int ROWB = KC * 2;           // bytes of one row of a stage (128)
constexpr int A_TILE = BM * ROWB;      // bytes of one slice of one stage (16 KB)
constexpr int B_STAGE = NBT * ROWB;    // 20 KB
// Digit pairs kept: p + q <= TMAX (p, q < NSL), 64 pairs = 1024 TMEM columns
// of 16.  They run in NPASS passes over K, groups of consecutive slices p
// whose pairs fit TMEM (512 columns).  nq(p) = number of q-slices paired
// with p; one MMA per slice p and K step covers all its q-slices.
constexpr int TMAX = 10;
__host__ __device__ constexpr int nq(int p) { return (TMAX - p + 1) < NSL ? (TMAX - p + 1) : NSL; }
constexpr int NPASS = 4;
__host__ __device__ constexpr int pass_p0(int pass) {  // slices {0,1,2}, {3,4,5}, {6,7}, {8,9}
    return pass == 0 ? 0 : pass == 1 ? 3 : pass == 2 ? 6 : pass == 3 ? 8 : NSL;
}
constexpr int MAX_PASS_SLICES = 3;
constexpr int A_STAGE = MAX_PASS_SLICES * A_TILE;  // 48 KB
constexpr int STAGES = 3;
constexpr int EPI_WARPS = 8;           // two per TMEM lane quadrant, 8 output columns each
constexpr int THREADS = 32 * (EPI_WARPS + 2);
// Operand tiles in shared memory (and in HBM) are K-major with the 128-byte
// swizzle: row r of a tile occupies bytes [128 r, 128 r + 128), its 16-byte
// chunk c stored at chunk c ^ (r mod 8); 8-row groups are 1024 bytes apart.
constexpr int SBO_SW = 1024;
constexpr int TMEM_COLS = 512;
constexpr int SMEM_BYTES = STAGES * (A_STAGE + B_STAGE) + 1024;  // + 1 KB for aligning the base
constexpr int kMaxK = 4096;      // exact FP32 digit sums need 63*63*K < 2^24

struct OzJob {
    const uint8_t *ad;  // X digit tiles [nrt][nkc][NSL][A_TILE]
    const int *rexp;    // [nrt * BM]
    const uint8_t *bd;  // A digit tiles [nkc][B_STAGE]
    const int *cexp;    // [NB]
    double *out;        // [rows][ldo]
    long long rows;
    int nrt;
};
struct OzBatch {
    OzJob job[4];
    int njob, nkc, ncols, ldo;
};

// Up to four products T_j = X_j A_j with the same shapes: X_j [rows, K]
// (row-major, ld = K), A_j [K, ncols] (ld = lda), T_j [rows, ncols] (ld = ldt).
struct OzPlan {
    int njob = 1;
    long long rows = 0;
    int K = 0, ncols = 0, nkc = 0, nrt = 0;
    OzPlan(int nj, long long r, int k, int nc)
        : njob(nj), rows(r), K(k), ncols(nc), nkc((k + KC - 1) / KC), nrt((int)((r + BM - 1) / BM)) {}
    size_t bytes() const;  // device workspace
};

// Enqueue digit splits + the tensor-core product on `st`.  work: bytes()
// of device memory (16-byte aligned).  0 on success; nonzero for bad shapes
// or launch failure.  The kernel's own error flag (a wait that timed out) is
// read back by oz_check_error (synchronises `st`; 0 = fine, 4 = timeout).
// rowmax (optional): per product, max_k |X[i,k]| of every row as the bit
// pattern of the double (the split then skips its own pass over X).
int oz_gemm_skinny(const OzPlan &pl, const double *const *X, const double *const *A, double *const *T, int lda,
                   int ldt, void *work, cudaStream_t st, const unsigned long long *const *rowmax = nullptr);
int oz_check_error(const void *work, cudaStream_t st);

// General products (ozaki_wide.cu): C[m, n] (row-major, ldc) =
// alpha X Y + beta C for FP64 operands of any shape, X[i, k] =
// A[i * a_r + k * a_k] (i < m, k < K), Y[k, j] = B[j * b_c + k * b_k].
// alpha must be a power of two times +-1 (it is folded into the column
// exponents).  lower: only the output tiles that meet the lower triangle
// (j <= i) are formed (symmetric products; the caller mirrors).
struct WideGemm {
    long long m = 0, n = 0;
    int K = 0;
    const double *A = nullptr;
    long long a_r = 0, a_k = 0;
    const double *B = nullptr;
    long long b_c = 0, b_k = 0;
    double alpha = 1.0, beta = 0.0;
    double *C = nullptr;
    long long ldc = 0;
    bool lower = false;
    bool c_trans = false;  // store C^T: element (i, j) at C[j * ldc + i]
};
constexpr int kWideMaxK = 1 << 19;  // keeps the 64-bit drain sums in range
size_t oz_wide_bytes(long long m, long long n, int K);  // device workspace (16-byte aligned)
// Enqueue on `st`; 0 on success, 1 bad arguments, 3 launch failure.  A wait
// that timed out sets the int at err (device memory, not reset here).
int oz_gemm_wide(const WideGemm &g, void *work, int *err, cudaStream_t st);

}  // namespace oz
}  // namespace nvpt
