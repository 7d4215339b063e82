// Split-precision tall-skinny products on tcgen05 (ozaki.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace nvpt {
namespace oz {

constexpr int BM = 128;                // rows per tile (UMMA M)
constexpr int KC = 32;                 // K columns per pipeline stage
constexpr int NSL = 9;                 // 6-bit digit slices per operand (54 bits)
constexpr int NB = 16;                 // output columns (padded) per slice
constexpr int NBT = NSL * NB;          // B rows per stage (all q-slices)
constexpr int A_TILE = BM * KC * 2;    // bytes of one slice of one stage
constexpr int B_STAGE = NBT * KC * 2;  // 9216
// The digit pairs (p, q), p + q <= NSL - 1, need 720 TMEM columns; they run
// in two passes over K, p in [0,4) (480 columns) and p in [4,9) (240).
constexpr int NPASS = 2;
constexpr int PASS_SPLIT = 4;  // first slice of the second pass
__host__ __device__ constexpr int pass_p0(int pass) { return pass == 0 ? 0 : pass == 1 ? PASS_SPLIT : NSL; }
constexpr int MAX_PASS_SLICES = 5;
constexpr int A_STAGE = MAX_PASS_SLICES * A_TILE;  // 40960
constexpr int STAGES = 4;
constexpr int LBO_A = BM * 16;   // next 8-column K octet
constexpr int LBO_B = NBT * 16;
constexpr int SBO = 128;         // next 8-row group
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
int oz_gemm_skinny(const OzPlan &pl, const double *const *X, const double *const *A, double *const *T, int lda,
                   int ldt, void *work, cudaStream_t st);
int oz_check_error(const void *work, cudaStream_t st);

}  // namespace oz
}  // namespace nvpt
