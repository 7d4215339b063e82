// Device tensor toolkit for the NEVPT2 energy stage.
//
// Tensors are dense, C-ordered (last index fastest) FP64 arrays with up to 6
// axes.  The stage-2 algebra is expressed with a few primitives: an axis
// permutation (materialised), the accessor builders of the reference's
// qdnevpt-local normal-ordered products (src/qdnevpt.F:6448-6519), dense
// GEMMs (cuBLAS FP64, or split-precision digit products on the tensor cores
// in split mode), symmetric eigendecompositions (cuSOLVER syevd) and, for
// the order-n^3 pencils, Cholesky + reduction to standard form + the device
// tridiagonalisation (tridiag.cu).  All work of one context is enqueued on
// its stream; allocations are stream-ordered.
#pragma once
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <array>
#include <stdexcept>
#include <string>
#include <vector>

#include "nvpt2_internal.h"

namespace nvpt {
namespace s2 {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(e == cudaErrorMemoryAllocation ? 3 : 2, std::string(what) + ": " + cudaGetErrorString(e));
}
inline void ck(cublasStatus_t e, const char *what) {
    if (e != CUBLAS_STATUS_SUCCESS) throw Error(2, std::string(what) + ": cuBLAS status " + std::to_string((int)e));
}
inline void ck(cusolverStatus_t e, const char *what) {
    if (e != CUSOLVER_STATUS_SUCCESS) throw Error(2, std::string(what) + ": cuSOLVER status " + std::to_string((int)e));
}

// Owning device tensor (stream-ordered allocation), or a non-owning view of
// one (T::view) that never frees.
struct T {
    double *p = nullptr;
    int nd = 0;
    std::array<long long, 6> sh{{1, 1, 1, 1, 1, 1}};
    cudaStream_t st = nullptr;
    bool own = true;
    T() = default;
    T(const T &) = delete;
    T &operator=(const T &) = delete;
    T(T &&o) noexcept { *this = std::move(o); }
    T &operator=(T &&o) noexcept {
        release();
        p = o.p; nd = o.nd; sh = o.sh; st = o.st; own = o.own;
        o.p = nullptr;
        return *this;
    }
    ~T() { release(); }
    static T view(const T &o) {
        T v;
        v.p = o.p; v.nd = o.nd; v.sh = o.sh; v.st = o.st; v.own = false;
        return v;
    }
    void release() {
        if (p && own) cudaFreeAsync(p, st);
        p = nullptr;
    }
    long long size() const {
        long long s = 1;
        for (int i = 0; i < nd; ++i) s *= sh[i];
        return s;
    }
    long long dim(int i) const { return sh[i]; }
};

struct Ctx {
    cudaStream_t st;
    cublasHandle_t blas;
    cusolverDnHandle_t sol;
    // Split precision: large GEMMs (and Gram matrices) run as Ozaki digit
    // products on the tensor cores; a pipeline timeout sets *oz_err.
    bool split = false;
    int *oz_err = nullptr;
    // Order-n^3 pencils tridiagonalised at the same time on other streams:
    // each takes 1/sm_share of the SMs (at most 4), so that they overlap.
    int sm_share = 1;
    // Polls a device-side wait (grid barrier) makes before it gives up and
    // the call reports NVPT_ETIMEDOUT; 0 = the built-in limit.
    unsigned wait_limit = 0;
    // Resolvents (no eigenvectors) for every PC class whose metric keeps all
    // its eigenvalues, not only the order-n^3 pencils of the (+-1') classes.
    bool all_pc_resolvent = false;
};

T alloc(Ctx &c, std::initializer_list<long long> shape, bool zero = true);
T alloc_v(Ctx &c, const std::vector<long long> &shape, bool zero = true);
// Non-owning 1-D view helpers are plain pointers.

// out = alpha * permute(in, axes) (+ out if accumulate).  `in` has shape
// in_shape (C order); axes as numpy.transpose.
void permute(Ctx &c, const double *in, const std::vector<long long> &in_shape, const std::vector<int> &axes,
             double *out, double alpha = 1.0, bool accumulate = false);
T permuted(Ctx &c, const T &in, const std::vector<int> &axes, double alpha = 1.0);

// Gather of a strided sub-block: out[i0..] = in[off + sum i_k * stride_k],
// out C-ordered with shape `shape`.
void gather(Ctx &c, const double *in, long long off, const std::vector<long long> &shape,
            const std::vector<long long> &stride, double *out, double alpha = 1.0, bool accumulate = false);

// Row-major GEMM: C[m,n] = alpha op(A)[m,k] op(B)[k,n] + beta C.
void gemm(Ctx &c, bool ta, bool tb, long long m, long long n, long long k, double alpha, const double *A, long long lda,
          const double *B, long long ldb, double beta, double *C, long long ldc);
void gemm_batched(Ctx &c, bool ta, bool tb, long long m, long long n, long long k, double alpha, const double *A,
                  long long lda, long long sA, const double *B, long long ldb, long long sB, double beta, double *C,
                  long long ldc, long long sC, long long batch);

// Symmetric eigendecomposition of the matrix whose upper triangle (row <=
// col) is held in A (n x n, row-major), as dsyev('V','U') of the reference
// sees it.  w ascending; V[k][i] = component i of eigenvector k.
void eigh_upper(Ctx &c, const double *A, long long n, double *w, double *V);
// out[m,m] (row-major) = X^T X for X [Q, m] row-major: the symmetric rank-Q
// update (cublasDsyrk, half the flops of a GEMM) mirrored to a full matrix.
void gram(Ctx &c, const double *X, long long Q, long long m, double *out);
// True if every eigenvalue of the symmetric matrix (upper triangle of A) is
// above thr: a Cholesky factorisation of A - thr I succeeds.
bool metric_above(Ctx &c, const double *A, long long n, double thr);
// Raise kernel's dynamic shared-memory limit to the most the current device
// allows next to its static shared memory, and return that limit.  The value
// is the same for every caller, so host threads launching the kernel with
// different sizes concurrently cannot undercut one another's launches.
int raise_dynamic_smem(const void *kernel);
// Generalised symmetric-definite eigenproblem K v = w S v (upper triangles;
// cusolverDnDsygvd): w ascending, V[k][i] = component i of eigenvector k,
// eigenvectors S-orthonormal.  False if S is not positive definite.
bool sygvd_upper(Ctx &c, const double *K, const double *S, long long n, double *w, double *V);
// Symmetric copy: out = triu(A) + triu(A,1)^T.
void symmetrize_upper(Ctx &c, const double *A, long long n, double *out);

// The pencil K v = w S v in tridiagonal form, without its eigenvectors:
// S = U^T U (Cholesky of the symmetric view of S), K~ = U^-T K U^-1 (K's
// symmetric view), K~ = Q T Q^T (Householder).  T: diagonal d[n],
// off-diagonal e[n-1].  U, Q (reflectors + tau) stay in the struct, which
// then maps right-hand sides into T's basis.  False if S is not positive
// definite.
struct PencilTridiag {
    T U, A, d, e, tau;  // U: column-major upper factor; A: reflectors of Q
    long long n = 0;
};
bool pencil_tridiag(Ctx &c, const double *K, const double *S, long long n, PencilTridiag &P);
// Upper triangle of A (column-major, symmetric) <- that of U^-T A U^-1.
void reduce_to_standard(Ctx &c, double *A, const double *U, long long n);
// Householder tridiagonalisation of the symmetric A (column-major; both
// triangles valid, or only the upper one with upper_valid) in the output
// form of dsytrd('L'): d[n], e[n-1], tau[n-1], reflectors below the
// subdiagonal of A (tridiag.cu); the panel kernels use 1/share of the SMs.
// 0, or 4 if a grid barrier timed out.
int sytrd_lower(Ctx &c, double *A, long long n, double *d, double *e, double *tau, bool upper_valid,
                int share = 1);
// Y <- Q^T U^-T Y for Y column-major [n, m] (= row-major [m, n]): each row
// z of the row-major view becomes y with z^T (K + s S)^-1 z = y^T (T + s)^-1 y.
void pencil_rhs(Ctx &c, const PencilTridiag &P, double *Y, long long m);
// The inverse map of m vectors of the tridiagonal basis (columns of a
// column-major [n, m] X, in place): X <- U^-1 Q X.
void pencil_back(Ctx &c, const PencilTridiag &P, double *X, long long m);

// Accessor builders (C-ordered n-index tensors of one state or pair).
void build_ee2L(Ctx &c, const double *taa, const double *dal, int n, double *out);
void build_eee2L(Ctx &c, const double *daaa, const double *taa, const double *dal, int n, double *out);
void build_eee2tL(Ctx &c, const double *E3, const double *E2, int n, double *out);
void build_ee2trL(Ctx &c, const double *E2, const double *dal, int n, double *out);
void build_ee2tlL(Ctx &c, const double *E2, const double *dal, int n, double *out);
void build_ro2toff(Ctx &c, const double *taa, const double *dal, int n, double *out);

// Elementwise helpers.
void axpby(Ctx &c, long long count, double a, const double *x, double b, const double *y, double *out);
void fill(Ctx &c, double *p, long long count, double v);
void add_diag_pairs(Ctx &c, double *T4, int n, int pos1, int pos2, const double *M2, bool transposeM, double alpha);

}  // namespace s2
}  // namespace nvpt
