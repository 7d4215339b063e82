// Implementation of the device tensor toolkit (see s2_tensor.cuh).
#include "s2_tensor.cuh"

#include <algorithm>
#include <cmath>

#include "ozaki.cuh"

namespace nvpt {
namespace s2 {

namespace {
constexpr int TPB = 256;
inline unsigned nblk(long long n) { return (unsigned)((n + TPB - 1) / TPB); }

struct PermArgs {
    int nd;
    long long shape[6];
    long long stride[6];  // input stride of each output axis
    long long off;
};

__global__ void k_permute(const double *__restrict__ in, double *__restrict__ out, PermArgs a, long long total,
                          double alpha, int acc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    long long x = t, src = a.off;
    for (int k = a.nd - 1; k >= 0; --k) {
        long long i = x % a.shape[k];
        x /= a.shape[k];
        src += i * a.stride[k];
    }
    double v = alpha * in[src];
    out[t] = acc ? out[t] + v : v;
}

__global__ void k_fill(double *p, long long n, double v) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) p[t] = v;
}

__global__ void k_axpby(long long n, double a, const double *x, double b, const double *y, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) o[t] = a * x[t] + b * (y ? y[t] : 0.0);
}

__global__ void k_symm_upper(const double *A, long long n, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    long long r = t / n, c = t % n;
    o[t] = r <= c ? A[r * n + c] : A[c * n + r];
}

// qdnevpt-local accessors, C-ordered tensors (index arithmetic only).
__global__ void k_ee2L(const double *taa, const double *dal, int n, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n2 = (long long)n * n;
    if (t >= n2 * n2) return;
    int d = t % n, c = (t / n) % n, b = (t / n2) % n, a = (int)(t / (n2 * n));
    // ee2(a,b,c,d) = taa(b,d,a,c) + [b==c] dal(d,a)
    double v = taa[((long long)(b * n + d) * n + a) * n + c];
    if (b == c) v += dal[d * n + a];
    o[t] = v;
}

__global__ void k_eee2L(const double *daaa, const double *taa, const double *dal, int n, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n2 = (long long)n * n, n3 = n2 * n;
    if (t >= n3 * n3) return;
    long long x = t;
    int f = x % n; x /= n;
    int e = x % n; x /= n;
    int d = x % n; x /= n;
    int c = x % n; x /= n;
    int b = x % n; x /= n;
    int a = (int)x;
    auto D2 = [&](int i, int j, int k, int l) { return taa[((long long)(i * n + j) * n + k) * n + l]; };
    // eee2(a,b,c,d,e,f) = daaa(b,d,f,a,c,e) + [e==d] taa(b,f,a,c) + [e==b] taa(f,d,a,c)
    //                     + [b==c] taa(d,f,a,e) + [b==c][e==d] dal(f,a)
    double v = daaa[((((((long long)b * n + d) * n + f) * n + a) * n + c) * n) + e];
    if (e == d) v += D2(b, f, a, c);
    if (e == b) v += D2(f, d, a, c);
    if (b == c) v += D2(d, f, a, e);
    if (b == c && e == d) v += dal[f * n + a];
    o[t] = v;
}

__global__ void k_eee2tL(const double *E3, const double *E2, int n, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n2 = (long long)n * n, n3 = n2 * n;
    if (t >= n3 * n3) return;
    long long x = t;
    int f = x % n; x /= n;
    int e = x % n; x /= n;
    int d = x % n; x /= n;
    int c = x % n; x /= n;
    int b = x % n; x /= n;
    int a = (int)x;
    // eee2t(a,b,c,d,e,f) = -eee2(a,b,d,c,e,f) + [c==d] 2 ee2(a,b,e,f)
    double v = -E3[(((((long long)a * n + b) * n + d) * n + c) * n + e) * n + f];
    if (c == d) v += 2.0 * E2[((long long)(a * n + b) * n + e) * n + f];
    o[t] = v;
}

__global__ void k_ee2trL(const double *E2, const double *dal, int n, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n2 = (long long)n * n;
    if (t >= n2 * n2) return;
    int d = t % n, c = (t / n) % n, b = (t / n2) % n, a = (int)(t / (n2 * n));
    // ee2tr(a,b,c,d) = -ee2(a,b,d,c) + [c==d] 2 dal(b,a)
    double v = -E2[((long long)(a * n + b) * n + d) * n + c];
    if (c == d) v += 2.0 * dal[b * n + a];
    o[t] = v;
}

__global__ void k_ee2tlL(const double *E2, const double *dal, int n, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n2 = (long long)n * n;
    if (t >= n2 * n2) return;
    int d = t % n, c = (t / n) % n, b = (t / n2) % n, a = (int)(t / (n2 * n));
    // ee2tl(a,b,c,d) = -ee2(b,a,c,d) + [a==b] 2 dal(d,c)
    double v = -E2[((long long)(b * n + a) * n + c) * n + d];
    if (a == b) v += 2.0 * dal[d * n + c];
    o[t] = v;
}

__global__ void k_ro2toff(const double *d2, const double *d1, int n, double *o) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n2 = (long long)n * n;
    if (t >= n2 * n2) return;
    int b = t % n, a = (t / n) % n, bp = (t / n2) % n, ap = (int)(t / (n2 * n));
    double v = d2[t];
    if (ap == a) v -= 2.0 * d1[bp * n + b];
    if (bp == b) v -= 2.0 * d1[ap * n + a];
    if (ap == b) v += d1[bp * n + a];
    if (bp == a) v += d1[ap * n + b];
    o[t] = v;
}

__global__ void k_add_diag_pairs(double *T4, int n, int pos1, int pos2, const double *M2, int transM, double alpha) {
    // For a 4-index tensor T[i0,i1,i2,i3]: where i_pos1 == i_pos2, add
    // alpha * M[other indices in order] (transposed if transM).
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long n2 = (long long)n * n;
    if (t >= n2 * n2) return;
    int idx[4] = {(int)(t / (n2 * n)), (int)((t / n2) % n), (int)((t / n) % n), (int)(t % n)};
    if (idx[pos1] != idx[pos2]) return;
    int o[2], k = 0;
    for (int q = 0; q < 4; ++q)
        if (q != pos1 && q != pos2) o[k++] = idx[q];
    T4[t] += alpha * (transM ? M2[o[1] * n + o[0]] : M2[o[0] * n + o[1]]);
}
}  // namespace

T alloc_v(Ctx &c, const std::vector<long long> &shape, bool zero) {
    T t;
    t.st = c.st;
    t.nd = (int)shape.size();
    for (int i = 0; i < t.nd; ++i) t.sh[i] = shape[i];
    long long n = t.size();
    ck(cudaMallocAsync((void **)&t.p, sizeof(double) * (size_t)(n > 0 ? n : 1), c.st), "cudaMallocAsync");
    if (zero) ck(cudaMemsetAsync(t.p, 0, sizeof(double) * (size_t)(n > 0 ? n : 1), c.st), "memset");
    return t;
}

T alloc(Ctx &c, std::initializer_list<long long> shape, bool zero) {
    return alloc_v(c, std::vector<long long>(shape), zero);
}

void gather(Ctx &c, const double *in, long long off, const std::vector<long long> &shape,
            const std::vector<long long> &stride, double *out, double alpha, bool accumulate) {
    PermArgs a;
    a.nd = (int)shape.size();
    a.off = off;
    long long total = 1;
    for (int k = 0; k < a.nd; ++k) {
        a.shape[k] = shape[k];
        a.stride[k] = stride[k];
        total *= shape[k];
    }
    if (total == 0) return;
    k_permute<<<nblk(total), TPB, 0, c.st>>>(in, out, a, total, alpha, accumulate ? 1 : 0);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ck(cudaGetLastError(), "permute launch");
}

void permute(Ctx &c, const double *in, const std::vector<long long> &in_shape, const std::vector<int> &axes,
             double *out, double alpha, bool accumulate) {
    int nd = (int)in_shape.size();
    std::vector<long long> istr(nd);
    long long s = 1;
    for (int k = nd - 1; k >= 0; --k) {
        istr[k] = s;
        s *= in_shape[k];
    }
    std::vector<long long> shape(nd), stride(nd);
    for (int k = 0; k < nd; ++k) {
        shape[k] = in_shape[axes[k]];
        stride[k] = istr[axes[k]];
    }
    gather(c, in, 0, shape, stride, out, alpha, accumulate);
}

T permuted(Ctx &c, const T &in, const std::vector<int> &axes, double alpha) {
    std::vector<long long> ish(in.sh.begin(), in.sh.begin() + in.nd), osh(in.nd);
    for (int k = 0; k < in.nd; ++k) osh[k] = ish[axes[k]];
    T out = alloc_v(c, osh, false);
    permute(c, in.p, ish, axes, out.p, alpha, false);
    return out;
}

namespace {
// Products big enough to pay for the digit splits; alpha = +-2^e.  A product
// with few rows runs transposed (its columns fill the 128-row tiles).
bool split_product(const Ctx &c, long long m, long long n, long long k, double alpha) {
    if (!c.split || k < 64 || k > oz::kWideMaxK) return false;
    if (!((m >= 64 && n >= 16) || (m >= 16 && n >= 128))) return false;
    if ((double)m * (double)n * (double)k < 6.7e7) return false;
    int e = 0;
    return std::frexp(std::fabs(alpha), &e) == 0.5;
}
void split_gemm(Ctx &c, const oz::WideGemm &g) {
    void *w = nullptr;
    ck(cudaMallocAsync(&w, oz::oz_wide_bytes(g.m, g.n, g.K), c.st), "cudaMallocAsync");
    const int rc = oz::oz_gemm_wide(g, w, c.oz_err, c.st);
    cudaFreeAsync(w, c.st);
    if (rc) throw Error(2, "split-precision product failed to launch");
}
}  // namespace

void gemm(Ctx &c, bool ta, bool tb, long long m, long long n, long long k, double alpha, const double *A, long long lda,
          const double *B, long long ldb, double beta, double *C, long long ldc) {
    if (m == 0 || n == 0) return;
    if (split_product(c, m, n, k, alpha)) {
        oz::WideGemm g;
        g.K = (int)k;
        g.alpha = alpha; g.beta = beta; g.C = C; g.ldc = ldc;
        if (m >= 64) {
            g.m = m; g.n = n;
            g.A = A; g.a_r = ta ? 1 : lda; g.a_k = ta ? lda : 1;
            g.B = B; g.b_c = tb ? ldb : 1; g.b_k = tb ? 1 : ldb;
        } else {  // C^T = op(B)^T op(A)^T: rows of the product are the columns of C
            g.m = n; g.n = m;
            g.A = B; g.a_r = tb ? ldb : 1; g.a_k = tb ? 1 : ldb;
            g.B = A; g.b_c = ta ? 1 : lda; g.b_k = ta ? lda : 1;
            g.c_trans = true;
        }
        split_gemm(c, g);
        return;
    }
    // Row-major C = op(A) op(B)  <=>  column-major C^T = op(B)^T op(A)^T.
    ck(cublasDgemm(c.blas, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, (int)n, (int)m, (int)k,
                   &alpha, B, (int)ldb, A, (int)lda, &beta, C, (int)ldc),
       "cublasDgemm");
}

void gemm_batched(Ctx &c, bool ta, bool tb, long long m, long long n, long long k, double alpha, const double *A,
                  long long lda, long long sA, const double *B, long long ldb, long long sB, double beta, double *C,
                  long long ldc, long long sC, long long batch) {
    if (m == 0 || n == 0 || batch == 0) return;
    ck(cublasDgemmStridedBatched(c.blas, tb ? CUBLAS_OP_T : CUBLAS_OP_N, ta ? CUBLAS_OP_T : CUBLAS_OP_N, (int)n,
                                 (int)m, (int)k, &alpha, B, (int)ldb, sB, A, (int)lda, sA, &beta, C, (int)ldc, sC,
                                 (int)batch),
       "cublasDgemmStridedBatched");
}

void symmetrize_upper(Ctx &c, const double *A, long long n, double *out) {
    k_symm_upper<<<nblk(n * n), TPB, 0, c.st>>>(A, n, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

void eigh_upper(Ctx &c, const double *A, long long n, double *w, double *V) {
    if (n == 0) return;
    // Symmetric copy, so that the triangle cuSOLVER reads is the reference's upper one.
    symmetrize_upper(c, A, n, V);
    int lwork = 0;
    ck(cusolverDnDsyevd_bufferSize(c.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, (int)n, V, (int)n, w,
                                   &lwork),
       "syevd_bufferSize");
    double *work = nullptr;
    int *info = nullptr;
    ck(cudaMallocAsync((void **)&work, sizeof(double) * (size_t)lwork, c.st), "cudaMallocAsync");
    ck(cudaMallocAsync((void **)&info, sizeof(int), c.st), "cudaMallocAsync");
    ck(cusolverDnDsyevd(c.sol, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, (int)n, V, (int)n, w, work, lwork,
                        info),
       "syevd");
    int hinfo = 0;
    ck(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, c.st), "info copy");
    ck(cudaStreamSynchronize(c.st), "syevd sync");
    cudaFreeAsync(work, c.st);
    cudaFreeAsync(info, c.st);
    if (hinfo != 0) throw Error(2, "syevd failed, info=" + std::to_string(hinfo));
    // The symmetric input makes row-/column-major identical; cuSOLVER stores
    // eigenvector k as column k (column-major) = row k of the row-major array.
}

__global__ void k_add_diag(double *A, long long n, double v) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) A[i * n + i] += v;
}

__global__ void k_mirror_lower(double *o, long long m) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m * m) return;
    long long r = t / m, col = t % m;
    if (r < col) o[t] = o[col * m + r];
}

void gram(Ctx &c, const double *X, long long Q, long long m, double *out) {
    if (m == 0) return;
    if (split_product(c, m, m, Q, 1.0)) {
        // the tiles meeting the lower triangle of out = X^T X, then mirrored
        oz::WideGemm g;
        g.m = m; g.n = m; g.K = (int)Q;
        g.A = X; g.a_r = 1; g.a_k = m;
        g.B = X; g.b_c = 1; g.b_k = m;
        g.C = out; g.ldc = m; g.lower = true;
        split_gemm(c, g);
        k_mirror_lower<<<nblk(m * m), TPB, 0, c.st>>>(out, m);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return;
    }
    const double one = 1.0, zero = 0.0;
    // column-major view: X is m x Q (ld m); C = X X^T fills the column-major
    // upper triangle = the row-major lower triangle of out
    ck(cublasDsyrk(c.blas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, (int)m, (int)Q, &one, X, (int)m, &zero, out, (int)m),
       "cublasDsyrk");
    k_mirror_lower<<<nblk(m * m), TPB, 0, c.st>>>(out, m);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

int raise_dynamic_smem(const void *kernel) {
    cudaFuncAttributes fa{};
    ck(cudaFuncGetAttributes(&fa, kernel), "cudaFuncGetAttributes");
    int dev = 0, optin = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "attr");
    const int lim = optin - (int)fa.sharedSizeBytes;
    ck(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, lim), "smem attr");
    return lim;
}

bool metric_above(Ctx &c, const double *A, long long n, double thr) {
    if (n == 0) return true;
    double *M = nullptr, *work = nullptr;
    int *info = nullptr;
    ck(cudaMallocAsync((void **)&M, sizeof(double) * (size_t)(n * n), c.st), "cudaMallocAsync");
    symmetrize_upper(c, A, n, M);
    k_add_diag<<<nblk(n), TPB, 0, c.st>>>(M, n, -thr);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    int lwork = 0;
    ck(cusolverDnDpotrf_bufferSize(c.sol, CUBLAS_FILL_MODE_UPPER, (int)n, M, (int)n, &lwork), "potrf_bufferSize");
    ck(cudaMallocAsync((void **)&work, sizeof(double) * (size_t)(lwork > 0 ? lwork : 1), c.st), "cudaMallocAsync");
    ck(cudaMallocAsync((void **)&info, sizeof(int), c.st), "cudaMallocAsync");
    ck(cusolverDnDpotrf(c.sol, CUBLAS_FILL_MODE_UPPER, (int)n, M, (int)n, work, lwork, info), "potrf");
    int hinfo = -1;
    ck(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, c.st), "info copy");
    ck(cudaStreamSynchronize(c.st), "potrf sync");
    cudaFreeAsync(work, c.st);
    cudaFreeAsync(info, c.st);
    cudaFreeAsync(M, c.st);
    return hinfo == 0;
}

bool sygvd_upper(Ctx &c, const double *K, const double *S, long long n, double *w, double *V) {
    if (n == 0) return true;
    double *B = nullptr, *work = nullptr;
    int *info = nullptr;
    symmetrize_upper(c, K, n, V);
    ck(cudaMallocAsync((void **)&B, sizeof(double) * (size_t)(n * n), c.st), "cudaMallocAsync");
    symmetrize_upper(c, S, n, B);
    int lwork = 0;
    ck(cusolverDnDsygvd_bufferSize(c.sol, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER,
                                   (int)n, V, (int)n, B, (int)n, w, &lwork),
       "sygvd_bufferSize");
    ck(cudaMallocAsync((void **)&work, sizeof(double) * (size_t)(lwork > 0 ? lwork : 1), c.st), "cudaMallocAsync");
    ck(cudaMallocAsync((void **)&info, sizeof(int), c.st), "cudaMallocAsync");
    ck(cusolverDnDsygvd(c.sol, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, (int)n, V,
                        (int)n, B, (int)n, w, work, lwork, info),
       "sygvd");
    int hinfo = -1;
    ck(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, c.st), "info copy");
    ck(cudaStreamSynchronize(c.st), "sygvd sync");
    cudaFreeAsync(work, c.st);
    cudaFreeAsync(info, c.st);
    cudaFreeAsync(B, c.st);
    return hinfo == 0;
}

namespace {
// cuSOLVER workspace of `count` doubles + info word, stream-ordered.
struct SolverWork {
    Ctx &c;
    double *w = nullptr;
    int *info = nullptr;
    SolverWork(Ctx &cc, int count) : c(cc) {
        ck(cudaMallocAsync((void **)&w, sizeof(double) * (size_t)(count > 0 ? count : 1), c.st), "cudaMallocAsync");
        ck(cudaMallocAsync((void **)&info, sizeof(int), c.st), "cudaMallocAsync");
    }
    int status() {
        int h = -1;
        ck(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, c.st), "info copy");
        ck(cudaStreamSynchronize(c.st), "solver sync");
        return h;
    }
    ~SolverWork() {
        cudaFreeAsync(w, c.st);
        cudaFreeAsync(info, c.st);
    }
};
}  // namespace

namespace {
// Mirror the upper triangle of the kb x kb diagonal block at A (column-major,
// ld) into its lower triangle.
__global__ void k_mirror_block(double *A, long long ld, int kb) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)kb * kb) return;
    const int i = (int)(t % kb), j = (int)(t / kb);
    if (i > j) A[i + j * ld] = A[j + i * ld];
}
}  // namespace

// Upper triangle of A (column-major n x n, symmetric on entry) <- the upper
// triangle of U^-T A U^-1, U upper triangular: the blocked right-looking
// reduction of a symmetric-definite pencil to standard form (n^3 flops, half
// of two full triangular solves).  Per diagonal block k of width kb, with the
// trailing blocks 12 (kb x m) and 22:
//   A11 <- U11^-T A11 U11^-1
//   A12 <- U11^-T A12 - 1/2 A11 U12
//   A22 <- A22 - A12^T U12 - U12^T A12          (upper triangle)
//   A12 <- (A12 - 1/2 A11 U12) U22^-1
// after which A22 is reduced in turn.  The lower triangle is left stale.
void reduce_to_standard(Ctx &c, double *A, const double *U, long long n) {
    constexpr int NB = 256;
    const double one = 1.0, mhalf = -0.5, mone = -1.0;
    for (long long k = 0; k < n; k += NB) {
        const int kb = (int)std::min<long long>(NB, n - k), m = (int)(n - k - kb);
        double *A11 = A + k + k * n;
        const double *U11 = U + k + k * n;
        k_mirror_block<<<nblk((long long)kb * kb), TPB, 0, c.st>>>(A11, n, kb);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        ck(cublasDtrsm(c.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, kb, kb,
                       &one, U11, (int)n, A11, (int)n),
           "trsm");
        ck(cublasDtrsm(c.blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, kb, kb,
                       &one, U11, (int)n, A11, (int)n),
           "trsm");
        if (m == 0) break;
        double *A12 = A + k + (k + kb) * n, *A22 = A + (k + kb) + (k + kb) * n;
        const double *U12 = U + k + (k + kb) * n, *U22 = U + (k + kb) + (k + kb) * n;
        ck(cublasDtrsm(c.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, kb, m,
                       &one, U11, (int)n, A12, (int)n),
           "trsm");
        ck(cublasDsymm(c.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, kb, m, &mhalf, A11, (int)n, U12, (int)n, &one,
                       A12, (int)n),
           "symm");
        ck(cublasDsyr2k(c.blas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, m, kb, &mone, A12, (int)n, U12, (int)n, &one, A22,
                        (int)n),
           "syr2k");
        ck(cublasDsymm(c.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, kb, m, &mhalf, A11, (int)n, U12, (int)n, &one,
                       A12, (int)n),
           "symm");
        ck(cublasDtrsm(c.blas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, kb, m,
                       &one, U22, (int)n, A12, (int)n),
           "trsm");
    }
}

bool pencil_tridiag(Ctx &c, const double *K, const double *S, long long n, PencilTridiag &P) {
    P.n = n;
    if (n == 0) return true;
    const int N = (int)n;
    P.U = alloc(c, {n, n}, false);
    P.A = alloc(c, {n, n}, false);
    P.d = alloc(c, {n}, false);
    P.e = alloc(c, {n}, true);
    P.tau = alloc(c, {n}, true);
    symmetrize_upper(c, S, n, P.U.p);
    symmetrize_upper(c, K, n, P.A.p);
    int lw_p = 0;
    ck(cusolverDnDpotrf_bufferSize(c.sol, CUBLAS_FILL_MODE_UPPER, N, P.U.p, N, &lw_p), "potrf_bufferSize");
    SolverWork sw(c, lw_p);
    ProfSpan sp;
    sp.begin("pencil_potrf", c.st, 0);
    ck(cusolverDnDpotrf(c.sol, CUBLAS_FILL_MODE_UPPER, N, P.U.p, N, sw.w, lw_p, sw.info), "potrf");
    sp.end();
    if (sw.status() != 0) return false;
    sp.begin("pencil_reduce", c.st, 0);
    reduce_to_standard(c, P.A.p, P.U.p, n);
    sp.end();
    sp.begin("pencil_sytrd", c.st, 0);
    const int trc = sytrd_lower(c, P.A.p, n, P.d.p, P.e.p, P.tau.p, true, std::min(4, std::max(1, c.sm_share)));
    sp.end();
    if (trc != 0) throw Error(4, "tridiagonalisation: a grid barrier timed out");
    return true;
}

void pencil_rhs(Ctx &c, const PencilTridiag &P, double *Y, long long m) {
    if (P.n == 0 || m == 0) return;
    const int N = (int)P.n, Mc = (int)m;
    const double one = 1.0;
    ProfSpan sp;
    sp.begin("pencil_rhs", c.st, 0);
    ck(cublasDtrsm(c.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, N, Mc, &one,
                   P.U.p, N, Y, N),
       "trsm");
    int lw = 0;
    ck(cusolverDnDormtr_bufferSize(c.sol, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, N, Mc, P.A.p, N,
                                   P.tau.p, Y, N, &lw),
       "ormtr_bufferSize");
    SolverWork sw(c, lw);
    ck(cusolverDnDormtr(c.sol, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_T, N, Mc, P.A.p, N, P.tau.p, Y, N,
                        sw.w, lw, sw.info),
       "ormtr");
    sp.end();
    const int st = sw.status();
    if (st != 0) throw Error(2, "ormtr failed, info=" + std::to_string(st));
}

void pencil_back(Ctx &c, const PencilTridiag &P, double *X, long long m) {
    if (P.n == 0 || m == 0) return;
    const int N = (int)P.n, Mc = (int)m;
    const double one = 1.0;
    ProfSpan sp;
    sp.begin("pencil_rhs", c.st, 0);
    int lw = 0;
    ck(cusolverDnDormtr_bufferSize(c.sol, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, N, Mc, P.A.p, N,
                                   P.tau.p, X, N, &lw),
       "ormtr_bufferSize");
    SolverWork sw(c, lw);
    ck(cusolverDnDormtr(c.sol, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, N, Mc, P.A.p, N, P.tau.p, X, N,
                        sw.w, lw, sw.info),
       "ormtr");
    ck(cublasDtrsm(c.blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, N, Mc, &one,
                   P.U.p, N, X, N),
       "trsm");
    sp.end();
    const int st = sw.status();
    if (st != 0) throw Error(2, "ormtr failed, info=" + std::to_string(st));
}

void build_ee2L(Ctx &c, const double *taa, const double *dal, int n, double *out) {
    long long N = (long long)n * n * n * n;
    k_ee2L<<<nblk(N), TPB, 0, c.st>>>(taa, dal, n, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void build_eee2L(Ctx &c, const double *daaa, const double *taa, const double *dal, int n, double *out) {
    long long N = (long long)n * n * n * n * n * n;
    k_eee2L<<<nblk(N), TPB, 0, c.st>>>(daaa, taa, dal, n, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void build_eee2tL(Ctx &c, const double *E3, const double *E2, int n, double *out) {
    long long N = (long long)n * n * n * n * n * n;
    k_eee2tL<<<nblk(N), TPB, 0, c.st>>>(E3, E2, n, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void build_ee2trL(Ctx &c, const double *E2, const double *dal, int n, double *out) {
    long long N = (long long)n * n * n * n;
    k_ee2trL<<<nblk(N), TPB, 0, c.st>>>(E2, dal, n, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void build_ee2tlL(Ctx &c, const double *E2, const double *dal, int n, double *out) {
    long long N = (long long)n * n * n * n;
    k_ee2tlL<<<nblk(N), TPB, 0, c.st>>>(E2, dal, n, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void build_ro2toff(Ctx &c, const double *taa, const double *dal, int n, double *out) {
    long long N = (long long)n * n * n * n;
    k_ro2toff<<<nblk(N), TPB, 0, c.st>>>(taa, dal, n, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void axpby(Ctx &c, long long count, double a, const double *x, double b, const double *y, double *out) {
    k_axpby<<<nblk(count), TPB, 0, c.st>>>(count, a, x, b, y, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void fill(Ctx &c, double *p, long long count, double v) {
    k_fill<<<nblk(count), TPB, 0, c.st>>>(p, count, v);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void add_diag_pairs(Ctx &c, double *T4, int n, int pos1, int pos2, const double *M2, bool transposeM, double alpha) {
    long long N = (long long)n * n * n * n;
    k_add_diag_pairs<<<nblk(N), TPB, 0, c.st>>>(T4, n, pos1, pos2, M2, transposeM ? 1 : 0, alpha);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

}  // namespace s2
}  // namespace nvpt
