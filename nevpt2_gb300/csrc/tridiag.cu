// Householder tridiagonalisation of a symmetric FP64 matrix (the PC pencils
// of the order-n^3 classes), in the output form of LAPACK dsytrd('L'):
// d, e, tau and the reflectors below the subdiagonal of A, so that cuSOLVER's
// ormtr applies Q.
//
// The algorithm is the blocked one-stage reduction: panels of NBP columns;
// inside a panel, column j is updated with the panel's earlier reflectors,
// its reflector (v, tau) is generated, and w = tau (A22 v - V W^T v - W V^T v)
// - (tau/2)(w^T v) v is formed from the trailing matrix as of the panel's
// start; after the panel the trailing matrix takes the rank-2 NBP update
// A22 -= V W^T + W V^T (cuBLAS syr2k) and is mirrored to full storage.
//
// GB300 form: a panel is one cooperative kernel, one CTA per SM.  A column
// costs three grid barriers; its symmetric matrix-vector product reads
// columns of the trailing matrix (full storage, so every read is a
// contiguous column), one warp per column, at L2/HBM bandwidth.  cuSOLVER's
// sytrd spends most of its time in per-column synchronisation; here a
// column's latency is three barriers plus one pass over the trailing matrix.
// Every barrier wait is bounded: a timeout sets an error flag and every CTA
// returns.
#include <cooperative_groups.h>

#include <algorithm>

#include "../../include/nvpt2.h"
#include "s2_tensor.cuh"

namespace nvpt {
namespace s2 {

namespace {

constexpr int NBP = 32;        // panel width
constexpr int TT = 256;        // threads per CTA
constexpr int PARTS = 2 + 2 * NBP;  // per-CTA partial sums: |x|^2, w.v, (W^T v, V^T v)[NBP]
constexpr unsigned kBarSpin = 1u << 22;  // polls (with back-off) before a barrier gives up

struct Bar {
    unsigned count, gen;
    int err;
};

// Grid-wide barrier (all CTAs co-resident: cooperative launch).  Returns
// false if the wait timed out or another CTA reported an error.
__device__ bool grid_bar(Bar *b, unsigned nblk, unsigned &gen) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned g = gen;
        __threadfence();
        if (atomicAdd(&b->count, 1u) == nblk - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicExch(&b->gen, g + 1);
        } else {
            unsigned spins = 0;
            while (*(volatile unsigned *)&b->gen == g) {
                if (++spins > kBarSpin || *(volatile int *)&b->err) {
                    atomicExch(&b->err, 1);
                    ok = 0;
                    break;
                }
                if (spins > 32) __nanosleep(20);
            }
        }
        __threadfence();
        gen = g + 1;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < TT / 32; ++i) s += red[i];
    return s;  // valid in thread 0
}

struct PanelArgs {
    double *A;       // column-major n x n, both triangles valid for the trailing matrix
    long long n;
    int j0, nbp;     // panel columns j0 .. j0 + nbp - 1
    double *V, *W;   // column-major n x NBP (ld n)
    double *d, *e, *tau;
    double *y;       // n
    double *part;    // gridDim.x x PARTS
    Bar *bar;
};

// Sum of part[b * PARTS + off] over the CTAs, by warp `w` (result in lane 0).
__device__ __forceinline__ double grid_part_sum(const double *part, unsigned G, int off) {
    double s = 0.0;
    for (unsigned b = threadIdx.x & 31; b < G; b += 32) s += part[(size_t)b * PARTS + off];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    return s;
}

__global__ void __launch_bounds__(TT, 1) k_sytrd_panel(PanelArgs p) {
    __shared__ double vj[NBP], wj[NBP], cwv[2 * NBP], red[TT / 32];
    __shared__ double s_tau, s_alpha2, s_scal, s_beta, s_wpiv;
    __shared__ int s_refl;
    const long long n = p.n;
    const unsigned G = gridDim.x;
    const long long chunk = (n + G - 1) / G, r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, sub = threadIdx.x & 7, grp = threadIdx.x >> 3;
    unsigned gen = *(volatile unsigned *)&p.bar->gen;  // barriers continue across the panel launches
    double *part = p.part + (size_t)blockIdx.x * PARTS;
    for (int jj = 0; jj < p.nbp; ++jj) {
        const long long j = p.j0 + jj;
        double *Aj = p.A + j * n;
        // ---- P1: column j -= V W(j,:)^T + W V(j,:)^T over the panel's earlier columns;
        // eight threads per row split the sum over those columns
        if (threadIdx.x < jj) {
            const int t = threadIdx.x;
            vj[t] = p.V[j + t * n];
            wj[t] = (t == jj - 1) ? s_wpiv : p.W[j + t * n];  // the pivot row's newest w is formed locally
        }
        __syncthreads();
        double ss = 0.0;
        for (long long i0 = max(r0, j); i0 < r1; i0 += TT / 8) {  // uniform trip count: full-warp shuffles
            const long long i = i0 + grp;
            const bool live = i < r1;
            double c = 0.0;
            if (live)
                for (int t = sub; t < jj; t += 8) c += p.V[i + t * n] * wj[t] + p.W[i + t * n] * vj[t];
            c += __shfl_xor_sync(0xffffffffu, c, 1);
            c += __shfl_xor_sync(0xffffffffu, c, 2);
            c += __shfl_xor_sync(0xffffffffu, c, 4);
            if (live && sub == 0) {
                const double a = Aj[i] - c;
                Aj[i] = a;
                if (i == j) p.d[j] = a;
                if (i >= j + 2) ss += a * a;
            }
        }
        ss = block_sum(ss, red);
        if (threadIdx.x == 0) part[0] = ss;
        if (j + 1 >= n) break;  // last column: only its diagonal
        if (!grid_bar(p.bar, G, gen)) return;
        // ---- P2: the reflector of column j (every CTA forms the same scalars)
        if (warp == 0) {
            const double x2 = grid_part_sum(p.part, G, 0);
            if (lane == 0) {
                const double alpha = Aj[j + 1];
                if (x2 == 0.0) {
                    s_tau = 0.0;
                    s_beta = alpha;
                    s_scal = 0.0;
                } else {
                    const double beta = -copysign(sqrt(alpha * alpha + x2), alpha);
                    s_tau = (beta - alpha) / beta;
                    s_beta = beta;
                    s_scal = 1.0 / (alpha - beta);
                }
                s_refl = x2 != 0.0;
                if (blockIdx.x == 0) {
                    p.e[j] = s_beta;
                    p.tau[j] = s_tau;
                }
            }
        }
        __syncthreads();
        double *Vc = p.V + jj * n, *Wc = p.W + jj * n;
        // A(j+1, j) keeps alpha until every CTA has read it (it becomes beta in P4)
        for (long long i = max(r0, j + 1) + threadIdx.x; i < r1; i += TT) {
            double v = 1.0;
            if (i > j + 1) {
                v = s_refl ? Aj[i] * s_scal : Aj[i];
                Aj[i] = v;
            }
            Vc[i] = v;
        }
        __syncthreads();
        // partial W^T v and V^T v over the panel's earlier columns: eight threads per column t
        {
            const int t = grp;
            double a = 0.0, b = 0.0;
            if (t < jj)
                for (long long i = max(r0, j + 1) + sub; i < r1; i += 8) {
                    const double v = Vc[i];
                    a += p.W[i + t * n] * v;
                    b += p.V[i + t * n] * v;
                }
            for (int o = 1; o < 8; o <<= 1) {
                a += __shfl_xor_sync(0xffffffffu, a, o);
                b += __shfl_xor_sync(0xffffffffu, b, o);
            }
            if (sub == 0 && t < jj) {
                part[2 + 2 * t] = a;
                part[3 + 2 * t] = b;
            }
        }
        if (!grid_bar(p.bar, G, gen)) return;
        // ---- P3: y = tau (A22 v - V (W^T v) - W (V^T v)), one warp per column of A22
        for (int idx = warp; idx < 2 * jj; idx += TT / 32) {
            const double sm = grid_part_sum(p.part, G, 2 + idx);
            if (lane == 0) cwv[idx] = sm;  // cwv[2t] = (W^T v)_t, cwv[2t+1] = (V^T v)_t
        }
        __syncthreads();
        double q = 0.0;
        const long long m0 = j + 1;
        for (long long i = m0 + (long long)blockIdx.x * (TT / 32) + warp; i < n; i += (long long)G * (TT / 32)) {
            const double *Ai = p.A + i * n;
            double s = 0.0;
            for (long long k = m0 + lane; k < n; k += 32) s += Ai[k] * Vc[k];
            for (int t = lane; t < jj; t += 32) s -= p.V[i + t * n] * cwv[2 * t] + p.W[i + t * n] * cwv[2 * t + 1];
            for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) {
                const double yi = s_tau * s;
                p.y[i] = yi;
                q += yi * Vc[i];
            }
        }
        q = block_sum(q, red);
        if (threadIdx.x == 0) part[1] = q;
        if (!grid_bar(p.bar, G, gen)) return;
        // ---- P4: w = y - (tau/2)(y^T v) v on this CTA's rows; the next pivot row's w locally
        if (warp == 0) {
            const double qs = grid_part_sum(p.part, G, 1);
            if (lane == 0) {
                s_alpha2 = -0.5 * s_tau * qs;
                s_wpiv = p.y[j + 1] + s_alpha2;  // v(j+1) = 1
            }
        }
        __syncthreads();
        for (long long i = max(r0, j + 1) + threadIdx.x; i < r1; i += TT) {
            Wc[i] = p.y[i] + s_alpha2 * Vc[i];
            if (i == j + 1) Aj[i] = s_beta;  // the subdiagonal of T, as dsytrd leaves it
        }
        __syncthreads();
    }
}

// Mirror the lower triangle of the trailing block A[k:, k:] (column-major, ld n) to its upper triangle.
__global__ void k_mirror_trailing(double *A, long long n, long long k) {
    const long long m = n - k;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m * m) return;
    const long long i = k + t % m, jc = k + t / m;  // row i, column jc
    if (i < jc) A[i + jc * n] = A[jc + i * n];
}

// Upper triangle -> lower (column-major): the full symmetric matrix.
__global__ void k_mirror_to_lower(double *A, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const long long i = t % n, jc = t / n;
    if (i > jc) A[i + jc * n] = A[jc + i * n];
}

}  // namespace

int sytrd_lower(Ctx &c, double *A, long long n, double *d, double *e, double *tau, bool upper_valid) {
    if (n <= 0) return 0;
    constexpr int TPB = 256;
    auto nb = [](long long x) { return (unsigned)((x + TPB - 1) / TPB); };
    if (upper_valid) {
        k_mirror_to_lower<<<nb(n * n), TPB, 0, c.st>>>(A, n);
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    int dev = 0, sms = 0, per = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attr");
    ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sytrd_panel, TT, 0), "occupancy");
    if (per < 1) throw Error(2, "sytrd panel kernel cannot be resident");
    const unsigned G = (unsigned)sms;
    T V = alloc(c, {NBP, n}, false), W = alloc(c, {NBP, n}, false), y = alloc(c, {n}, false);
    T part = alloc(c, {(long long)G, PARTS}, false);
    T barw = alloc(c, {2}, true);  // Bar (12 bytes) in 16 zeroed bytes
    Bar *bar = (Bar *)barw.p;
    const double mone = -1.0, one = 1.0;
    for (long long j0 = 0; j0 < n; j0 += NBP) {
        const int nbp = (int)std::min<long long>(NBP, n - j0);
        PanelArgs a{A, n, (int)j0, nbp, V.p, W.p, d, e, tau, y.p, part.p, bar};
        void *args[] = {&a};
        ck(cudaLaunchCooperativeKernel((const void *)k_sytrd_panel, dim3(G), dim3(TT), args, 0, c.st),
           "cooperative launch");
        g_launches.fetch_add(1, std::memory_order_relaxed);
        const long long k = j0 + nbp, m = n - k;
        if (m <= 0) break;
        // A22 -= V W^T + W V^T (lower), then full storage again
        ck(cublasDsyr2k(c.blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, (int)m, nbp, &mone, V.p + k, (int)n, W.p + k,
                        (int)n, &one, A + k + k * n, (int)n),
           "syr2k");
        k_mirror_trailing<<<nb(m * m), TPB, 0, c.st>>>(A, n, k);
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    int h[3] = {0, 0, 0};
    ck(cudaMemcpyAsync(h, barw.p, sizeof(int) * 3, cudaMemcpyDeviceToHost, c.st), "barrier state");
    ck(cudaStreamSynchronize(c.st), "sytrd sync");
    return h[2] ? 4 : 0;
}

}  // namespace s2
}  // namespace nvpt

// ===================================================================== C ABI
extern "C" const char *nvpt_context_error_set(nvpt_context *ctx, const char *msg);
extern "C" void *nvpt_context_stream(nvpt_context *ctx);

extern "C" int nvpt_sytrd_d(nvpt_context *ctx, int64_t n, double *A, double *d, double *e, double *tau,
                            void *stream) {
    using namespace nvpt::s2;
    if (!ctx || n < 1 || !A || !d || (n > 1 && (!e || !tau))) return NVPT_EINVAL;
    cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)nvpt_context_stream(ctx);
    try {
        static thread_local struct H {
            cublasHandle_t h = nullptr;
            ~H() {
                if (h) cublasDestroy(h);
            }
        } blas;
        if (!blas.h) ck(cublasCreate(&blas.h), "cublasCreate");
        ck(cublasSetStream(blas.h, st), "cublasSetStream");
        Ctx c{st, blas.h, nullptr};
        const int rc = sytrd_lower(c, A, n, d, e, tau, false);
        if (rc) {
            nvpt_context_error_set(ctx, "sytrd: a grid barrier timed out");
            return NVPT_ETIMEDOUT;
        }
        return NVPT_OK;
    } catch (const Error &err) {
        nvpt_context_error_set(ctx, err.what());
        return err.code == 3 ? NVPT_ENOMEM : NVPT_ECUDA;
    }
}
