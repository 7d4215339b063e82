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
// costs two grid barriers: one after the column's update (partial norms and
// the dot products with the panel's earlier reflectors, all taken against the
// unscaled column), one after the symmetric matrix-vector product; the
// reflector's scalars are formed redundantly by every CTA, v sits in shared
// memory, and w is finished with the next column's update.  The product
// reads columns of the trailing matrix (full storage, so every read is a
// contiguous column), one warp per column.  GB300's FP64 rate (~2 FMA per
// clock per SM) makes the product itself ~2n^3/3 FMAs of pure FP64 work, so
// the per-column latency around it is what is left to remove.
// Every barrier wait is bounded: a timeout sets an error flag and every CTA
// returns.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>

#include "../../include/nvpt2.h"
#include "s2_tensor.cuh"

namespace nvpt {
namespace s2 {

namespace {

constexpr int NBP = 32;        // panel width
constexpr int TT = 256;        // threads per CTA
constexpr int PARTS = 2 + 2 * NBP;  // column sums: |x|^2, w.v, (W^T a, V^T a)[NBP]
// NVPT_SYTRD_SHARE (1..16) overrides the caller's SM split, for tuning on other parts.
int sm_share(int share) {
    static const int v = [] {
        const char *e = std::getenv("NVPT_SYTRD_SHARE");
        const int x = e ? std::atoi(e) : 0;
        return (x >= 1 && x <= 16) ? x : 0;
    }();
    return v ? v : share;
}
constexpr unsigned kBarSpin = 1u << 22;  // polls (with back-off) before a barrier gives up

struct Bar {
    unsigned count, gen;
    int err;
};

// Grid-wide barrier (all CTAs co-resident: cooperative launch).  Arrival is
// an acq_rel add on the counter; the last CTA resets it and publishes the
// next generation with a release store; the others poll the generation with
// acquire loads.  Returns false if the wait timed out or another CTA
// reported an error.
__device__ bool grid_bar(Bar *b, unsigned nblk, unsigned &gen, unsigned limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned g = gen;
        unsigned old;
        asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(&b->count) : "memory");
        if (old == nblk - 1) {
            asm volatile("st.relaxed.gpu.global.u32 [%0], 0;" ::"l"(&b->count) : "memory");
            asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(&b->gen), "r"(g + 1) : "memory");
        } else {
            unsigned spins = 0, cur;
            for (;;) {
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(&b->gen) : "memory");
                if (cur != g) break;
                if (++spins > limit || *(volatile int *)&b->err) {
                    atomicExch(&b->err, 1);
                    ok = 0;
                    break;
                }
                if (spins > 64) __nanosleep(32);
            }
        }
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
    double *acc;     // 2 x PARTS: the column sums (atomics), by column parity
    Bar *bar;
    unsigned spin;   // polls before a barrier wait gives up
};

__global__ void __launch_bounds__(TT, 1) k_sytrd_panel(PanelArgs p) {
    extern __shared__ double vsh[];  // v of the current column, rows 0..n-1 (rows <= j unused)
    __shared__ double vj[NBP], wj[NBP], cwv[2 * NBP], red[TT / 32];
    __shared__ double s_tau, s_scal, s_beta, s_alpha2, s_wpiv, s_tau_p, s_beta_p, s_x2;
    const long long n = p.n;
    const unsigned G = gridDim.x;
    const long long chunk = (n + G - 1) / G, r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, sub = threadIdx.x & 7, grp = threadIdx.x >> 3;
    unsigned gen = *(volatile unsigned *)&p.bar->gen;  // barriers continue across the panel launches
    // P4 of column jp (pending until the partial sums of its w^T v are in):
    // W(:,jp) = y + alpha2 v on this CTA's rows, V(:,jp) = v, the reflector
    // into A(:,jp) and beta into A(jp+1,jp).
    auto finish = [&](int jjp) {
        const long long jp = p.j0 + jjp;
        if (threadIdx.x == 0) {
            const double qs = __ldcg(p.acc + (size_t)(jjp & 1) * PARTS + 1);
            {
                s_alpha2 = -0.5 * s_tau_p * qs;
                s_wpiv = __ldcg(p.y + jp + 1) + s_alpha2;  // w of the next pivot row (v = 1 there)
            }
        }
        __syncthreads();
        double *Vp = p.V + jjp * n, *Wp = p.W + jjp * n, *Ap = p.A + jp * n;
        for (long long i = max(r0, jp + 1) + threadIdx.x; i < r1; i += TT) {
            const double v = vsh[i];
            Wp[i] = __ldcg(p.y + i) + s_alpha2 * v;
            Vp[i] = v;
            Ap[i] = (i == jp + 1) ? s_beta_p : v;
        }
        __syncthreads();
    };
    int pending = -1;
    for (int jj = 0; jj < p.nbp; ++jj) {
        const long long j = p.j0 + jj;
        double *Aj = p.A + j * n;
        // the sums of column j accumulate in acc (by the parity of jj); column j+1 uses accn
        double *acc = p.acc + (size_t)(jj & 1) * PARTS, *accn = p.acc + (size_t)((jj + 1) & 1) * PARTS;
        if (pending >= 0) finish(pending);
        pending = -1;
        // ---- P1: column j -= V W(j,:)^T + W V(j,:)^T over the panel's earlier columns
        if (threadIdx.x < jj) {
            const int t = threadIdx.x;
            vj[t] = (t == jj - 1) ? 1.0 : __ldcg(p.V + j + t * n);     // v of column j-1 is 1 at its pivot row j
            wj[t] = (t == jj - 1) ? s_wpiv : __ldcg(p.W + j + t * n);  // formed locally in finish()
        }
        __syncthreads();
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
            }
        }
        if (j + 1 >= n) break;  // last column: only its diagonal
        __syncthreads();
        // partials over rows i >= j+2: |a|^2, W(:,t)^T a, V(:,t)^T a (eight threads per t)
        {
            double x2 = 0.0;
            for (long long i = max(r0, j + 2) + threadIdx.x; i < r1; i += TT) x2 += Aj[i] * Aj[i];
            x2 = block_sum(x2, red);
            if (threadIdx.x == 0) atomicAdd(acc + 0, x2);
            const int t = grp;
            double a = 0.0, b = 0.0;
            if (t < jj)
                for (long long i = max(r0, j + 2) + sub; i < r1; i += 8) {
                    const double ai = Aj[i];
                    a += p.W[i + t * n] * ai;
                    b += p.V[i + t * n] * ai;
                }
            for (int o = 1; o < 8; o <<= 1) {
                a += __shfl_xor_sync(0xffffffffu, a, o);
                b += __shfl_xor_sync(0xffffffffu, b, o);
            }
            if (sub == 0 && t < jj) {
                atomicAdd(acc + 2 + 2 * t, a);
                atomicAdd(acc + 3 + 2 * t, b);
            }
        }
        if (!grid_bar(p.bar, G, gen, p.spin)) return;
        // the other parity's sums were last read before this barrier: clear them for column j+1
        if (blockIdx.x == 0 && threadIdx.x < PARTS) accn[threadIdx.x] = 0.0;
        // ---- P2: the reflector of column j (every CTA forms the same scalars), v into shared memory
        if (threadIdx.x < 1 + 2 * jj) {
            const int v = threadIdx.x;
            const double sm = __ldcg(acc + (v == 0 ? 0 : v + 1));
            if (v == 0) s_x2 = sm;
            else cwv[v - 1] = sm;  // raw sums, scaled below
        }
        __syncthreads();
        if (warp == 0) {
            const double x2 = s_x2;
            if (lane == 0) {
                const double alpha = __ldcg(Aj + j + 1);
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
                if (blockIdx.x == 0) {
                    p.e[j] = s_beta;
                    p.tau[j] = s_tau;
                }
            }
        }
        __syncthreads();
        for (long long k = j + 1 + threadIdx.x; k < n; k += TT) vsh[k] = (k == j + 1) ? 1.0 : __ldcg(Aj + k) * s_scal;
        // W^T v and V^T v: v = scal a below the pivot row, 1 at it
        if (threadIdx.x < 2 * jj) {
            const int idx = threadIdx.x, t = idx >> 1;
            const double piv = (idx & 1) ? __ldcg(p.V + j + 1 + t * n) : __ldcg(p.W + j + 1 + t * n);
            cwv[idx] = s_scal * cwv[idx] + piv;  // cwv[2t] = (W^T v)_t, cwv[2t+1] = (V^T v)_t
        }
        __syncthreads();
        // ---- P3: y = tau (A22 v - V (W^T v) - W (V^T v)), one warp per column of A22
        double q = 0.0;
        const long long m0 = j + 1;
        for (long long i = m0 + (long long)blockIdx.x * (TT / 32) + warp; i < n; i += (long long)G * (TT / 32)) {
            const double *Ai = p.A + i * n;
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
            long long k = m0 + lane;
            for (; k + 96 < n; k += 128) {
                s0 += __ldcg(Ai + k) * vsh[k];
                s1 += __ldcg(Ai + k + 32) * vsh[k + 32];
                s2 += __ldcg(Ai + k + 64) * vsh[k + 64];
                s3 += __ldcg(Ai + k + 96) * vsh[k + 96];
            }
            for (; k < n; k += 32) s0 += __ldcg(Ai + k) * vsh[k];
            double s = (s0 + s1) + (s2 + s3);
            for (int t = lane; t < jj; t += 32)
                s -= __ldcg(p.V + i + t * n) * cwv[2 * t] + __ldcg(p.W + i + t * n) * cwv[2 * t + 1];
            for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) {
                const double yi = s_tau * s;
                p.y[i] = yi;
                q += yi * vsh[i];
            }
        }
        q = block_sum(q, red);
        if (threadIdx.x == 0) {
            atomicAdd(acc + 1, q);
            s_tau_p = s_tau;
            s_beta_p = s_beta;
        }
        if (!grid_bar(p.bar, G, gen, p.spin)) return;
        pending = jj;
    }
    if (pending >= 0) finish(pending);
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

int sytrd_lower(Ctx &c, double *A, long long n, double *d, double *e, double *tau, bool upper_valid, int share) {
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
    const size_t vbytes = sizeof(double) * (size_t)n;  // v of the current column in shared memory
    // one limit for every caller: tridiagonalisations of different orders run
    // concurrently on other host threads
    const int lim = raise_dynamic_smem((const void *)k_sytrd_panel);
    if (vbytes > 200 * 1024 || (long long)vbytes > lim)
        throw Error(1, "sytrd: order too large for the shared-memory column");
    ck(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sytrd_panel, TT, vbytes), "occupancy");
    if (per < 1) throw Error(2, "sytrd panel kernel cannot be resident");
    // 1/share of the SMs per tridiagonalisation: the pencils of a QD step
    // reach this point together on their own streams and then share the GPU
    // -- the per-column barrier latency of one overlaps the FP64 products of
    // the others.
    const unsigned G = (unsigned)std::max(1, sms / std::max(1, sm_share(share)));
    T V = alloc(c, {NBP, n}, false), W = alloc(c, {NBP, n}, false), y = alloc(c, {n}, false);
    T accs = alloc(c, {2, PARTS}, true);  // zero: the first column of every panel has parity 0
    T barw = alloc(c, {2}, true);  // Bar (12 bytes) in 16 zeroed bytes
    Bar *bar = (Bar *)barw.p;
    const double mone = -1.0, one = 1.0;
    for (long long j0 = 0; j0 < n; j0 += NBP) {
        const int nbp = (int)std::min<long long>(NBP, n - j0);
        PanelArgs a{A, n, (int)j0, nbp, V.p, W.p, d, e, tau, y.p, accs.p, bar, c.wait_limit ? c.wait_limit : kBarSpin};
        void *args[] = {&a};
        ck(cudaLaunchCooperativeKernel((const void *)k_sytrd_panel, dim3(G), dim3(TT), args, vbytes, c.st),
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
extern "C" unsigned nvpt_context_wait_limit(const nvpt_context *ctx);

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
        c.wait_limit = nvpt_context_wait_limit(ctx);
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
