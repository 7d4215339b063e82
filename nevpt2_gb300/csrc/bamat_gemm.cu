// A-matrices of the (+-1') classes, src/koopro4QD.F90:3974-4104, as dense
// contractions.
//
// The n^9 part of bamat contracts the four-operator products
//   X_{cp,ap}[u,v,d,f,w,z] = <E_{cp ap} E_{u v} E_{d f} E_{w z}> = eeee(cp,ap,u,v,d,f,w,z)
// with the active integrals.  For one "slab" (cp, ap) these are four GEMMs
// (K = n^3, N = n):
//   T1[(bp,b,c),a]  = sum_{d,f,e} X[bp,b,d,f,e,c] atwo(d,f,e,a)
//   T2[(bp,b,a),c]  = sum_{d,f,e} X[bp,b,d,f,a,e] atwo(d,f,c,e)
//   T3[(bp,a,c),b]  = sum_{e,d,f} X[bp,e,d,f,a,c] atwo(d,f,b,e)
//   T3'[(bp,a,c),b] = sum_{e,d,f} X[e,bp,d,f,a,c] atwo(d,f,b,e)
// and, per the reference's loop (amat, plus the EA terms it scatters into the
// b<->bp transposed element):
//   amat(ap,bp,cp,a,b,c)  += T1 - T2 - T3
//   atmat(ap,bp,cp,a,b,c) += -T3' - (T1 - T2)[b <-> bp]
// Everything else of the reference loop -- the one-electron terms, the
// eee2/ee2 terms of the ie loop and the Kronecker-delta pieces of e1t, e2t and
// eeeet -- is lower order and computed per output element by k_bamat_rest.
// The slabs are materialised from the packed 4-RDM (ord8 gathers, delta
// corrections of eeee) in the four K-major layouts the GEMMs read.
#include "nvpt2_internal.h"

#include <cublas_v2.h>

#include <algorithm>
#include <vector>

namespace nvpt {

#define ATWO(i, j, k, l) atwo[((i)-1) + (ll)n * (((j)-1) + (ll)n * (((k)-1) + (ll)n * ((l)-1)))]
#define FF(i, j) f[tri_index((i) + ncore, (j) + ncore) - 1]

// Slab materialisation: one thread per (slab in batch, u,v,d,f,w,z), 0-based.
__global__ void __launch_bounds__(256) k_bamat_slabs(Rdm r, int s, const int *slab_cp, const int *slab_ap,
                                                     int nslab, double *X1, double *X2, double *X3, double *X4) {
    const int n = r.n;
    const ll n3 = (ll)n * n * n, n6 = n3 * n3;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n6 * nslab) return;
    int sl = (int)(t / n6);
    ll x = t % n6;
    const int z = (int)(x % n); x /= n;
    const int w = (int)(x % n); x /= n;
    const int f = (int)(x % n); x /= n;
    const int d = (int)(x % n); x /= n;
    const int v = (int)(x % n); x /= n;
    const int u = (int)x;
    const int cp = slab_cp[sl], ap = slab_ap[sl];
    double val = r.eeee(cp + 1, ap + 1, u + 1, v + 1, d + 1, f + 1, w + 1, z + 1, s + 1);
    ll base = (ll)sl * n6;
    // X1 rows (u,v,z) cols (d,f,w)
    X1[base + (((ll)u * n + v) * n + z) * n3 + ((ll)d * n + f) * n + w] = val;
    // X2 rows (u,v,w) cols (d,f,z)
    X2[base + (((ll)u * n + v) * n + w) * n3 + ((ll)d * n + f) * n + z] = val;
    // X3 rows (u,w,z) cols (v,d,f)
    X3[base + (((ll)u * n + w) * n + z) * n3 + ((ll)v * n + d) * n + f] = val;
    // X4 rows (v,w,z) cols (u,d,f)
    X4[base + (((ll)v * n + w) * n + z) * n3 + ((ll)u * n + d) * n + f] = val;
}

// Integral operands (row-major [K, N]) from the Fortran atwo(n,n,n,n).
__global__ void k_bamat_ints(const double *atwo, int n, double *A1, double *A2, double *A3) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    ll n4 = (ll)n * n * n * n;
    if (t >= n4) return;
    // decode as (p,q,r,s) row-major over [K=(p,q,r), N=s]
    int s4 = (int)(t % n), r3 = (int)((t / n) % n), q2 = (int)((t / (n * n)) % n), p1 = (int)(t / ((ll)n * n * n));
    // A1[(d,f,e), a] = atwo(d,f,e,a)
    A1[t] = ATWO(p1 + 1, q2 + 1, r3 + 1, s4 + 1);
    // A2[(d,f,e), c] = atwo(d,f,c,e)
    A2[t] = ATWO(p1 + 1, q2 + 1, s4 + 1, r3 + 1);
    // A3[(e,d,f), b] = atwo(d,f,b,e)
    A3[t] = ATWO(q2 + 1, r3 + 1, s4 + 1, p1 + 1);
}

// Lower-order terms of the reference loop for one output element (all but
// the eeee(...) products that the GEMMs cover).  Mirrors k_bamat_direct.
__global__ void __launch_bounds__(128) k_bamat_rest(Rdm r, const double *atwo, const double *f, int ncore,
                                                    double *amat, double *atmat) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    ll n6 = (ll)n * n * n * n * n * n;
    if (t >= n6) return;
    ll x = t;
    const int ap = (int)(x % n) + 1; x /= n;
    const int bp = (int)(x % n) + 1; x /= n;
    const int cp = (int)(x % n) + 1; x /= n;
    const int a = (int)(x % n) + 1; x /= n;
    const int b = (int)(x % n) + 1; x /= n;
    const int c = (int)(x % n) + 1;
    for (int s = 1; s <= M; ++s) {
        double A = 0.0, At = 0.0;
        for (int d = 1; d <= n; ++d) {
            double fda = FF(d, a), fcd = FF(c, d), fbd = FF(b, d);
            A += fda * r.eee2(cp, ap, bp, b, d, c, s) - fcd * r.eee2(cp, ap, bp, b, a, d, s) -
                 fbd * r.eee2(cp, ap, bp, d, a, c, s);
            At += fda * r.eee2t(cp, ap, bp, b, d, c, s) - fcd * r.eee2t(cp, ap, bp, b, a, d, s) +
                  fbd * r.eee2t(cp, ap, bp, d, a, c, s);
            for (int ie = 1; ie <= n; ++ie) {
                double dint1 = ATWO(c, ie, d, a), dint2 = ATWO(d, ie, ie, a);
                double dint3 = ATWO(c, d, d, ie), dint4 = ATWO(b, d, d, ie);
                double dum1 = r.eee2(cp, ap, bp, b, d, ie, s);
                double dum2 = r.eee2(cp, ap, bp, b, d, c, s);
                double dum3 = r.eee2(cp, ap, bp, b, a, ie, s);
                double dum4 = r.eee2(cp, ap, bp, ie, a, c, s);
                A += dum1 * dint1 - 0.5 * (dum2 * dint2 + dum3 * dint3 - dum4 * dint4);
                At += 0.5 * r.eee2t(cp, ap, bp, ie, a, c, s) * dint4;
                double m1 = -r.eee2(cp, ap, b, bp, d, ie, s);
                double m2 = -r.eee2(cp, ap, b, bp, d, c, s);
                double m3 = -r.eee2(cp, ap, b, bp, a, ie, s);
                if (b == bp) {
                    m1 += 2.0 * r.ee2(cp, ap, d, ie, s);
                    m2 += 2.0 * r.ee2(cp, ap, d, c, s);
                    m3 += 2.0 * r.ee2(cp, ap, a, ie, s);
                }
                At += m1 * dint1 - 0.5 * (m2 * dint2 + m3 * dint3);
                // delta piece of eeeet(cp,ap,bp,ie,d,ief,a,c): [bp == ie] 2 eee2(cp,ap,d,ief,a,c)
                if (ie == bp)
                    for (int ief = 1; ief <= n; ++ief)
                        At += 2.0 * r.eee2(cp, ap, d, ief, a, c, s) * ATWO(d, ief, b, ie);
                // delta pieces of the mirrored e1t / e2t: [b == bp] 2 eee2(...)
                if (b == bp)
                    for (int ief = 1; ief <= n; ++ief)
                        At += 2.0 * r.eee2(cp, ap, d, ief, ie, c, s) * ATWO(d, ief, ie, a) -
                              2.0 * r.eee2(cp, ap, d, ief, a, ie, s) * ATWO(d, ief, c, ie);
            }
        }
        ll o = (s - 1) + (ll)M * t;
        amat[o] = A;
        atmat[o] = At;
    }
}

// Add the GEMM results: Tk are [(cp,ap) slab][rows][n] with the row layouts
// of the GEMMs above (slab index = cp*n + ap).
__global__ void k_bamat_assemble(int n, int M, int s, const double *T1, const double *T2, const double *T3,
                                 const double *T4, double *amat, double *atmat) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const ll n3 = (ll)n * n * n, n4 = n3 * n;
    ll n6 = n3 * n3;
    if (t >= n6) return;
    ll x = t;
    const int ap = (int)(x % n); x /= n;
    const int bp = (int)(x % n); x /= n;
    const int cp = (int)(x % n); x /= n;
    const int a = (int)(x % n); x /= n;
    const int b = (int)(x % n); x /= n;
    const int c = (int)x;
    const ll sb = ((ll)cp * n + ap) * n4;
    auto row3 = [n](int i, int j, int k) { return (((ll)i * n + j) * n + k) * n; };
    double t1 = T1[sb + row3(bp, b, c) + a];
    double t2 = T2[sb + row3(bp, b, a) + c];
    double t3 = T3[sb + row3(bp, a, c) + b];
    double t4 = T4[sb + row3(bp, a, c) + b];
    double u1 = T1[sb + row3(b, bp, c) + a];
    double u2 = T2[sb + row3(b, bp, a) + c];
    ll o = s + (ll)M * t;
    amat[o] += t1 - t2 - t3;
    atmat[o] += -t4 - (u1 - u2);
}

// ---------------------------------------------------------------------------
struct BamatGemm {
    cublasHandle_t h = nullptr;
    ~BamatGemm() {
        if (h) cublasDestroy(h);
    }
};

static int dgemm_rm(cublasHandle_t h, long long m, long long nn, long long k, const double *A, const double *B,
                    double *C) {
    // row-major C[m,nn] = A[m,k] B[k,nn]  <=>  column-major C^T = B^T A^T
    const double one = 1.0, zero = 0.0;
    return (int)cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, (int)nn, (int)m, (int)k, &one, B, (int)nn, A, (int)k,
                            &zero, C, (int)nn);
}

// Returns 0 on success, else a CUDA / cuBLAS error code (nonzero).
int launch_bamat_gemm(const Rdm &r, const double *atwo, const double *f, int ncore, double *amat, double *atmat,
                      cudaStream_t st, int slabs_per_batch) {
    const int n = r.n, M = r.M;
    const ll n3 = (ll)n * n * n, n4 = n3 * n, n6 = n3 * n3;
    static thread_local BamatGemm handle;
    if (!handle.h && cublasCreate(&handle.h) != CUBLAS_STATUS_SUCCESS) return 1;
    if (cublasSetStream(handle.h, st) != CUBLAS_STATUS_SUCCESS) return 1;
    cublasSetMathMode(handle.h, CUBLAS_DEFAULT_MATH);
    // lower-order part first (writes amat/atmat), then add the GEMM terms
    k_bamat_rest<<<(unsigned)((n6 + 127) / 128), 128, 0, st>>>(r, atwo, f, ncore, amat, atmat);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    double *A1, *A2, *A3, *T, *X;
    const int B = slabs_per_batch;
    if (cudaMallocAsync((void **)&A1, sizeof(double) * 3 * n4, st) != cudaSuccess) return 2;
    A2 = A1 + n4;
    A3 = A2 + n4;
    k_bamat_ints<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(atwo, n, A1, A2, A3);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (cudaMallocAsync((void **)&T, sizeof(double) * 4 * n6, st) != cudaSuccess) return 2;
    if (cudaMallocAsync((void **)&X, sizeof(double) * 4 * (size_t)B * n6, st) != cudaSuccess) return 2;
    int *slabs;
    if (cudaMallocAsync((void **)&slabs, sizeof(int) * 2 * n * n, st) != cudaSuccess) return 2;
    {
        std::vector<int> h(2 * n * n);
        for (int cp = 0; cp < n; ++cp)
            for (int ap = 0; ap < n; ++ap) {
                h[cp * n + ap] = cp;
                h[n * n + cp * n + ap] = ap;
            }
        cudaMemcpyAsync(slabs, h.data(), sizeof(int) * 2 * n * n, cudaMemcpyHostToDevice, st);
        cudaStreamSynchronize(st);
    }
    int rc = 0;
    for (int s = 0; s < M && !rc; ++s) {
        for (int s0 = 0; s0 < n * n && !rc; s0 += B) {
            int nb = std::min(B, n * n - s0);
            double *X1 = X, *X2 = X + (ll)B * n6, *X3 = X2 + (ll)B * n6, *X4 = X3 + (ll)B * n6;
            ll work = (ll)nb * n6;
            k_bamat_slabs<<<(unsigned)((work + 255) / 256), 256, 0, st>>>(r, s, slabs + s0, slabs + n * n + s0, nb, X1,
                                                                        X2, X3, X4);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            ll rows = (ll)nb * n3;
            double *T1 = T + (ll)s0 * n4, *T2 = T + n6 + (ll)s0 * n4, *T3 = T + 2 * n6 + (ll)s0 * n4,
                   *T4 = T + 3 * n6 + (ll)s0 * n4;
            rc |= dgemm_rm(handle.h, rows, n, n3, X1, A1, T1);
            rc |= dgemm_rm(handle.h, rows, n, n3, X2, A2, T2);
            rc |= dgemm_rm(handle.h, rows, n, n3, X3, A3, T3);
            rc |= dgemm_rm(handle.h, rows, n, n3, X4, A3, T4);
        }
        if (!rc) {
            k_bamat_assemble<<<(unsigned)((n6 + 255) / 256), 256, 0, st>>>(n, M, s, T, T + n6, T + 2 * n6, T + 3 * n6,
                                                                        amat, atmat);
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
    }
    cudaFreeAsync(slabs, st);
    cudaFreeAsync(X, st);
    cudaFreeAsync(T, st);
    cudaFreeAsync(A1, st);
    return rc ? 3 : 0;
}

}  // namespace nvpt
