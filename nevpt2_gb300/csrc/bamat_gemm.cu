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
// eeeet -- is lower order; it is evaluated as n^8 GEMMs plus n^7 per-element
// sums (bamat_rest below).
// The slabs are materialised from the packed 4-RDM (ord8 gathers, delta
// corrections of eeee) in the four K-major layouts the GEMMs read.
#include "nvpt2_internal.h"
#include "ozaki.cuh"
#include "tuner.h"

#include <cublas_v2.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
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

// Tiled slab materialisation: one block per (slab, u, v, d) evaluates the n^3
// products for all (f, w, z) into shared memory, then writes each layout
// with consecutive threads on consecutive addresses (n^2 doubles per row
// segment for X1/X2, n for X3/X4).  The tile is [f][w][z] with odd strides
// (n+1, n(n+1)+1 doubles), so every read pattern is free of bank conflicts.
// With rmax, the block also folds the magnitudes into the row maxima of the
// four layouts (bit patterns of non-negative doubles order like integers):
// rmax[L * nslab n^3 + row] for layout L.
constexpr int kSlabTileMax = 16 * (16 * 17 + 1);
__global__ void __launch_bounds__(256) k_bamat_slabs_t(Rdm r, int s, const int *slab_cp, const int *slab_ap,
                                                       int nslab, double *X1, double *X2, double *X3, double *X4,
                                                       unsigned long long *rmax) {
    __shared__ double tile[kSlabTileMax];
    __shared__ double mwz[256];
    const int n = r.n, sw = n + 1, sf = n * (n + 1) + 1;
    const ll n2 = (ll)n * n, n3 = n2 * n, n6 = n3 * n3;
    ll b = blockIdx.x;
    const int d = (int)(b % n); b /= n;
    const int v = (int)(b % n); b /= n;
    const int u = (int)(b % n); b /= n;
    const int sl = (int)b;
    const int cp = slab_cp[sl], ap = slab_ap[sl];
    for (int i = threadIdx.x; i < n3; i += blockDim.x) {
        const int z = i % n, w = (i / n) % n, f = i / (int)n2;
        tile[f * sf + w * sw + z] = r.eeee(cp + 1, ap + 1, u + 1, v + 1, d + 1, f + 1, w + 1, z + 1, s + 1);
    }
    __syncthreads();
    const ll base = (ll)sl * n6;
    for (int i = threadIdx.x; i < n3; i += blockDim.x) {
        // X1 rows (u,v,z) cols (d,f,w): i = (z, f, w)
        {
            const int w = i % n, f = (i / n) % n, z = i / (int)n2;
            X1[base + (((ll)u * n + v) * n + z) * n3 + ((ll)d * n + f) * n + w] = tile[f * sf + w * sw + z];
        }
        // X2 rows (u,v,w) cols (d,f,z): i = (w, f, z)
        {
            const int z = i % n, f = (i / n) % n, w = i / (int)n2;
            X2[base + (((ll)u * n + v) * n + w) * n3 + ((ll)d * n + f) * n + z] = tile[f * sf + w * sw + z];
        }
        // X3 rows (u,w,z) cols (v,d,f), X4 rows (v,w,z) cols (u,d,f): i = (w, z, f)
        {
            const int f = i % n, z = (i / n) % n, w = i / (int)n2;
            const double x = tile[f * sf + w * sw + z];
            X3[base + (((ll)u * n + w) * n + z) * n3 + ((ll)v * n + d) * n + f] = x;
            X4[base + (((ll)v * n + w) * n + z) * n3 + ((ll)u * n + d) * n + f] = x;
        }
    }
    if (!rmax) return;
    // m(w,z) = max_f |x|: the X3 / X4 partials; X1 (row z) = max_w, X2 (row w) = max_z
    for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int z = i % n, w = i / n;
        double m = 0.0;
        for (int f = 0; f < n; ++f) m = fmax(m, fabs(tile[f * sf + w * sw + z]));
        mwz[i] = m;
    }
    __syncthreads();
    const ll rows = (ll)nslab * n3, r0 = (ll)sl * n3;
    for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int z = i % n, w = i / n;
        const unsigned long long m = (unsigned long long)__double_as_longlong(mwz[i]);
        atomicMax(rmax + 2 * rows + r0 + ((ll)u * n + w) * n + z, m);
        atomicMax(rmax + 3 * rows + r0 + ((ll)v * n + w) * n + z, m);
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double m1 = 0.0, m2 = 0.0;
        for (int j = 0; j < n; ++j) {
            m1 = fmax(m1, mwz[j * n + i]);  // row z = i: over w
            m2 = fmax(m2, mwz[i * n + j]);  // row w = i: over z
        }
        atomicMax(rmax + 0 * rows + r0 + ((ll)u * n + v) * n + i, (unsigned long long)__double_as_longlong(m1));
        atomicMax(rmax + 1 * rows + r0 + ((ll)u * n + v) * n + i, (unsigned long long)__double_as_longlong(m2));
    }
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

// ---------------------------------------------------------------------------
// Lower-order terms (everything of the reference loop but the eeee products).
//
// With the three-operator products materialised once per state,
//   E2[cp,ap,x3,x4,x5,x6]  = eee2(cp,ap,x3,x4,x5,x6)   (n^6)
//   E2t[cp,ap,x3,x4,x5,x6] = eee2t(cp,ap,x3,x4,x5,x6)  (n^6)
//   EE2[cp,ap,x3,x4]       = ee2(cp,ap,x3,x4)          (n^4)
// and K(x,y) = sum_z atwo(x,z,z,y), f the active block of f(*),
// Fm = f - K/2, Fp = f + K/2, the ie/ief sums of the loop collapse to
//   amat  = sum_d [E2[cp,ap,bp,b,d,c] Fm(d,a) - E2[cp,ap,bp,b,a,d] Fp(c,d)
//                  - E2[cp,ap,bp,d,a,c] Fm(b,d)] + T[cp,ap,bp,b,c,a]
//   atmat = sum_d [E2t[cp,ap,bp,b,d,c] f(d,a) - E2t[cp,ap,bp,b,a,d] f(c,d)
//                  + E2t[cp,ap,bp,d,a,c] Fp(b,d) + E2[cp,ap,b,bp,d,c] K(d,a)/2
//                  + E2[cp,ap,b,bp,a,d] K(c,d)/2]
//           - T[cp,ap,b,bp,c,a] + 2 V[cp,ap,a,c,b,bp] + [b == bp] D[cp,ap,c,a]
// with the n^8 contractions (GEMMs)
//   T[cp,ap,bp,b,c,a] = sum_{d,e} E2[cp,ap,bp,b,d,e] atwo(c,e,d,a)
//   V[cp,ap,a,c,b,bp] = sum_{d,e} E2[cp,ap,d,e,a,c] atwo(d,e,b,bp)
// and the n^7 delta block
//   D[cp,ap,c,a] = 2 sum_{d,e} EE2[cp,ap,d,e] atwo(c,e,d,a)
//                - sum_d EE2[cp,ap,d,c] K(d,a) - sum_d EE2[cp,ap,a,d] K(c,d)
//                + 2 sum_{d,e,g} (E2[cp,ap,d,e,g,c] atwo(d,e,g,a) - E2[cp,ap,d,e,a,g] atwo(d,e,c,g)).
// (The reference's loop at src/koopro4QD.F90:4008-4100 sums the same terms
// element by element.)  All dense tensors keep (cp,ap) as their two fastest
// indices, so the per-output kernels read them coalesced along ap.

// 0-based row-major offset of X[x3,x4,x5,x6,cp,ap] ("cp,ap last" layout).
#define RX6(x3, x4, x5, x6) (((((ll)(x3) * n + (x4)) * n + (x5)) * n + (x6)) * n2 + cpap)

__global__ void __launch_bounds__(256) k_rest_dense(Rdm r, int s, double *E2, double *E2t, double *EE2) {
    const int n = r.n;
    const ll n4 = (ll)n * n * n * n, n6 = n4 * n * n;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n6) return;
    ll x = t;
    const int ap = (int)(x % n); x /= n;
    const int cp = (int)(x % n); x /= n;
    const int x6 = (int)(x % n); x /= n;
    const int x5 = (int)(x % n); x /= n;
    const int x4 = (int)(x % n); x /= n;
    const int x3 = (int)x;
    E2[t] = r.eee2(cp + 1, ap + 1, x3 + 1, x4 + 1, x5 + 1, x6 + 1, s + 1);
    E2t[t] = r.eee2t(cp + 1, ap + 1, x3 + 1, x4 + 1, x5 + 1, x6 + 1, s + 1);
    // for t < n^4 the decode gives x3 = x4 = 0 and (x5, x6, cp, ap) = EE2 layout
    if (t < n4) EE2[t] = r.ee2(cp + 1, ap + 1, x5 + 1, x6 + 1, s + 1);
}

// Small operands: Fs = [f | K | Fm | Fp] (4 n x n, row-major [x][y]),
// G[(d,e),(c,a)] = atwo(c,e,d,a) and H[(d,e),(b,bp)] = atwo(d,e,b,bp).
__global__ void k_rest_ints(const double *atwo, const double *f, int ncore, int n, double *Fs, double *G,
                            double *H) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const ll n2 = (ll)n * n, n4 = n2 * n2;
    if (t >= n4) return;
    ll x = t;
    const int q4 = (int)(x % n); x /= n;
    const int q3 = (int)(x % n); x /= n;
    const int q2 = (int)(x % n); x /= n;
    const int q1 = (int)x;
    // t = ((q1*n + q2)*n + q3)*n + q4
    G[t] = ATWO(q3 + 1, q2 + 1, q1 + 1, q4 + 1);  // (d,e)=(q1,q2), (c,a)=(q3,q4)
    H[t] = ATWO(q1 + 1, q2 + 1, q3 + 1, q4 + 1);  // (d,e)=(q1,q2), (b,bp)=(q3,q4)
    if (t < n2) {
        const int i = (int)(t / n), j = (int)(t % n);
        double k = 0.0;
        for (int z = 1; z <= n; ++z) k += ATWO(i + 1, z, z, j + 1);
        const double fij = FF(i + 1, j + 1);
        Fs[t] = fij;
        Fs[n2 + t] = k;
        Fs[2 * n2 + t] = fij - 0.5 * k;
        Fs[3 * n2 + t] = fij + 0.5 * k;
    }
}

// D[c,a,cp,ap] (n^4 outputs, ap fastest).  U = the EE2 x atwo GEMM, same layout.
__global__ void __launch_bounds__(256) k_rest_delta(int n, const double *atwo, const double *Fs, const double *E2,
                                                    const double *EE2, const double *U, double *D) {
    const ll n2 = (ll)n * n, n4 = n2 * n2;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n4) return;
    const ll cpap = t % n2;
    const int a = (int)((t / n2) % n), c = (int)(t / (n2 * n));
    const double *K = Fs + n2;
    double acc = 2.0 * U[t];
    for (int d = 0; d < n; ++d)
        acc -= EE2[((ll)d * n + c) * n2 + cpap] * K[d * n + a] + EE2[((ll)a * n + d) * n2 + cpap] * K[c * n + d];
    double p = 0.0;
    for (int d = 0; d < n; ++d)
        for (int e = 0; e < n; ++e)
            for (int g = 0; g < n; ++g)
                p += E2[RX6(d, e, g, c)] * ATWO(d + 1, e + 1, g + 1, a + 1) -
                     E2[RX6(d, e, a, g)] * ATWO(d + 1, e + 1, c + 1, g + 1);
    D[t] = acc + 2.0 * p;
}

// Writes amat/atmat(s, ap,bp,cp,a,b,c) (=, not +=) with the lower-order terms.
__global__ void __launch_bounds__(256) k_rest_out(int n, int M, int s, const double *Fs, const double *E2,
                                                  const double *E2t, const double *T, const double *V,
                                                  const double *D, double *amat, double *atmat) {
    __shared__ double sF[4 * 16 * 16];
    const ll n2 = (ll)n * n, n4 = n2 * n2;
    for (int i = threadIdx.x; i < 4 * n2; i += blockDim.x) sF[i] = Fs[i];
    __syncthreads();
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const ll n6 = n4 * n2;
    if (t >= n6) return;
    ll x = t;
    const int ap = (int)(x % n); x /= n;
    const int bp = (int)(x % n); x /= n;
    const int cp = (int)(x % n); x /= n;
    const int a = (int)(x % n); x /= n;
    const int b = (int)(x % n); x /= n;
    const int c = (int)x;
    const ll cpap = (ll)cp * n + ap;
    const double *f = sF, *K = sF + n2, *Fm = sF + 2 * n2, *Fp = sF + 3 * n2;
    double A = 0.0, At = 0.0;
    for (int d = 0; d < n; ++d) {
        A += E2[RX6(bp, b, d, c)] * Fm[d * n + a] - E2[RX6(bp, b, a, d)] * Fp[c * n + d] -
             E2[RX6(bp, d, a, c)] * Fm[b * n + d];
        At += E2t[RX6(bp, b, d, c)] * f[d * n + a] - E2t[RX6(bp, b, a, d)] * f[c * n + d] +
              E2t[RX6(bp, d, a, c)] * Fp[b * n + d] +
              0.5 * (E2[RX6(b, bp, d, c)] * K[d * n + a] + E2[RX6(b, bp, a, d)] * K[c * n + d]);
    }
    A += T[RX6(bp, b, c, a)];
    At += 2.0 * V[RX6(b, bp, a, c)] - T[RX6(b, bp, c, a)];
    if (b == bp) At += D[((ll)c * n + a) * n2 + cpap];
    const ll o = s + (ll)M * t;
    amat[o] = A;
    atmat[o] = At;
}
#undef RX6

// row-major C[m,nn] = A^T B with A [k,m] and B [k,nn] row-major (batched over
// B and C with the given strides; A shared).
static int dgemm_rm_tA(cublasHandle_t h, long long m, long long nn, long long k, const double *A, const double *B,
                       long long strideB, double *C, long long strideC, int batch) {
    const double one = 1.0, zero = 0.0;
    if (batch == 1)
        return (int)cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, (int)nn, (int)m, (int)k, &one, B, (int)nn, A, (int)m,
                                &zero, C, (int)nn);
    return (int)cublasDgemmStridedBatched(h, CUBLAS_OP_N, CUBLAS_OP_T, (int)nn, (int)m, (int)k, &one, B, (int)nn,
                                          strideB, A, (int)m, 0, &zero, C, (int)nn, strideC, batch);
}

// Lower-order part of bamat for state s into amat/atmat; scratch holds
// 4 n^6 + 5 n^4 + 4 n^2 doubles.
static int bamat_rest(cublasHandle_t h, const Rdm &r, int s, const double *atwo, const double *f, int ncore,
                      double *amat, double *atmat, double *scratch, cudaStream_t st) {
    const int n = r.n, M = r.M;
    const ll n2 = (ll)n * n, n4 = n2 * n2, n6 = n4 * n2;
    double *E2 = scratch, *E2t = E2 + n6, *T = E2t + n6, *V = T + n6;
    double *EE2 = V + n6, *U = EE2 + n4, *D = U + n4, *G = D + n4, *H = G + n4, *Fs = H + n4;
    k_rest_dense<<<(unsigned)((n6 + 255) / 256), 256, 0, st>>>(r, s, E2, E2t, EE2);
    k_rest_ints<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(atwo, f, ncore, n, Fs, G, H);
    g_launches.fetch_add(2, std::memory_order_relaxed);
    int rc = 0;
    // T[(bp,b)][(c,a),(cp,ap)] = G^T E2[(bp,b)][(d,e),(cp,ap)]
    rc |= dgemm_rm_tA(h, n2, n2, n2, G, E2, n4, T, n4, (int)n2);
    // V[(b,bp),(a,c,cp,ap)] = H^T E2[(d,e),(a,c,cp,ap)]
    rc |= dgemm_rm_tA(h, n2, n4, n2, H, E2, 0, V, 0, 1);
    // U[(c,a),(cp,ap)] = G^T EE2[(d,e),(cp,ap)]
    rc |= dgemm_rm_tA(h, n2, n2, n2, G, EE2, 0, U, 0, 1);
    if (rc) return rc;
    k_rest_delta<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(n, atwo, Fs, E2, EE2, U, D);
    k_rest_out<<<(unsigned)((n6 + 255) / 256), 256, 0, st>>>(n, M, s, Fs, E2, E2t, T, V, D, amat, atmat);
    g_launches.fetch_add(2, std::memory_order_relaxed);
    return 0;
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
// FP64 slab products.  Per slab batch the four contractions are row-major
// C[rows, N] = X[rows, K] B[K, N] with K = n^3 and N = n <= 16: skinny
// products whose cost is the FP64 pipe alone (2 FMA/clock/SM on GB300; the
// 8 flops per X byte loaded are far above the HBM balance point), so the
// kernel only has to keep that pipe busy.  One CTA computes a BM x 16 tile
// (BM = 32 RPT; columns beyond N are zero in shared memory and never
// stored); 256 threads, each an RPT x 2 register block; X is staged 32
// columns at a time, transposed in shared memory (stride BM + 1 doubles) so
// that a thread's rows at one k are contiguous, with the next chunk's global
// loads issued before the current chunk's FMAs.  blockIdx.y selects one of up
// to four products.  The tile height RPT is tuned per shape (tuner.h).
constexpr int kSkBK = 32;
struct SkinnyJobs {
    const double *X[4];
    const double *B[4];
    double *C[4];
};

template <int RPT>
__global__ void __launch_bounds__(256, 2) k_dgemm_skinny(SkinnyJobs jobs, ll rows, int N, int K) {
    constexpr int BM = 32 * RPT, LD = BM + 1, NX = BM / 8;
    __shared__ double Xs[kSkBK * LD];
    __shared__ __align__(16) double Bs[kSkBK * 16];
    // constant indices only (a dynamic index would copy the struct to local memory)
    const int jb = blockIdx.y;
    const double *__restrict__ X = jb == 0 ? jobs.X[0] : jb == 1 ? jobs.X[1] : jb == 2 ? jobs.X[2] : jobs.X[3];
    const double *__restrict__ B = jb == 0 ? jobs.B[0] : jb == 1 ? jobs.B[1] : jb == 2 ? jobs.B[2] : jobs.B[3];
    double *__restrict__ C = jb == 0 ? jobs.C[0] : jb == 1 ? jobs.C[1] : jb == 2 ? jobs.C[2] : jobs.C[3];
    const int tid = threadIdx.x;
    const ll r0 = (ll)blockIdx.x * BM;
    // loader mapping: lane = k within the chunk, warp = row (+ 8 i)
    const int lk = tid & 31, lr = tid >> 5;
    // compute mapping: RPT rows (tr*RPT..) x 2 columns (2 tc, 2 tc + 1)
    const int tc = tid & 7, tr = tid >> 3;
    double xr[NX], br[2];
    auto load = [&](int k0) {
        const int k = k0 + lk;
#pragma unroll
        for (int i = 0; i < NX; ++i) {
            const ll r = r0 + lr + 8 * i;
            xr[i] = (r < rows && k < K) ? X[r * K + k] : 0.0;
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int e = tid + 256 * i, kk = e >> 4, c = e & 15;
            br[i] = (c < N && k0 + kk < K) ? B[(ll)(k0 + kk) * N + c] : 0.0;
        }
    };
    double acc[RPT][2] = {};
    load(0);
    for (int k0 = 0; k0 < K; k0 += kSkBK) {
#pragma unroll
        for (int i = 0; i < NX; ++i) Xs[lk * LD + lr + 8 * i] = xr[i];
#pragma unroll
        for (int i = 0; i < 2; ++i) Bs[tid + 256 * i] = br[i];
        __syncthreads();
        if (k0 + kSkBK < K) load(k0 + kSkBK);
#pragma unroll 8
        for (int k = 0; k < kSkBK; ++k) {
            const double *xs = Xs + k * LD + tr * RPT;
            const double2 b = *reinterpret_cast<const double2 *>(Bs + k * 16 + 2 * tc);
#pragma unroll
            for (int i = 0; i < RPT; ++i) {
                const double x = xs[i];
                acc[i][0] = fma(x, b.x, acc[i][0]);
                acc[i][1] = fma(x, b.y, acc[i][1]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < RPT; ++i) {
        const ll r = r0 + tr * RPT + i;
        if (r >= rows) continue;
#pragma unroll
        for (int j = 0; j < 2; ++j)
            if (2 * tc + j < N) C[r * N + 2 * tc + j] = acc[i][j];
    }
}

// The same product on the FP64 tensor cores: mma.sync m8n8k4 (DMMA).  CTA
// tile 128 x 16 as above (X staged transposed, B as [k][16] in shared
// memory); warp w owns rows 16w .. 16w+15 as two 8-row blocks times two 8-col
// blocks, four accumulators of two doubles per lane.  Fragments (PTX m8n8k4
// .f64): A a0 = A[lane/4][lane%4], B b0 = B[lane%4][lane/4], C c0,c1 =
// C[lane/4][2(lane%4) + {0,1}].
__global__ void __launch_bounds__(256, 2) k_dgemm_skinny_dmma(SkinnyJobs jobs, ll rows, int N, int K) {
    constexpr int BM = 128, LD = BM + 1, NX = BM / 8;
    __shared__ double Xs[kSkBK * LD];
    __shared__ __align__(16) double Bs[kSkBK * 16];
    const int jb = blockIdx.y;
    const double *__restrict__ X = jb == 0 ? jobs.X[0] : jb == 1 ? jobs.X[1] : jb == 2 ? jobs.X[2] : jobs.X[3];
    const double *__restrict__ B = jb == 0 ? jobs.B[0] : jb == 1 ? jobs.B[1] : jb == 2 ? jobs.B[2] : jobs.B[3];
    double *__restrict__ C = jb == 0 ? jobs.C[0] : jb == 1 ? jobs.C[1] : jb == 2 ? jobs.C[2] : jobs.C[3];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const ll r0 = (ll)blockIdx.x * BM;
    const int lk = tid & 31, lr = tid >> 5;
    double xr[NX], br[2];
    auto load = [&](int k0) {
        const int k = k0 + lk;
#pragma unroll
        for (int i = 0; i < NX; ++i) {
            const ll r = r0 + lr + 8 * i;
            xr[i] = (r < rows && k < K) ? X[r * K + k] : 0.0;
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int e = tid + 256 * i, kk = e >> 4, c = e & 15;
            br[i] = (c < N && k0 + kk < K) ? B[(ll)(k0 + kk) * N + c] : 0.0;
        }
    };
    double acc[2][2][2] = {};  // [m block][n block][c0, c1]
    const int g = lane >> 2, q = lane & 3;
    load(0);
    for (int k0 = 0; k0 < K; k0 += kSkBK) {
#pragma unroll
        for (int i = 0; i < NX; ++i) Xs[lk * LD + lr + 8 * i] = xr[i];
#pragma unroll
        for (int i = 0; i < 2; ++i) Bs[tid + 256 * i] = br[i];
        __syncthreads();
        if (k0 + kSkBK < K) load(k0 + kSkBK);
#pragma unroll
        for (int kk = 0; kk < kSkBK; kk += 4) {
            double a[2], b[2];
#pragma unroll
            for (int mb = 0; mb < 2; ++mb) a[mb] = Xs[(kk + q) * LD + warp * 16 + mb * 8 + g];
#pragma unroll
            for (int nb = 0; nb < 2; ++nb) b[nb] = Bs[(kk + q) * 16 + nb * 8 + g];
#pragma unroll
            for (int mb = 0; mb < 2; ++mb)
#pragma unroll
                for (int nb = 0; nb < 2; ++nb)
                    asm volatile(
                        "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                        : "+d"(acc[mb][nb][0]), "+d"(acc[mb][nb][1])
                        : "d"(a[mb]), "d"(b[nb]));
        }
        __syncthreads();
    }
#pragma unroll
    for (int mb = 0; mb < 2; ++mb) {
        const ll r = r0 + warp * 16 + mb * 8 + g;
        if (r >= rows) continue;
#pragma unroll
        for (int nb = 0; nb < 2; ++nb)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int col = nb * 8 + 2 * q + i;
                if (col < N) C[r * N + col] = acc[mb][nb][i];
            }
    }
}

// variant: 2, 4 = DFMA register blocks of 2 or 4 rows per thread; 1 = DMMA
static void launch_skinny(int rpt, cudaStream_t st, const SkinnyJobs &j, ll rows, int N, int K) {
    if (rpt == 1) {
        dim3 grid((unsigned)((rows + 127) / 128), 4);
        k_dgemm_skinny_dmma<<<grid, 256, 0, st>>>(j, rows, N, K);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return;
    }
    const ll bm = 32LL * rpt;
    dim3 grid((unsigned)((rows + bm - 1) / bm), 4);
    if (rpt == 2) k_dgemm_skinny<2><<<grid, 256, 0, st>>>(j, rows, N, K);
    else k_dgemm_skinny<4><<<grid, 256, 0, st>>>(j, rows, N, K);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

static int dgemm_skinny4(cudaStream_t st, ll rows, int N, int K, const double *const X[4], const double *const B[4],
                         double *const C[4]) {
    SkinnyJobs j;
    for (int i = 0; i < 4; ++i) {
        j.X[i] = X[i];
        j.B[i] = B[i];
        j.C[i] = C[i];
    }
    // rows per thread (tile height 32 RPT), tuned per shape
    // variant, tuned per shape: DFMA with 2 or 4 rows per thread, or DMMA;
    // NVPT_SKINNY_VARIANT (1, 2, 4) fixes it (tests of each variant)
    static const int kRpt[] = {2, 4, 1};
    static const int forced = [] {
        const char *e = std::getenv("NVPT_SKINNY_VARIANT");
        const int v = e ? std::atoi(e) : 0;
        return (v == 1 || v == 2 || v == 4) ? v : 0;
    }();
    if (forced) {
        launch_skinny(forced, st, j, rows, N, K);
        return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
    }
    const std::string key = "bamat_skinny.rows_per_thread/" + std::to_string(rows) + "x" + std::to_string(K) + "x" +
                            std::to_string(N);
    int used = -1;
    const int rpt = tune::choose(key, kRpt, 3, 4, st, [&](int c) { launch_skinny(c, st, j, rows, N, K); used = c; });
    if (used < 0) launch_skinny(rpt, st, j, rows, N, K);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
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

// Device buffers of one launch_bamat_gemm call, released on every return path
// (stream-ordered frees on the call's stream).
struct AsyncBuffers {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit AsyncBuffers(cudaStream_t s) : st(s) {}
    template <class T>
    bool get(T **p, size_t bytes) {
        void *q = nullptr;
        if (cudaMallocAsync(&q, bytes, st) != cudaSuccess) return false;
        ptrs.push_back(q);
        *p = (T *)q;
        return true;
    }
    ~AsyncBuffers() {
        for (auto it = ptrs.rbegin(); it != ptrs.rend(); ++it) cudaFreeAsync(*it, st);
    }
};

__global__ void k_slab_list(int n, int *cp, int *ap);

// Returns 0 on success, else a CUDA / cuBLAS error code (nonzero).
int launch_bamat_gemm(const Rdm &r, const double *atwo, const double *f, int ncore, double *amat, double *atmat,
                      cudaStream_t st, int slabs_per_batch, bool split) {
    const int n = r.n, M = r.M;
    const ll n3 = (ll)n * n * n, n4 = n3 * n, n6 = n3 * n3;
    static thread_local BamatGemm handle;
    if (!handle.h && cublasCreate(&handle.h) != CUBLAS_STATUS_SUCCESS) return 1;
    if (cublasSetStream(handle.h, st) != CUBLAS_STATUS_SUCCESS) return 1;
    cublasSetMathMode(handle.h, CUBLAS_DEFAULT_MATH);
    // lower-order part first (writes amat/atmat), then add the GEMM terms
    {
        AsyncBuffers rest(st);
        double *scr;
        const ll n2 = (ll)n * n;
        if (!rest.get(&scr, sizeof(double) * (4 * n6 + 5 * n4 + 4 * n2))) return 2;
        int rrc = 0;
        for (int s = 0; s < M && !rrc; ++s) rrc = bamat_rest(handle.h, r, s, atwo, f, ncore, amat, atmat, scr, st);
        if (rrc) return 3;
    }
    AsyncBuffers buf(st);
    double *A1, *A2, *A3, *T, *X[2];
    const int B = slabs_per_batch;
    int *slabs;
    if (!buf.get(&A1, sizeof(double) * 3 * n4) || !buf.get(&T, sizeof(double) * 4 * n6) ||
        !buf.get(&X[0], sizeof(double) * 4 * (size_t)B * n6) || !buf.get(&X[1], sizeof(double) * 4 * (size_t)B * n6) ||
        !buf.get(&slabs, sizeof(int) * 2 * n * n))
        return 2;
    A2 = A1 + n4;
    A3 = A2 + n4;
    k_bamat_ints<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(atwo, n, A1, A2, A3);
    k_slab_list<<<(unsigned)((n * n + 255) / 256), 256, 0, st>>>(n, slabs, slabs + n * n);
    g_launches.fetch_add(2, std::memory_order_relaxed);
    int rc = 0;
    // split precision: digit workspace for a full batch of slabs
    void *ozw = nullptr;
    unsigned long long *rmax[2] = {nullptr, nullptr};  // row maxima of the four slab layouts (split digits)
    if (split) {
        oz::OzPlan pl(4, (ll)B * n3, (int)n3, n);
        if (!buf.get(&ozw, pl.bytes()) || !buf.get(&rmax[0], sizeof(unsigned long long) * 4 * (size_t)B * n3) ||
            !buf.get(&rmax[1], sizeof(unsigned long long) * 4 * (size_t)B * n3))
            return 2;
    }
    // Slab production (gather-bound on the packed 4-RDM) runs one batch ahead
    // on a stream of its own into the other of two slab buffers, so that it
    // overlaps the products of the current batch (FP64 pipe, or HBM-bound
    // digit streams in split mode).  Events order buffer reuse; the guard
    // joins the producer stream into st before the buffers are released
    // (it is destroyed before `buf`).
    struct Producer {
        cudaStream_t st, g = nullptr;
        cudaEvent_t in = nullptr, gen[2] = {nullptr, nullptr}, use[2] = {nullptr, nullptr}, end = nullptr;
        bool ok = false;
        explicit Producer(cudaStream_t s) : st(s) {
            ok = cudaStreamCreateWithFlags(&g, cudaStreamNonBlocking) == cudaSuccess;
            for (cudaEvent_t *e : {&in, &gen[0], &gen[1], &use[0], &use[1], &end})
                ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
            ok = ok && cudaEventRecord(in, st) == cudaSuccess && cudaStreamWaitEvent(g, in, 0) == cudaSuccess;
        }
        ~Producer() {
            if (g && end) {
                cudaEventRecord(end, g);
                cudaStreamWaitEvent(st, end, 0);
            }
            for (cudaEvent_t e : {in, gen[0], gen[1], use[0], use[1], end})
                if (e) cudaEventDestroy(e);
            if (g) cudaStreamDestroy(g);
        }
    } prod(st);
    if (!prod.ok) return 1;
    const int per_state = (n * n + B - 1) / B, nbatch = M * per_state;
    auto batch = [&](int gb, int &s, int &s0, int &nb) {
        s = gb / per_state;
        s0 = (gb % per_state) * B;
        nb = std::min(B, n * n - s0);
    };
    auto produce = [&](int gb) {
        int s, s0, nb;
        batch(gb, s, s0, nb);
        const int q = gb & 1;
        if (gb >= 2) cudaStreamWaitEvent(prod.g, prod.use[q], 0);
        const ll rows = (ll)nb * n3;
        double *X1 = X[q], *X2 = X1 + (ll)B * n6, *X3 = X2 + (ll)B * n6, *X4 = X3 + (ll)B * n6;
        if (rmax[q]) cudaMemsetAsync(rmax[q], 0, sizeof(unsigned long long) * 4 * (size_t)rows, prod.g);
        k_bamat_slabs_t<<<(unsigned)rows, 256, 0, prod.g>>>(r, s, slabs + s0, slabs + n * n + s0, nb, X1, X2, X3, X4,
                                                             rmax[q]);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        cudaEventRecord(prod.gen[q], prod.g);
    };
    produce(0);
    for (int gb = 0; gb < nbatch && !rc; ++gb) {
        if (gb + 1 < nbatch) produce(gb + 1);
        int s, s0, nb;
        batch(gb, s, s0, nb);
        const int q = gb & 1;
        cudaStreamWaitEvent(st, prod.gen[q], 0);
        const ll rows = (ll)nb * n3;
        double *X1 = X[q], *X2 = X1 + (ll)B * n6, *X3 = X2 + (ll)B * n6, *X4 = X3 + (ll)B * n6;
        double *T1 = T + (ll)s0 * n4, *T2 = T + n6 + (ll)s0 * n4, *T3 = T + 2 * n6 + (ll)s0 * n4,
               *T4 = T + 3 * n6 + (ll)s0 * n4;
        const double *Xs[4] = {X1, X2, X3, X4}, *As[4] = {A1, A2, A3, A3};
        double *Ts[4] = {T1, T2, T3, T4};
        if (split) {
            const unsigned long long *Rm[4] = {rmax[q], rmax[q] + rows, rmax[q] + 2 * rows, rmax[q] + 3 * rows};
            rc |= oz::oz_gemm_skinny(oz::OzPlan(4, rows, (int)n3, n), Xs, As, Ts, n, n, ozw, st, Rm);
        } else {
            rc |= dgemm_skinny4(st, rows, n, (int)n3, Xs, As, Ts);
        }
        cudaEventRecord(prod.use[q], st);
        if (!rc && s0 + nb == n * n) {  // last batch of state s
            k_bamat_assemble<<<(unsigned)((n6 + 255) / 256), 256, 0, st>>>(n, M, s, T, T + n6, T + 2 * n6, T + 3 * n6,
                                                                        amat, atmat);
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
    }
    // the product kernels share one error flag (a wait that timed out)
    if (ozw && !rc && oz::oz_check_error(ozw, st) != 0) rc = 5;
    return rc == 5 ? 5 : (rc ? 3 : 0);
}

// ===========================================================================
// No-allocation variant (nvpt_bamat_static_d).  Same kernels and the same
// sequence of contractions as launch_bamat_gemm, but every scratch word lives
// in one file-scope device array and the GEMMs run on k_dgemm_small below
// instead of cuBLAS (whose handles and workspaces allocate).  One slab is
// processed at a time and assembled right away, so the scratch is
//   max(rest: 4n^6 + 5n^4 + 4n^2, slabs: 4n^6 + 7n^4 + n^2)  doubles,
// 1,077,312 doubles (8.6 MB) at the maximum of 8 active orbitals.  No word of
// it has to start at zero: every call writes each word before reading it.
// Calls that overlap in time (two streams, two host threads, or two devices'
// contexts sharing the module on one device) race on this array.

static __device__ __align__(256) double g_bamat_scratch[kBamatStaticDoubles];

// Row-major C[m,nn] = op(A) B, op(A) = A [m,k] or, with ta, A^T for A [k,m];
// B [k,nn].  blockIdx.z selects the batch (strides sA, sB, sC).
__global__ void __launch_bounds__(256) k_dgemm_small(int m, int nn, int k, int ta, const double *A, ll sA,
                                                     const double *B, ll sB, double *C, ll sC) {
    __shared__ double As[16][17], Bs[16][17];
    const int tx = threadIdx.x, ty = threadIdx.y;
    A += (ll)blockIdx.z * sA;
    B += (ll)blockIdx.z * sB;
    C += (ll)blockIdx.z * sC;
    const int row = blockIdx.y * 16 + ty, col = blockIdx.x * 16 + tx;
    double acc = 0.0;
    for (int k0 = 0; k0 < k; k0 += 16) {
        const int ka = k0 + tx, kb = k0 + ty;
        As[ty][tx] = (row < m && ka < k) ? (ta ? A[(ll)ka * m + row] : A[(ll)row * k + ka]) : 0.0;
        Bs[ty][tx] = (kb < k && col < nn) ? B[(ll)kb * nn + col] : 0.0;
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) acc += As[ty][q] * Bs[q][tx];
        __syncthreads();
    }
    if (row < m && col < nn) C[(ll)row * nn + col] = acc;
}

static void dgemm_small(cudaStream_t st, ll m, ll nn, ll k, bool ta, const double *A, ll sA, const double *B, ll sB,
                        double *C, ll sC, int batch) {
    dim3 grid((unsigned)((nn + 15) / 16), (unsigned)((m + 15) / 16), (unsigned)batch);
    k_dgemm_small<<<grid, dim3(16, 16), 0, st>>>((int)m, (int)nn, (int)k, ta ? 1 : 0, A, sA, B, sB, C, sC);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

// slab_cp[i] = i / n, slab_ap[i] = i % n for the n^2 slabs.
__global__ void k_slab_list(int n, int *cp, int *ap) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n * n) {
        cp[i] = i / n;
        ap[i] = i % n;
    }
}

// k_bamat_assemble for the single slab (cp, ap) whose four GEMM results sit
// at T1..T4 ([n^3 rows][n]).
__global__ void k_bamat_assemble_slab(int n, int M, int s, int cp, int ap, const double *T1, const double *T2,
                                      const double *T3, const double *T4, double *amat, double *atmat) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const ll n4 = (ll)n * n * n * n;
    if (t >= n4) return;
    ll x = t;
    const int bp = (int)(x % n); x /= n;
    const int a = (int)(x % n); x /= n;
    const int b = (int)(x % n); x /= n;
    const int c = (int)x;
    auto row3 = [n](int i, int j, int k) { return (((ll)i * n + j) * n + k) * n; };
    double t1 = T1[row3(bp, b, c) + a];
    double t2 = T2[row3(bp, b, a) + c];
    double t3 = T3[row3(bp, a, c) + b];
    double t4 = T4[row3(bp, a, c) + b];
    double u1 = T1[row3(b, bp, c) + a];
    double u2 = T2[row3(b, bp, a) + c];
    const ll o = s + (ll)M * (ap + (ll)n * (bp + (ll)n * (cp + (ll)n * (a + (ll)n * (b + (ll)n * c)))));
    amat[o] += t1 - t2 - t3;
    atmat[o] += -t4 - (u1 - u2);
}

double *bamat_static_scratch(int device) {
    // The array's address differs per device, so every call checks that the
    // context's device is the current one before it hands out an address
    // (the cached address of another device would be a wild pointer here).
    // The address is looked up once per device and cached.
    static std::atomic<double *> addr[64];
    if (device < 0 || device >= 64) return nullptr;
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != device) return nullptr;
    double *p = addr[device].load(std::memory_order_acquire);
    if (!p) {
        void *q = nullptr;
        if (cudaGetSymbolAddress(&q, g_bamat_scratch) != cudaSuccess) return nullptr;
        p = (double *)q;
        addr[device].store(p, std::memory_order_release);
    }
    return p;
}

int launch_bamat_static(const Rdm &r, const double *atwo, const double *f, int ncore, double *amat, double *atmat,
                        cudaStream_t st, double *scratch) {
    const int n = r.n, M = r.M;
    if (n > kBamatStaticNactMax) return 1;
    const ll n2 = (ll)n * n, n3 = n2 * n, n4 = n2 * n2, n6 = n4 * n2;
    for (int s = 0; s < M; ++s) {
        // lower-order terms (bamat_rest with the small GEMM kernel)
        double *E2 = scratch, *E2t = E2 + n6, *T = E2t + n6, *V = T + n6;
        double *EE2 = V + n6, *U = EE2 + n4, *D = U + n4, *G = D + n4, *H = G + n4, *Fs = H + n4;
        k_rest_dense<<<(unsigned)((n6 + 255) / 256), 256, 0, st>>>(r, s, E2, E2t, EE2);
        k_rest_ints<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(atwo, f, ncore, n, Fs, G, H);
        g_launches.fetch_add(2, std::memory_order_relaxed);
        dgemm_small(st, n2, n2, n2, true, G, 0, E2, n4, T, n4, (int)n2);
        dgemm_small(st, n2, n4, n2, true, H, 0, E2, 0, V, 0, 1);
        dgemm_small(st, n2, n2, n2, true, G, 0, EE2, 0, U, 0, 1);
        k_rest_delta<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(n, atwo, Fs, E2, EE2, U, D);
        k_rest_out<<<(unsigned)((n6 + 255) / 256), 256, 0, st>>>(n, M, s, Fs, E2, E2t, T, V, D, amat, atmat);
        g_launches.fetch_add(2, std::memory_order_relaxed);
        // n^9 part, one slab at a time (the same scratch, reused in stream order)
        double *A1 = scratch, *A2 = A1 + n4, *A3 = A2 + n4;
        double *T1 = A3 + n4, *T2 = T1 + n4, *T3 = T2 + n4, *T4 = T3 + n4;
        double *X1 = T4 + n4, *X2 = X1 + n6, *X3 = X2 + n6, *X4 = X3 + n6;
        int *cpl = (int *)(X4 + n6), *apl = cpl + n2;
        k_bamat_ints<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(atwo, n, A1, A2, A3);
        k_slab_list<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>(n, cpl, apl);
        g_launches.fetch_add(2, std::memory_order_relaxed);
        for (int sl = 0; sl < n2; ++sl) {
            k_bamat_slabs<<<(unsigned)((n6 + 255) / 256), 256, 0, st>>>(r, s, cpl + sl, apl + sl, 1, X1, X2, X3, X4);
            g_launches.fetch_add(1, std::memory_order_relaxed);
            dgemm_small(st, n3, n, n3, false, X1, 0, A1, 0, T1, 0, 1);
            dgemm_small(st, n3, n, n3, false, X2, 0, A2, 0, T2, 0, 1);
            dgemm_small(st, n3, n, n3, false, X3, 0, A3, 0, T3, 0, 1);
            dgemm_small(st, n3, n, n3, false, X4, 0, A3, 0, T4, 0, 1);
            k_bamat_assemble_slab<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(n, M, s, sl / n, sl % n, T1, T2, T3,
                                                                                T4, amat, atmat);
            g_launches.fetch_add(1, std::memory_order_relaxed);
        }
    }
    return 0;
}

}  // namespace nvpt
