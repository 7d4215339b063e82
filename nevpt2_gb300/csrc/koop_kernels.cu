// Stage-1 kernels: partial traces of the packed 4-RDM, active integrals and
// the generalised Koopmans matrices, FP64.
//
// One thread owns one output element and performs the reference's reduction
// for it in the reference's summation order, so no atomics are needed and
// results are deterministic.  The reference loop nests each kernel restates
// are cited on the kernel.  The n^9 A-matrix builder has its own file
// (bamat.cu); this file holds the n^5..n^7 work.
#include "nvpt2_internal.h"

#include <cublas_v2.h>

#include <algorithm>
#include <vector>

namespace nvpt {

#define ATWO(i, j, k, l) atwo[((i)-1) + (ll)n * (((j)-1) + (ll)n * (((k)-1) + (ll)n * ((l)-1)))]
#define FF(i, j) f[tri_index((i) + ncore, (j) + ncore) - 1]
#define AJ(i, j) aj[tri_index((i) + ncore, (j) + ncore) - 1]
#define O3(arr, s, a, b) arr[((s)-1) + (ll)M * (((a)-1) + (ll)n * ((b)-1))]
#define O5(arr, s, a, b, c, d) arr[((s)-1) + (ll)M * (((a)-1) + (ll)n * (((b)-1) + (ll)n * (((c)-1) + (ll)n * ((d)-1))))]

// Decode a flat 0-based index into `k` 1-based orbital indices, first fastest.
__device__ __forceinline__ void decode(ll x, int n, int k, int *out) {
    for (int i = 0; i < k; ++i) { out[i] = (int)(x % n) + 1; x /= n; }
}

// ---------------------------------------------------------------------------
// One-electron operator of each builder (src/koop_matrices.F90:191-200 and
// siblings): active upper triangle of f, mode 0: aj; 1: aj - 1/2 sum_c
// atwo(a,c,c,b); 2: aj - sum_c atwo(a,c,c,b).
__global__ void k_build_f(double *f, const double *aj, const double *atwo, int n, int ncore, int mode) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    int a = t % n + 1, b = t / n + 1;
    if (b < a) return;
    double v = AJ(a, b);
    if (mode != 0)
        for (int c = 1; c <= n; ++c) v -= (mode == 1 ? 0.5 : 1.0) * ATWO(a, c, c, b);
    FF(a, b) = v;
}

// ---------------------------------------------------------------------------
// src/koopro4QD.F90:4881-4959 bro3.
// bro3 as two passes over case-A terms.  Each term of the reference's sum,
// ro4[ord8(i,j,k,l; ii,jj,kk,l)], is read with the key taken from the group
// of larger normind (the first on ties).  Call a term "case A" for the output
// O = (i,j,k; ii,jj,kk) when that is the first group.  A term of O that is
// not case A is, entry for entry, a strict case-A term of the transposed
// output O^T = (ii,jj,kk; i,j,k): ord8 sees the same key group with the same
// partner.  So with
//   P[O] = sum of the case-A terms of O,  Q[O] = the strict (>) ones,
// daaa[O] = (P[O] + Q[O^T]) / (nele - 3).  In the first pass one CTA owns
// the column group (ii,jj,kk) and its threads the rows (i,j,k): every term's
// partner is a permutation of (ii,jj,kk,l), so a CTA reads at most 24 n
// columns of ro4, each W contiguous doubles, and the CTAs of the
// permutations of one multiset -- which read the same columns -- run side by
// side (blockIdx orders them together).  The second pass is a tiled
// transpose-add.  Summation order per element: the case-A terms in l order,
// then the others in l order (the reference adds all in l order).
constexpr int kBro3States = 8;  // states per pass of the first kernel
__global__ void __launch_bounds__(256) k_bro3_case_a(Rdm r, const int *col_order, int s0, int ns, double *P,
                                                     double *Q) {
    const int n = r.n, M = r.M;
    const ll n3 = (ll)n * n * n;
    const int c = col_order[blockIdx.x];
    const int ii = c % n + 1, jj = (c / n) % n + 1, kk = c / (n * n) + 1;
    __shared__ int s_n2[16];  // normind(ii,jj,kk,l) per l
    if (threadIdx.x < n) s_n2[threadIdx.x] = normind4(ii, jj, kk, threadIdx.x + 1);
    __syncthreads();
    for (ll rr = threadIdx.x; rr < n3; rr += blockDim.x) {
        const int i = (int)(rr % n) + 1, j = (int)((rr / n) % n) + 1, k = (int)(rr / ((ll)n * n)) + 1;
        double p[kBro3States], q[kBro3States];
#pragma unroll
        for (int t = 0; t < kBro3States; ++t) p[t] = q[t] = 0.0;
        for (int l = 1; l <= n; ++l) {
            // ord8 with the first group as key (case A): its selection sort,
            // the same swaps on the partner; lindice of the sorted key is
            // normind of the first group
            int kq[4] = {i, j, k, l}, pq[4] = {ii, jj, kk, l};
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                int imax = kq[a], jmax = a;
#pragma unroll
                for (int b = a + 1; b < 4; ++b)
                    if (kq[b] > imax) { imax = kq[b]; jmax = b; }
#pragma unroll
                for (int b = a + 1; b < 4; ++b)  // static indices: the arrays stay in registers
                    if (jmax == b) {
                        int t = kq[a]; kq[a] = kq[b]; kq[b] = t;
                        t = pq[a]; pq[a] = pq[b]; pq[b] = t;
                    }
            }
            const int n1 = lindice4(kq[0], kq[1], kq[2], kq[3]), n2 = s_n2[l - 1];
            if (n1 < n2) continue;
            const int ind = n1, q0 = pq[0], q1 = pq[1], q2 = pq[2], q3 = pq[3];
#pragma unroll
            for (int t = 0; t < kBro3States; ++t) {
                if (t >= ns) break;
                const double x = r.R4(ind, q0, q1, q2, q3, s0 + t + 1);
                p[t] += x;
                if (n1 > n2) q[t] += x;
            }
        }
        const ll o = (ll)M * (rr + n3 * c);
#pragma unroll
        for (int t = 0; t < kBro3States; ++t)
            if (t < ns) {
                P[o + s0 + t] = p[t];
                Q[o + s0 + t] = q[t];
            }
    }
}

// daaa[s, r, c] = (P[s, r, c] + Q[s, c, r]) * inv over the n^3 x n^3 matrix
// of each state (r = (i,j,k), c = (ii,jj,kk), r fastest), 32 x 32 tiles
// through shared memory so both reads and the write are coalesced.
__global__ void __launch_bounds__(256) k_bro3_combine(const double *P, const double *Q, double *daaa, ll n3, int M,
                                                      double inv) {
    __shared__ double t[32][33];
    const ll r0 = (ll)blockIdx.x * 32, c0 = (ll)blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int s = 0; s < M; ++s) {
        // Q tile at (row c0.., col r0..): element Q[s, c, r] with c fastest
        for (int y = ty; y < 32; y += 8) {
            const ll c = c0 + tx, rr = r0 + y;
            t[y][tx] = (c < n3 && rr < n3) ? Q[s + (ll)M * (c + n3 * rr)] : 0.0;
        }
        __syncthreads();
        for (int y = ty; y < 32; y += 8) {
            const ll rr = r0 + tx, c = c0 + y;
            if (rr < n3 && c < n3) {
                const ll o = s + (ll)M * (rr + n3 * c);
                daaa[o] = (P[o] + t[tx][y]) * inv;
            }
        }
        __syncthreads();
    }
}

// src/koopro4QD.F90:4961-5000 bro2
__global__ void k_bro2(Rdm r, double *taa, double inv) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    for (int s = 1; s <= M; ++s) {
        double acc = 0.0;
        for (int l = 1; l <= n; ++l) acc += r.D3(s, x[0], x[1], l, x[2], x[3], l);
        taa[(s - 1) + (ll)M * t] = acc * inv;
    }
}

// src/koopro4QD.F90:5002-5049 bro1
__global__ void k_bro1(Rdm r, double *dal, double inv) {
    const int n = r.n, M = r.M;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    int i = t % n + 1, j = t / n + 1;
    for (int s = 1; s <= M; ++s) {
        double acc = 0.0;
        for (int l = 1; l <= n; ++l) acc += r.D2(s, i, l, j, l);
        dal[(s - 1) + (ll)M * t] = acc * inv;
    }
}

// ---------------------------------------------------------------------------
// src/koopro4QD.F90:3900-3971 get_aj_atwo with the Cholesky integrals of
// src/ijkl_utils.F90:637-688: (ij|kl) = sum_Q L(Q,indice(i,j)) L(Q,indice(k,l)).
__device__ __forceinline__ double chol_ai(const double *L, int Q, int i, int j, int k, int l) {
    const double *x = L + (ll)Q * (tri_index(i, j) - 1);
    const double *y = L + (ll)Q * (tri_index(k, l) - 1);
    double s = 0.0;
    for (int q = 0; q < Q; ++q) s += x[q] * y[q];
    return s;
}

__global__ void k_atwo(const double *L, int Q, int n, int ncore, double *atwo) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    atwo[t] = chol_ai(L, Q, x[0] + ncore, x[1] + ncore, x[2] + ncore, x[3] + ncore);
}

// aj(active upper triangle) = oneint + sum_{j<=ncore} [2(ab|jj) - (aj|jb)]; the
// rest of aj is a copy of oneint (made by the caller).
__global__ void k_aj(const double *oneint, const double *L, int Q, int n, int ncore, double *aj) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    int a = t % n + 1, b = t / n + 1;
    if (b < a) return;
    int ac = a + ncore, bc = b + ncore;
    ll jab = tri_index(ac, bc) - 1;
    double v = oneint[jab];
    for (int j = 1; j <= ncore; ++j) v = v + 2.0 * chol_ai(L, Q, ac, bc, j, j) - chol_ai(L, Q, ac, j, j, bc);
    aj[jab] = v;
}

// ---------------------------------------------------------------------------
// src/koop_matrices.F90:165-250 koopE.  Thread per (ap, a).
__global__ void k_koopE(Rdm r, const double *atwo, const double *f, int ncore, double *koopipa, double *koopeaa) {
    const int n = r.n, M = r.M;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    int ap = t % n + 1, a = t / n + 1;
    for (int s = 1; s <= M; ++s) {
        double ip = 0.0;
        for (int c = 1; c <= n; ++c) {
            ip -= FF(a, c) * r.D1(s, ap, c);
            for (int d = 1; d <= n; ++d)
                for (int ie = 1; ie <= n; ++ie) ip -= ATWO(c, ie, a, d) * r.D2(s, ap, c, d, ie);
        }
        ip = 2.0 * ip;
        double dumm = 2.0 * FF(ap, a);
        for (int d = 1; d <= n; ++d)
            for (int ie = 1; ie <= n; ++ie) dumm += (2.0 * ATWO(d, ie, ap, a) - ATWO(ap, ie, d, a)) * r.D1(s, d, ie);
        O3(koopipa, s, ap, a) = ip;
        O3(koopeaa, s, ap, a) = ip + 2.0 * dumm;
    }
}

// src/koop_matrices.F90:78-88 (2-HRDM through ro2t)
__global__ void k_hrdm(Rdm r, double *hrdm) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    for (int s = 1; s <= M; ++s) hrdm[(s - 1) + (ll)M * t] = r.ro2t(x[0], x[1], x[2], x[3], s);
}

// src/koop_matrices.F90:297-335 koop2E, 2-IP part.  Thread per (ap,bp,a,b).
__global__ void k_koop2E_ip(Rdm r, const double *atwo, const double *f, int ncore, double *koopaa) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    const int ap = x[0], bp = x[1], a = x[2], b = x[3];
    for (int s = 1; s <= M; ++s) {
        double acc = 0.0;
        for (int d = 1; d <= n; ++d) {
            acc = acc - FF(a, d) * r.D2(s, ap, bp, d, b) - FF(b, d) * r.D2(s, ap, bp, a, d);
            for (int ie = 1; ie <= n; ++ie)
                for (int ief = 1; ief <= n; ++ief) {
                    double dint = ATWO(d, ie, a, ief), dint2 = ATWO(d, ie, b, ief);
                    double dum = r.D3(s, ap, bp, d, ief, b, ie);
                    if (d == ief) dum += 0.5 * r.D2(s, ap, bp, ie, b);
                    if (d == b) dum += 0.5 * r.D2(s, ap, bp, ief, ie);
                    acc -= dint * dum;
                    dum = r.D3(s, ap, bp, d, a, ief, ie);
                    if (d == a) dum += 0.5 * r.D2(s, ap, bp, ie, ief);
                    if (d == ief) dum += 0.5 * r.D2(s, ap, bp, a, ie);
                    acc -= dint2 * dum;
                }
        }
        O5(koopaa, s, ap, bp, a, b) = acc;
    }
}

// src/koop_matrices.F90:336-384 koop2E, 2-EA part.  Thread per (ap,bp,a,b).
__global__ void k_koop2E_ea(Rdm r, const double *atwo, const double *f, int ncore, double *koopeaa) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    const int ap = x[0], bp = x[1], a = x[2], b = x[3];
    for (int s = 1; s <= M; ++s) {
        double acc = 0.0;
        for (int c = 1; c <= n; ++c) {
            acc += FF(a, c) * r.ro2t(ap, bp, c, b, s) + FF(b, c) * r.ro2t(ap, bp, a, c, s);
            for (int d = 1; d <= n; ++d)
                for (int ie = 1; ie <= n; ++ie) {
                    double dint = ATWO(c, ie, d, a);
                    double dum = -r.ro3t(ap, bp, ie, d, b, c, s);
                    if (c == ie) dum += 2.0 * r.ro2t(ap, bp, d, b, s);
                    if (d == ie) dum -= 0.5 * r.ro2t(ap, bp, c, b, s);
                    if (b == ie) dum -= 0.5 * r.ro2t(ap, bp, d, c, s);
                    acc += dint * dum;
                    dint = ATWO(c, ie, d, b);
                    dum = -r.ro3t(ap, bp, ie, a, d, c, s);
                    if (c == ie) dum += 2.0 * r.ro2t(ap, bp, a, d, s);
                    if (a == ie) dum -= 0.5 * r.ro2t(ap, bp, c, d, s);
                    if (d == ie) dum -= 0.5 * r.ro2t(ap, bp, a, c, s);
                    acc += dint * dum;
                }
        }
        O5(koopeaa, s, ap, bp, a, b) = acc;
    }
}

// The same 2-EA matrix as products.  Per state, the bracketed operands of
// the reference's inner sum over (c, d, ie) are materialised as two n^3 x n^3
// row blocks,
//   G[(ap,bp,b), (c,d,ie)]       = -ro3t(ap,bp,ie,d,b,c) + 2[c=ie] ro2t(ap,bp,d,b)
//                                  - 1/2 [d=ie] ro2t(ap,bp,c,b) - 1/2 [b=ie] ro2t(ap,bp,d,c)
//   G[n^3 + (ap,bp,a), (c,d,ie)] = -ro3t(ap,bp,ie,a,d,c) + 2[c=ie] ro2t(ap,bp,a,d)
//                                  - 1/2 [a=ie] ro2t(ap,bp,c,d) - 1/2 [d=ie] ro2t(ap,bp,a,c)
// and one GEMM with A1[(c,d,ie), x] = atwo(c,ie,d,x) gives both contractions;
// k_koop2E_ea_out adds the one-electron terms.  Indices 0-based, last fastest.
__global__ void k_koop2E_ea_ops(Rdm r, int s, double *G) {
    const int n = r.n;
    const ll n3 = (ll)n * n * n, n6 = n3 * n3;
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * n6) return;
    const int half = (int)(t / n6);
    const ll x = t % n6, col = x % n3, row = x / n3;
    const int ie = (int)(col % n) + 1, d = (int)((col / n) % n) + 1, c = (int)(col / ((ll)n * n)) + 1;
    const int z = (int)(row % n) + 1, bp = (int)((row / n) % n) + 1, ap = (int)(row / ((ll)n * n)) + 1;
    double dum;
    if (half == 0) {
        const int b = z;
        dum = -r.ro3t(ap, bp, ie, d, b, c, s);
        if (c == ie) dum += 2.0 * r.ro2t(ap, bp, d, b, s);
        if (d == ie) dum -= 0.5 * r.ro2t(ap, bp, c, b, s);
        if (b == ie) dum -= 0.5 * r.ro2t(ap, bp, d, c, s);
    } else {
        const int a = z;
        dum = -r.ro3t(ap, bp, ie, a, d, c, s);
        if (c == ie) dum += 2.0 * r.ro2t(ap, bp, a, d, s);
        if (a == ie) dum -= 0.5 * r.ro2t(ap, bp, c, d, s);
        if (d == ie) dum -= 0.5 * r.ro2t(ap, bp, a, c, s);
    }
    G[t] = dum;
}
__global__ void k_koop2E_ea_ints(const double *atwo, int n, double *A1) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    const int x = (int)(t % n) + 1;
    const ll k = t / n;
    const int ie = (int)(k % n) + 1, d = (int)((k / n) % n) + 1, c = (int)(k / ((ll)n * n)) + 1;
    A1[t] = ATWO(c, ie, d, x);
}
__global__ void k_koop2E_ea_out(Rdm r, int s, const double *f, int ncore, const double *P, double *koopeaa) {
    const int n = r.n, M = r.M;
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const ll n4 = (ll)n * n * n * n;
    if (t >= n4) return;
    int x[4];
    decode(t, n, 4, x);
    const int ap = x[0], bp = x[1], a = x[2], b = x[3];
    double acc = 0.0;
    for (int c = 1; c <= n; ++c) acc += FF(a, c) * r.ro2t(ap, bp, c, b, s) + FF(b, c) * r.ro2t(ap, bp, a, c, s);
    const ll pre = ((ll)(ap - 1) * n + (bp - 1)) * n;
    acc += P[(pre + (b - 1)) * n + (a - 1)] + P[n4 + (pre + (a - 1)) * n + (b - 1)];
    O5(koopeaa, s, ap, bp, a, b) = acc;
}

// src/koop_matrices.F90:433-541 koopman0pE, A (koopaa) and D (koopbb) of the
// 0' class.  Thread per (bp,ap,a,b).
__global__ void k_koop0p_ad(Rdm r, const double *atwo, const double *f, int ncore, double *koopaa,
                            double *koopbb) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    const int bp = x[0], ap = x[1], a = x[2], b = x[3];
    for (int s = 1; s <= M; ++s) {
        double A = 0.0, Dm = 0.0;
        for (int c = 1; c <= n; ++c) {
            double fca = FF(c, a), fbc = FF(b, c);
            A += 2.0 * (fca * r.ee2(bp, ap, c, b, s) - fbc * r.ee2(bp, ap, a, c, s));
            for (int d = 1; d <= n; ++d)
                for (int ie = 1; ie <= n; ++ie) {
                    double dum1 = r.eee2(bp, ap, c, ie, d, b, s) + r.eee2(bp, ap, d, b, c, ie, s);
                    double dum2 = r.eee2(bp, ap, a, ie, c, d, s) + r.eee2(bp, ap, c, d, a, ie, s);
                    A += ATWO(c, ie, d, a) * dum1 - ATWO(b, ie, c, d) * dum2;
                }
        }
        for (int c = 1; c <= n; ++c) {
            double fca = FF(c, a), fbc = FF(b, c);
            double dum1 = -r.ee2(a, ap, bp, c, s);
            if (a == ap) dum1 += 2.0 * r.D1(s, bp, c);
            if (bp == ap) dum1 += r.D1(s, a, c);
            double dum2 = -r.ee2(c, ap, bp, b, s);
            if (ap == c) dum2 += 2.0 * r.D1(s, bp, b);
            if (bp == ap) dum2 += r.D1(s, c, b);
            Dm += -fbc * dum1 + fca * dum2;
            for (int d = 1; d <= n; ++d)
                for (int ie = 1; ie <= n; ++ie) {
                    double e1 = -r.eee2(c, ie, a, ap, bp, d, s) - r.eee2(a, ap, bp, d, c, ie, s);
                    if (ap == a) e1 += 2.0 * (r.ee2(c, ie, bp, d, s) + r.ee2(bp, d, c, ie, s));
                    if (bp == ap) e1 += r.ee2(c, ie, a, d, s) + r.ee2(a, d, c, ie, s);
                    if (ap == c) {
                        e1 -= r.ee2(a, ie, bp, d, s);
                        if (ie == a) e1 += 2.0 * r.D1(s, bp, d);
                    }
                    if (bp == ie) {
                        e1 += r.ee2(a, ap, c, d, s);
                        if (ap == a) e1 -= 2.0 * r.D1(s, c, d);
                    }
                    double e2 = -r.eee2(c, ie, d, ap, bp, b, s) - r.eee2(d, ap, bp, b, c, ie, s);
                    if (ap == d) e2 += 2.0 * (r.ee2(c, ie, bp, b, s) + r.ee2(bp, b, c, ie, s));
                    if (bp == ap) e2 += r.ee2(c, ie, d, b, s) + r.ee2(d, b, c, ie, s);
                    if (ap == c) {
                        e2 -= r.ee2(d, ie, bp, b, s);
                        if (d == ie) e2 += 2.0 * r.D1(s, bp, b);
                    }
                    if (bp == ie) {
                        e2 += r.ee2(d, ap, c, b, s);
                        if (d == ap) e2 -= 2.0 * r.D1(s, c, b);
                    }
                    Dm += -0.5 * ATWO(c, ie, b, d) * e1 + 0.5 * ATWO(c, ie, d, a) * e2;
                }
        }
        O5(koopaa, s, bp, ap, a, b) = A;
        O5(koopbb, s, bp, ap, a, b) = Dm;
    }
}

// The same A and D of the 0' class as products.  Per state, the operands of
// the reference's sums over (c, d, ie) are materialised as four n^3 x n^3
// blocks (rows (bp,ap,z), columns (c,d,ie), ie fastest):
//   0: eee2(bp,ap,c,ie,d,z) + eee2(bp,ap,d,z,c,ie)             (A, z = b) x atwo(c,ie,d,a)
//   1: the D operand of the atwo(c,ie,d,a) term               (D, z = b) x atwo(c,ie,d,a)
//   2: eee2(bp,ap,z,ie,c,d) + eee2(bp,ap,c,d,z,ie)             (A, z = a) x atwo(b,ie,c,d)
//   3: the D operand of the atwo(c,ie,b,d) term               (D, z = a) x atwo(c,ie,b,d)
// and three GEMMs give the n^7 sums; k_koop0p_out adds the n^5 one-electron
// terms, with the signs and halves of the reference.
__device__ __forceinline__ double koop0p_e1(const Rdm &r, int c, int d, int ie, int bp, int ap, int a, int s) {
    double e1 = -r.eee2(c, ie, a, ap, bp, d, s) - r.eee2(a, ap, bp, d, c, ie, s);
    if (ap == a) e1 += 2.0 * (r.ee2(c, ie, bp, d, s) + r.ee2(bp, d, c, ie, s));
    if (bp == ap) e1 += r.ee2(c, ie, a, d, s) + r.ee2(a, d, c, ie, s);
    if (ap == c) {
        e1 -= r.ee2(a, ie, bp, d, s);
        if (ie == a) e1 += 2.0 * r.D1(s, bp, d);
    }
    if (bp == ie) {
        e1 += r.ee2(a, ap, c, d, s);
        if (ap == a) e1 -= 2.0 * r.D1(s, c, d);
    }
    return e1;
}
__device__ __forceinline__ double koop0p_e2(const Rdm &r, int c, int d, int ie, int bp, int ap, int b, int s) {
    double e2 = -r.eee2(c, ie, d, ap, bp, b, s) - r.eee2(d, ap, bp, b, c, ie, s);
    if (ap == d) e2 += 2.0 * (r.ee2(c, ie, bp, b, s) + r.ee2(bp, b, c, ie, s));
    if (bp == ap) e2 += r.ee2(c, ie, d, b, s) + r.ee2(d, b, c, ie, s);
    if (ap == c) {
        e2 -= r.ee2(d, ie, bp, b, s);
        if (d == ie) e2 += 2.0 * r.D1(s, bp, b);
    }
    if (bp == ie) {
        e2 += r.ee2(d, ap, c, b, s);
        if (d == ap) e2 -= 2.0 * r.D1(s, c, b);
    }
    return e2;
}
__global__ void k_koop0p_ops(Rdm r, int s, double *G) {
    const int n = r.n;
    const ll n3 = (ll)n * n * n, n6 = n3 * n3;
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 4 * n6) return;
    const int blk = (int)(t / n6);
    const ll x = t % n6, col = x % n3, row = x / n3;
    const int ie = (int)(col % n) + 1, d = (int)((col / n) % n) + 1, c = (int)(col / ((ll)n * n)) + 1;
    const int z = (int)(row % n) + 1, ap = (int)((row / n) % n) + 1, bp = (int)(row / ((ll)n * n)) + 1;
    double v;
    if (blk == 0) v = r.eee2(bp, ap, c, ie, d, z, s) + r.eee2(bp, ap, d, z, c, ie, s);
    else if (blk == 1) v = koop0p_e2(r, c, d, ie, bp, ap, z, s);
    else if (blk == 2) v = r.eee2(bp, ap, z, ie, c, d, s) + r.eee2(bp, ap, c, d, z, ie, s);
    else v = koop0p_e1(r, c, d, ie, bp, ap, z, s);
    G[t] = v;
}
// A2[(c,d,ie), x] = atwo(x,ie,c,d), A3[(c,d,ie), x] = atwo(c,ie,x,d)
__global__ void k_koop0p_ints(const double *atwo, int n, double *A2, double *A3) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    const int x = (int)(t % n) + 1;
    const ll k = t / n;
    const int ie = (int)(k % n) + 1, d = (int)((k / n) % n) + 1, c = (int)(k / ((ll)n * n)) + 1;
    A2[t] = ATWO(x, ie, c, d);
    A3[t] = ATWO(c, ie, x, d);
}
__global__ void k_koop0p_out(Rdm r, int s, const double *f, int ncore, const double *P01, const double *P2,
                             const double *P3, double *koopaa, double *koopbb) {
    const int n = r.n, M = r.M;
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const ll n3 = (ll)n * n * n, n4 = n3 * n;
    if (t >= n4) return;
    int x[4];
    decode(t, n, 4, x);
    const int bp = x[0], ap = x[1], a = x[2], b = x[3];
    double A = 0.0, Dm = 0.0;
    for (int c = 1; c <= n; ++c) {
        const double fca = FF(c, a), fbc = FF(b, c);
        A += 2.0 * (fca * r.ee2(bp, ap, c, b, s) - fbc * r.ee2(bp, ap, a, c, s));
    }
    for (int c = 1; c <= n; ++c) {
        const double fca = FF(c, a), fbc = FF(b, c);
        double dum1 = -r.ee2(a, ap, bp, c, s);
        if (a == ap) dum1 += 2.0 * r.D1(s, bp, c);
        if (bp == ap) dum1 += r.D1(s, a, c);
        double dum2 = -r.ee2(c, ap, bp, b, s);
        if (ap == c) dum2 += 2.0 * r.D1(s, bp, b);
        if (bp == ap) dum2 += r.D1(s, c, b);
        Dm += -fbc * dum1 + fca * dum2;
    }
    const ll rb = ((ll)(bp - 1) * n + (ap - 1)) * n + (b - 1), ra = ((ll)(bp - 1) * n + (ap - 1)) * n + (a - 1);
    A += P01[rb * n + (a - 1)] - P2[ra * n + (b - 1)];
    Dm += -0.5 * P3[ra * n + (b - 1)] + 0.5 * P01[(n3 + rb) * n + (a - 1)];
    O5(koopaa, s, bp, ap, a, b) = A;
    O5(koopbb, s, bp, ap, a, b) = Dm;
}

// src/koop_matrices.F90:546-571 koopman0pE, F (koopab).  Thread per (a,b).
__global__ void k_koop0p_f(Rdm r, const double *atwo, const double *f, int ncore, double *koopab) {
    const int n = r.n, M = r.M;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    int a = t % n + 1, b = t / n + 1;
    for (int s = 1; s <= M; ++s) {
        double acc = 0.0;
        for (int c = 1; c <= n; ++c) {
            acc += 2.0 * (FF(c, a) * r.D1(s, c, b) - FF(b, c) * r.D1(s, a, c));
            for (int d = 1; d <= n; ++d)
                for (int ie = 1; ie <= n; ++ie) {
                    double dum1 = r.ee2(c, ie, d, b, s) + r.ee2(d, b, c, ie, s);
                    double dum2 = r.ee2(a, ie, c, d, s) + r.ee2(c, d, a, ie, s);
                    acc += ATWO(c, ie, d, a) * dum1 - ATWO(b, ie, c, d) * dum2;
                }
        }
        O3(koopab, s, a, b) = acc;
    }
}

// ---------------------------------------------------------------------------
// src/koopro4QD.F90:4231-4299 bbmat.  Thread per (ap,bp,cp,a).  The EA part
// multiplies by aj, not by the modified f (reference quirk kept).
__global__ void k_bbmat(Rdm r, const double *atwo, const double *f, const double *aj, int ncore, double *bmat,
                        double *btmat) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    const int ap = x[0], bp = x[1], cp = x[2], a = x[3];
    for (int s = 1; s <= M; ++s) {
        double B = 0.0, Bt = 0.0;
        for (int c = 1; c <= n; ++c) {
            B -= FF(c, a) * r.ee2(cp, ap, bp, c, s);
            Bt += AJ(c, a) * r.ee2tr(cp, ap, bp, c, s);
            for (int ie = 1; ie <= n; ++ie)
                for (int ief = 1; ief <= n; ++ief) {
                    double dint = ATWO(a, ie, c, ief);
                    B -= r.eee2(cp, ap, bp, ie, c, ief, s) * dint;
                    Bt += r.eee2t(cp, ap, bp, ie, c, ief, s) * dint;
                }
        }
        O5(bmat, s, ap, bp, cp, a) = B;
        O5(btmat, s, ap, bp, cp, a) = Bt;
    }
}

// src/koopro4QD.F90:4301-4397 bcmat.  Thread per (ap,a,b,c); the reference's
// d loop is the reduction.
__global__ void k_bcmat(Rdm r, const double *atwo, const double *f, int ncore, double *cmat, double *ctmat) {
    const int n = r.n, M = r.M;
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    int x[4];
    decode(t, n, 4, x);
    const int ap = x[0], a = x[1], b = x[2], c = x[3];
    for (int s = 1; s <= M; ++s) {
        double C = 0.0, Ct = 0.0;
        for (int d = 1; d <= n; ++d) {
            double fda = FF(d, a), fcd = FF(c, d), fbd = FF(b, d);
            C += fda * r.ee2(ap, b, d, c, s) - fcd * r.ee2(ap, b, a, d, s) - fbd * r.ee2(ap, d, a, c, s);
            Ct += fda * r.ee2t(ap, b, d, c, s) - fcd * r.ee2t(ap, b, a, d, s) + fbd * r.ee2t(ap, d, a, c, s);
            for (int ie = 1; ie <= n; ++ie) {
                double dint1 = ATWO(c, ie, d, a), dint2 = ATWO(d, ie, ie, a);
                double dint3 = ATWO(c, d, d, ie), dint4 = ATWO(b, d, d, ie);
                C += r.ee2(ap, b, d, ie, s) * dint1 -
                     0.5 * (r.ee2(ap, b, d, c, s) * dint2 + r.ee2(ap, b, a, ie, s) * dint3 - r.ee2(ap, ie, a, c, s) * dint4);
                Ct += r.ee2t(ap, b, d, ie, s) * dint1 -
                      0.5 * (r.ee2t(ap, b, d, c, s) * dint2 + r.ee2t(ap, b, a, ie, s) * dint3 -
                             r.ee2t(ap, ie, a, c, s) * dint4);
                for (int ief = 1; ief <= n; ++ief) {
                    double di1 = ATWO(d, ief, ie, a), di2 = ATWO(d, ief, c, ie), di3 = ATWO(d, ief, b, ie);
                    C += r.eee2(ap, b, d, ief, ie, c, s) * di1 - r.eee2(ap, b, d, ief, a, ie, s) * di2 -
                         r.eee2(ap, ie, d, ief, a, c, s) * di3;
                    Ct += r.eee2tl(ap, b, d, ief, ie, c, s) * di1 - r.eee2tl(ap, b, d, ief, a, ie, s) * di2 +
                          r.eee2tl(ap, ie, d, ief, a, c, s) * di3;
                }
            }
        }
        O5(cmat, s, ap, a, b, c) = C;
        O5(ctmat, s, ap, a, b, c) = Ct;
    }
}

// The same C / C~ matrices as products.  Per state, the operands of the n^7
// sums over (d, ief, ie) are materialised as six n^3 x n^3 blocks (rows
// (ap,u,w), columns (d,ief,ie), ie fastest), eee2 for C and eee2tl for C~:
//   0/1: e(ap,u,d,ief,ie,w), u = b, w = c     x atwo(d,ief,ie,a)
//   2/3: e(ap,u,d,ief,w,ie), u = b, w = a     x atwo(d,ief,c,ie)
//   4/5: e(ap,ie,d,ief,u,w), u = a, w = c     x atwo(d,ief,b,ie)
// three GEMMs (the C and C~ blocks stacked) give them; k_bcmat_out adds the
// one-electron and n^6 terms in the reference's form.
__global__ void k_bcmat_ops(Rdm r, int s, double *G) {
    const int n = r.n;
    const ll n3 = (ll)n * n * n, n6 = n3 * n3;
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 6 * n6) return;
    const int blk = (int)(t / n6);
    const ll x = t % n6, col = x % n3, row = x / n3;
    const int ie = (int)(col % n) + 1, ief = (int)((col / n) % n) + 1, d = (int)(col / ((ll)n * n)) + 1;
    const int w = (int)(row % n) + 1, u = (int)((row / n) % n) + 1, ap = (int)(row / ((ll)n * n)) + 1;
    double v;
    switch (blk) {
    case 0: v = r.eee2(ap, u, d, ief, ie, w, s); break;
    case 1: v = r.eee2tl(ap, u, d, ief, ie, w, s); break;
    case 2: v = r.eee2(ap, u, d, ief, w, ie, s); break;
    case 3: v = r.eee2tl(ap, u, d, ief, w, ie, s); break;
    case 4: v = r.eee2(ap, ie, d, ief, u, w, s); break;
    default: v = r.eee2tl(ap, ie, d, ief, u, w, s); break;
    }
    G[t] = v;
}
// B1[(d,ief,ie), x] = atwo(d,ief,ie,x), B2[(d,ief,ie), x] = atwo(d,ief,x,ie)
__global__ void k_bcmat_ints(const double *atwo, int n, double *B1, double *B2) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    const int x = (int)(t % n) + 1;
    const ll k = t / n;
    const int ie = (int)(k % n) + 1, ief = (int)((k / n) % n) + 1, d = (int)(k / ((ll)n * n)) + 1;
    B1[t] = ATWO(d, ief, ie, x);
    B2[t] = ATWO(d, ief, x, ie);
}
__global__ void k_bcmat_out(Rdm r, int s, const double *atwo, const double *f, int ncore, const double *P,
                            double *cmat, double *ctmat) {
    const int n = r.n, M = r.M;
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const ll n3 = (ll)n * n * n, n4 = n3 * n;
    if (t >= n4) return;
    int x[4];
    decode(t, n, 4, x);
    const int ap = x[0], a = x[1], b = x[2], c = x[3];
    double C = 0.0, Ct = 0.0;
    for (int d = 1; d <= n; ++d) {
        const double fda = FF(d, a), fcd = FF(c, d), fbd = FF(b, d);
        C += fda * r.ee2(ap, b, d, c, s) - fcd * r.ee2(ap, b, a, d, s) - fbd * r.ee2(ap, d, a, c, s);
        Ct += fda * r.ee2t(ap, b, d, c, s) - fcd * r.ee2t(ap, b, a, d, s) + fbd * r.ee2t(ap, d, a, c, s);
        for (int ie = 1; ie <= n; ++ie) {
            const double dint1 = ATWO(c, ie, d, a), dint2 = ATWO(d, ie, ie, a);
            const double dint3 = ATWO(c, d, d, ie), dint4 = ATWO(b, d, d, ie);
            C += r.ee2(ap, b, d, ie, s) * dint1 -
                 0.5 * (r.ee2(ap, b, d, c, s) * dint2 + r.ee2(ap, b, a, ie, s) * dint3 - r.ee2(ap, ie, a, c, s) * dint4);
            Ct += r.ee2t(ap, b, d, ie, s) * dint1 -
                  0.5 * (r.ee2t(ap, b, d, c, s) * dint2 + r.ee2t(ap, b, a, ie, s) * dint3 -
                         r.ee2t(ap, ie, a, c, s) * dint4);
        }
    }
    // P: [3 GEMMs][2 n^3 rows (C block, C~ block)][n]
    const ll rbc = ((ll)(ap - 1) * n + (b - 1)) * n + (c - 1), rba = ((ll)(ap - 1) * n + (b - 1)) * n + (a - 1);
    const ll rac = ((ll)(ap - 1) * n + (a - 1)) * n + (c - 1);
    const double *P1 = P, *P2 = P + 2 * n4, *P3 = P + 4 * n4;
    C += P1[rbc * n + (a - 1)] - P2[rba * n + (c - 1)] - P3[rac * n + (b - 1)];
    Ct += P1[(n3 + rbc) * n + (a - 1)] - P2[(n3 + rba) * n + (c - 1)] + P3[(n3 + rac) * n + (b - 1)];
    O5(cmat, s, ap, a, b, c) = C;
    O5(ctmat, s, ap, a, b, c) = Ct;
}

// src/koopro4QD.F90:4399-4459 bdmat.  Thread per (ap,a); EA part uses aj.
__global__ void k_bdmat(Rdm r, const double *atwo, const double *f, const double *aj, int ncore, double *dmat,
                        double *dtmat) {
    const int n = r.n, M = r.M;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    int ap = t % n + 1, a = t / n + 1;
    for (int s = 1; s <= M; ++s) {
        double D = 0.0, Dt = 0.0;
        for (int c = 1; c <= n; ++c) {
            D -= FF(c, a) * r.D1(s, ap, c);
            double dum = -r.D1(s, ap, c);
            if (ap == c) dum += 2.0;
            Dt += AJ(c, a) * dum;
            for (int ie = 1; ie <= n; ++ie)
                for (int ief = 1; ief <= n; ++ief) {
                    double dint = ATWO(a, ie, c, ief);
                    D -= r.ee2(ap, ie, c, ief, s) * dint;
                    Dt += r.ee2t(ap, ie, c, ief, s) * dint;
                }
        }
        O3(dmat, s, ap, a) = D;
        O3(dtmat, s, ap, a) = Dt;
    }
}

// ---------------------------------------------------------------------------
// Host launchers.
static inline unsigned blocks_for(ll work, int tpb) { return (unsigned)((work + tpb - 1) / tpb); }

void launch_build_f(double *f, const double *aj, const double *atwo, int n, int ncore, int mode, cudaStream_t st) {
    k_build_f<<<blocks_for((ll)n * n, 128), 128, 0, st>>>(f, aj, atwo, n, ncore, mode);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

// Column groups in an order that puts the permutations of one multiset
// {ii,jj,kk} next to each other (they read the same ro4 columns).
static void bro3_column_order(int n, std::vector<int> &ord) {
    ord.clear();
    for (int a = 0; a < n; ++a)
        for (int b = a; b < n; ++b)
            for (int c = b; c < n; ++c) {
                const int v[3] = {a, b, c};
                static const int P[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
                int seen[6], ns = 0;
                for (auto &pp : P) {
                    const int code = v[pp[0]] + n * (v[pp[1]] + n * v[pp[2]]);
                    bool dup = false;
                    for (int q = 0; q < ns; ++q) dup |= seen[q] == code;
                    if (!dup) {
                        seen[ns++] = code;
                        ord.push_back(code);
                    }
                }
            }
}

int launch_bro3(const Rdm &r, double *daaa, int nele, cudaStream_t st) {
    const int n = r.n, M = r.M;
    const ll n3 = (ll)n * n * n, n6 = n3 * n3;
    std::vector<int> ord;
    bro3_column_order(n, ord);
    double *P = nullptr;
    int *d_ord = nullptr;
    if (cudaMallocAsync((void **)&P, sizeof(double) * 2 * (size_t)(M * n6), st) != cudaSuccess) return 2;
    if (cudaMallocAsync((void **)&d_ord, sizeof(int) * ord.size(), st) != cudaSuccess) {
        cudaFreeAsync(P, st);
        return 2;
    }
    double *Q = P + (size_t)M * n6;
    cudaMemcpyAsync(d_ord, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice, st);
    ProfSpan span;
    span.begin("bro3", st, 0);
    for (int s0 = 0; s0 < M; s0 += kBro3States) {
        k_bro3_case_a<<<(unsigned)n3, 256, 0, st>>>(r, d_ord, s0, std::min(kBro3States, M - s0), P, Q);
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    dim3 g((unsigned)((n3 + 31) / 32), (unsigned)((n3 + 31) / 32));
    k_bro3_combine<<<g, 256, 0, st>>>(P, Q, daaa, n3, M, 1.0 / (double)(nele - 3));
    span.end();
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaFreeAsync(d_ord, st);
    cudaFreeAsync(P, st);
    return 0;
}
void launch_bro2(const Rdm &r, double *taa, int nele, cudaStream_t st) {
    ll n4 = (ll)r.n * r.n * r.n * r.n;
    k_bro2<<<blocks_for(n4, 256), 256, 0, st>>>(r, taa, 1.0 / (double)(nele - 2));
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void launch_bro1(const Rdm &r, double *dal, int nele, cudaStream_t st) {
    k_bro1<<<blocks_for((ll)r.n * r.n, 128), 128, 0, st>>>(r, dal, 1.0 / (double)(nele - 1));
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

void launch_aj_atwo(const double *oneint, const double *L, int Q, int n, int ncore, int norb, double *atwo,
                    double *aj, cudaStream_t st) {
    cudaMemcpyAsync(aj, oneint, sizeof(double) * (size_t)norb * (norb + 1) / 2, cudaMemcpyDeviceToDevice, st);
    k_aj<<<blocks_for((ll)n * n, 64), 64, 0, st>>>(oneint, L, Q, n, ncore, aj);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ll n4 = (ll)n * n * n * n;
    k_atwo<<<blocks_for(n4, 128), 128, 0, st>>>(L, Q, n, ncore, atwo);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

void launch_koopE(const Rdm &r, const double *atwo, const double *f, int ncore, double *ip, double *ea,
                  cudaStream_t st) {
    k_koopE<<<blocks_for((ll)r.n * r.n, 64), 64, 0, st>>>(r, atwo, f, ncore, ip, ea);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void launch_hrdm(const Rdm &r, double *hrdm, cudaStream_t st) {
    ll n4 = (ll)r.n * r.n * r.n * r.n;
    k_hrdm<<<blocks_for(n4, 256), 256, 0, st>>>(r, hrdm);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
namespace {
struct KoopBlas {
    cublasHandle_t h = nullptr;
    ~KoopBlas() {
        if (h) cublasDestroy(h);
    }
};
}  // namespace

void launch_koop2E(const Rdm &r, const double *atwo, const double *f, int ncore, double *ip2, double *ea2,
                   cudaStream_t st) {
    const int n = r.n;
    const ll n3 = (ll)n * n * n, n4 = n3 * n, n6 = n3 * n3;
    k_koop2E_ip<<<blocks_for(n4, 64), 64, 0, st>>>(r, atwo, f, ncore, ip2);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    // 2-EA: operand blocks + one GEMM per state
    static thread_local KoopBlas blas;
    double *G = nullptr, *A1 = nullptr, *P = nullptr;
    bool ok = (blas.h || cublasCreate(&blas.h) == CUBLAS_STATUS_SUCCESS) &&
              cublasSetStream(blas.h, st) == CUBLAS_STATUS_SUCCESS &&
              cudaMallocAsync((void **)&G, sizeof(double) * 2 * (size_t)n6, st) == cudaSuccess &&
              cudaMallocAsync((void **)&A1, sizeof(double) * (size_t)n4, st) == cudaSuccess &&
              cudaMallocAsync((void **)&P, sizeof(double) * 2 * (size_t)n4, st) == cudaSuccess;
    if (!ok) {  // no room for the operand blocks: the per-element kernel
        if (G) cudaFreeAsync(G, st);
        if (A1) cudaFreeAsync(A1, st);
        k_koop2E_ea<<<blocks_for(n4, 64), 64, 0, st>>>(r, atwo, f, ncore, ea2);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return;
    }
    k_koop2E_ea_ints<<<blocks_for(n4, 256), 256, 0, st>>>(atwo, n, A1);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const double one = 1.0, zero = 0.0;
    for (int s = 1; s <= r.M; ++s) {
        k_koop2E_ea_ops<<<blocks_for(2 * n6, 256), 256, 0, st>>>(r, s, G);
        // row-major P[2 n^3, n] = G[2 n^3, n^3] A1[n^3, n]
        cublasDgemm(blas.h, CUBLAS_OP_N, CUBLAS_OP_N, n, (int)(2 * n3), (int)n3, &one, A1, n, G, (int)n3, &zero, P, n);
        k_koop2E_ea_out<<<blocks_for(n4, 256), 256, 0, st>>>(r, s, f, ncore, P, ea2);
        g_launches.fetch_add(2, std::memory_order_relaxed);
    }
    cudaFreeAsync(G, st);
    cudaFreeAsync(A1, st);
    cudaFreeAsync(P, st);
}
void launch_koop0p(const Rdm &r, const double *atwo, const double *f, int ncore, double *gk0pa, double *gk0pd,
                   double *gk0pf, cudaStream_t st) {
    const int n = r.n;
    const ll n3 = (ll)n * n * n, n4 = n3 * n, n6 = n3 * n3;
    static thread_local KoopBlas blas;
    double *G = nullptr, *Ai = nullptr, *P = nullptr;
    const bool ok = (blas.h || cublasCreate(&blas.h) == CUBLAS_STATUS_SUCCESS) &&
                    cublasSetStream(blas.h, st) == CUBLAS_STATUS_SUCCESS &&
                    cudaMallocAsync((void **)&G, sizeof(double) * 4 * (size_t)n6, st) == cudaSuccess &&
                    cudaMallocAsync((void **)&Ai, sizeof(double) * 3 * (size_t)n4, st) == cudaSuccess &&
                    cudaMallocAsync((void **)&P, sizeof(double) * 4 * (size_t)n4, st) == cudaSuccess;
    if (ok) {
        double *A1 = Ai, *A2 = Ai + n4, *A3 = Ai + 2 * n4;
        k_koop2E_ea_ints<<<blocks_for(n4, 256), 256, 0, st>>>(atwo, n, A1);
        k_koop0p_ints<<<blocks_for(n4, 256), 256, 0, st>>>(atwo, n, A2, A3);
        g_launches.fetch_add(2, std::memory_order_relaxed);
        const double one = 1.0, zero = 0.0;
        for (int s = 1; s <= r.M; ++s) {
            k_koop0p_ops<<<blocks_for(4 * n6, 256), 256, 0, st>>>(r, s, G);
            // row-major P01[2 n^3, n] = G[0:2 n^3] A1; P2 = G[2 n^3:3 n^3] A2; P3 = G[3 n^3:] A3
            cublasDgemm(blas.h, CUBLAS_OP_N, CUBLAS_OP_N, n, (int)(2 * n3), (int)n3, &one, A1, n, G, (int)n3, &zero,
                        P, n);
            cublasDgemm(blas.h, CUBLAS_OP_N, CUBLAS_OP_N, n, (int)n3, (int)n3, &one, A2, n, G + 2 * n6, (int)n3, &zero,
                        P + 2 * n4, n);
            cublasDgemm(blas.h, CUBLAS_OP_N, CUBLAS_OP_N, n, (int)n3, (int)n3, &one, A3, n, G + 3 * n6, (int)n3, &zero,
                        P + 3 * n4, n);
            k_koop0p_out<<<blocks_for(n4, 256), 256, 0, st>>>(r, s, f, ncore, P, P + 2 * n4, P + 3 * n4, gk0pa, gk0pd);
            g_launches.fetch_add(2, std::memory_order_relaxed);
        }
        cudaFreeAsync(G, st);
        cudaFreeAsync(Ai, st);
        cudaFreeAsync(P, st);
    } else {  // no room for the operand blocks: the per-element kernel
        if (G) cudaFreeAsync(G, st);
        if (Ai) cudaFreeAsync(Ai, st);
        k_koop0p_ad<<<blocks_for(n4, 64), 64, 0, st>>>(r, atwo, f, ncore, gk0pa, gk0pd);
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    k_koop0p_f<<<blocks_for((ll)r.n * r.n, 64), 64, 0, st>>>(r, atwo, f, ncore, gk0pf);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void launch_bbmat(const Rdm &r, const double *atwo, const double *f, const double *aj, int ncore, double *b,
                  double *bt, cudaStream_t st) {
    ll n4 = (ll)r.n * r.n * r.n * r.n;
    k_bbmat<<<blocks_for(n4, 64), 64, 0, st>>>(r, atwo, f, aj, ncore, b, bt);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
void launch_bcmat(const Rdm &r, const double *atwo, const double *f, int ncore, double *c, double *ct,
                  cudaStream_t st) {
    const int n = r.n;
    const ll n3 = (ll)n * n * n, n4 = n3 * n, n6 = n3 * n3;
    static thread_local KoopBlas blas;
    double *G = nullptr, *Bi = nullptr, *P = nullptr;
    const bool ok = (blas.h || cublasCreate(&blas.h) == CUBLAS_STATUS_SUCCESS) &&
                    cublasSetStream(blas.h, st) == CUBLAS_STATUS_SUCCESS &&
                    cudaMallocAsync((void **)&G, sizeof(double) * 6 * (size_t)n6, st) == cudaSuccess &&
                    cudaMallocAsync((void **)&Bi, sizeof(double) * 2 * (size_t)n4, st) == cudaSuccess &&
                    cudaMallocAsync((void **)&P, sizeof(double) * 6 * (size_t)n4, st) == cudaSuccess;
    if (!ok) {  // no room for the operand blocks: the per-element kernel
        if (G) cudaFreeAsync(G, st);
        if (Bi) cudaFreeAsync(Bi, st);
        k_bcmat<<<blocks_for(n4, 64), 64, 0, st>>>(r, atwo, f, ncore, c, ct);
        g_launches.fetch_add(1, std::memory_order_relaxed);
        return;
    }
    double *B1 = Bi, *B2 = Bi + n4;
    k_bcmat_ints<<<blocks_for(n4, 256), 256, 0, st>>>(atwo, n, B1, B2);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const double one = 1.0, zero = 0.0;
    const double *Bs[3] = {B1, B2, B2};
    for (int s = 1; s <= r.M; ++s) {
        k_bcmat_ops<<<blocks_for(6 * n6, 256), 256, 0, st>>>(r, s, G);
        for (int g = 0; g < 3; ++g)  // row-major P_g[2 n^3, n] = G[blocks 2g, 2g+1] B_g
            cublasDgemm(blas.h, CUBLAS_OP_N, CUBLAS_OP_N, n, (int)(2 * n3), (int)n3, &one, Bs[g], n, G + 2 * g * n6,
                        (int)n3, &zero, P + 2 * g * n4, n);
        k_bcmat_out<<<blocks_for(n4, 256), 256, 0, st>>>(r, s, atwo, f, ncore, P, c, ct);
        g_launches.fetch_add(2, std::memory_order_relaxed);
    }
    cudaFreeAsync(G, st);
    cudaFreeAsync(Bi, st);
    cudaFreeAsync(P, st);
}
void launch_bdmat(const Rdm &r, const double *atwo, const double *f, const double *aj, int ncore, double *d,
                  double *dt, cudaStream_t st) {
    k_bdmat<<<blocks_for((ll)r.n * r.n, 64), 64, 0, st>>>(r, atwo, f, aj, ncore, d, dt);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

}  // namespace nvpt
