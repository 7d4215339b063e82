// NEVPT2 energy stage on the device: src/qdnevpt.F:369-993 (Cholesky
// integrals, C1) for every state, with the QD off-diagonal terms.
//
// Per state:  core / virtual Fock operators -> cuSOLVER eigensolve (epsnew,
// ccore, cvirt) -> half-transformed DF blocks (cholesky_transform :7599) ->
// the eight perturber classes.  Every strongly contracted (SC) class sum is a
// set of bilinear forms  v_L^T X v_L  over external labels L (GEMM + row
// dot), finished by one kernel that applies the reference's denominator and
// threshold rules; every partially contracted (PC) class runs the metric
// pseudo-inverse sequence (syevd, drop eigenvalues < thr, X = U w^-1/2,
// K~ = X^T K X, syevd, C = X V; caux0p :4744) and then its energy sums as
// GEMMs over (label, mu) with a finishing kernel -- except the order-n^3
// metrics of the (+-1') classes when every metric eigenvalue is kept: there
// the sums over the eigenpairs are resolvents of the pencil K v = w S v,
// evaluated in its tridiagonal form without eigenvectors.  Energies
// accumulate in FP64 on the device.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <exception>
#include <vector>

#include "../../include/nvpt2.h"
#include "s2_tensor.cuh"

extern "C" unsigned nvpt_context_wait_limit(const nvpt_context *ctx);
extern "C" int nvpt_context_pc_route(const nvpt_context *ctx);

namespace nvpt {
namespace s2 {
namespace {

constexpr int TPB = 256;
inline unsigned nblk(long long n) { return (unsigned)((n + TPB - 1) / TPB); }
#define LAUNCHED() g_launches.fetch_add(1, std::memory_order_relaxed)

// ---------------------------------------------------------------- kernels
__global__ void k_unpack_B(const double *chol, long long Q, int norb, double *B) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long nn = (long long)norb * norb;
    if (t >= Q * nn) return;
    long long x = t / nn, pq = t % nn;
    int p = (int)(pq / norb), q = (int)(pq % norb);
    int mx = p > q ? p : q, mn = p > q ? q : p;
    long long tri = (long long)(mx + 1) * mx / 2 + mn;
    B[t] = chol[x + Q * tri];
}

__global__ void k_unpack_tri(const double *v, int norb, double *h) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)norb * norb) return;
    int p = (int)(t / norb), q = (int)(t % norb);
    int mx = p > q ? p : q, mn = p > q ? q : p;
    h[t] = v[(long long)(mx + 1) * mx / 2 + mn];
}

// diag sums: out[x] = sum_k B[x, o+k, o+k]
__global__ void k_diag_sum(const double *B, long long Q, int norb, int o, int cnt, double *out) {
    long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= Q) return;
    double s = 0.0;
    for (int k = 0; k < cnt; ++k) s += B[(x * norb + o + k) * norb + o + k];
    out[x] = s;
}

// out[L] = sum_k A[L,k] * B[L,k] (row dot); grid over rows, warp per row.
__global__ void k_rowdot(const double *A, const double *B, long long L, long long m, double *out, double alpha,
                         int acc) {
    long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    int lane = threadIdx.x & 31;
    if (row >= L) return;
    double s = 0.0;
    for (long long k = lane; k < m; k += 32) s += A[row * m + k] * B[row * m + k];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[row] = acc ? out[row] + alpha * s : alpha * s;
}

// Block reduction into acc[slot] (double atomics).
__device__ __forceinline__ void block_add(double v, double *dst) {
    __shared__ double red[32];
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) red[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? red[l] : 0.0;
        for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (l == 0) atomicAdd(dst, v);
    }
    __syncthreads();
}

// SC finishing: per label L with norm dn[L], Koopmans numerator dk[L],
// denominator base[L] and the norms of the other states dnj[j*L + L]:
//   if dn passes the threshold:  den = base - dk/dn, co = dn/den
//      -> acc[0] += co (energy), acc[1] += co/den (norm)
//   acc[2+j] += dnj / den   (den != 0)
// mode: 0 |dn| > 0; 1 |dn| >= 1e-14; 2 |dn| > 1e-14.
__global__ void k_sc_finish(const double *dn, const double *dk, const double *base, const double *dnj, int nother,
                            long long L, int mode, double *acc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0, ps = 0.0, den = 0.0;
    double offs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (t < L) {
        double d = dn[t];
        double a = fabs(d);
        bool ok = mode == 0 ? a > 0.0 : (mode == 1 ? a >= 1e-14 : a > 1e-14);
        if (ok) {
            den = base[t] - dk[t] / d;
            double co = d / den;
            e = co;
            ps = co / den;
        }
        if (den != 0.0)
            for (int j = 0; j < nother && j < 8; ++j) offs[j] = dnj[(long long)j * L + t] / den;
    }
    block_add(e, acc + 0);
    block_add(ps, acc + 1);
    for (int j = 0; j < nother && j < 8; ++j) block_add(offs[j], acc + 2 + j);
}

// PC finishing over (label, mu): deno = w[mu] + base[L];
//  type 0:  r (own state) and rj (other states): e2 -= r^2/deno, psi += r^2/deno^2,
//           e2_j -= rj r / deno
//  type 1:  additionally rp, rpj: contri = (0.5 r^2 + 1.5 rp^2)/deno, off (0.5 rj r + 1.5 rpj rp)/deno
// R arrays are [L, nmu] (own) and [nother, L, nmu]; mu >= nmu_live adds 0.
__global__ void k_pc_finish(const double *R, const double *Rp, const double *Rj, const double *Rpj, int nother,
                            const double *w, const double *base, long long L, long long nmu, int type, double *acc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0, ps = 0.0;
    double offs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (t < L * nmu) {
        long long l = t / nmu, mu = t % nmu;
        double deno = w[mu] + base[l];
        double r = R[t];
        if (type == 0) {
            double c = r * r / deno;
            e = -c;
            ps = c / deno;
            for (int j = 0; j < nother && j < 8; ++j) offs[j] = -(Rj[(long long)j * L * nmu + t] * r) / deno;
        } else {
            double rp = Rp[t];
            double c = (0.5 * r * r + 1.5 * rp * rp) / deno;
            e = -c;
            ps = c / deno;
            for (int j = 0; j < nother && j < 8; ++j)
                offs[j] = -(0.5 * Rj[(long long)j * L * nmu + t] * r + 1.5 * Rpj[(long long)j * L * nmu + t] * rp) / deno;
        }
    }
    block_add(e, acc + 0);
    block_add(ps, acc + 1);
    for (int j = 0; j < nother && j < 8; ++j) block_add(offs[j], acc + 2 + j);
}

// PC sums of one class from the tridiagonal form of its pencil: for label l
// (one CTA each) with shift sig[l], x = (T + sig I)^-1 y_l by Gaussian
// elimination with partial pivoting on the tridiagonal T (d[n], e[n-1]),
// then
//   acc[0] -= y_l . x,   acc[1] += x . x,   acc[2 + k] -= y_{k+1,l} . x,
// which are the type-0 sums of k_pc_finish over the eigenpairs of T
// (sum_mu r_mu^2 / (w_mu + sig) = y^T (T + sig)^-1 y with r = G^T y).
// Y is row-major [n][ncol], column k L + l holding block k (0: own state,
// k > 0: the other states) of label l.  The CTA stages d, e and y_l in
// shared memory; one thread runs the elimination and the back substitution
// there (every step a shared-memory access, no global latency), then all
// threads form the dot products.  Shared memory: 6 n doubles.
// With nd > 0 the kernel also forms rho[l nd + k] = -x . Y[:, dcol0 + k] for
// k < nd: the first-order density of the label against nd extra right-hand
// sides transformed with the labels' (sum_mu r_mu v_mu,k / (w_mu + sig) =
// z^T (K + sig S)^-1 g_k with v = C^T g).  xout, when given, receives the
// solution x of each label, row-major [n][L].
__global__ void k_tridiag_resolvent(const double *d, const double *e, long long n, const double *Y, long long ncol,
                                    long long L, int nother, const double *sig, double *acc, int nd,
                                    long long dcol0, double *rho, double *xout) {
    extern __shared__ double sm[];
    double *sd = sm, *se = sm + n, *wb = sm + 2 * n, *wc = sm + 3 * n, *wd = sm + 4 * n, *wy = sm + 5 * n;
    const long long l = blockIdx.x;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        sd[i] = d[i];
        se[i] = i + 1 < n ? e[i] : 0.0;
        wy[i] = Y[i * ncol + l];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double s = sig[l];
        // row i: diagonal b, super-diagonal c; the fill of a row exchange goes to wd
        double b = sd[0] + s, cc = se[0], y = wy[0];
        for (long long i = 0; i + 1 < n; ++i) {
            const double a1 = se[i];                        // row i+1, column i
            const double b1 = sd[i + 1] + s;                // row i+1, column i+1
            const double c1 = i + 2 < n ? se[i + 1] : 0.0;  // row i+1, column i+2
            const double y1 = wy[i + 1];
            if (fabs(b) >= fabs(a1)) {  // keep row i as pivot row
                const double f = a1 / b;
                wb[i] = b; wc[i] = cc; wd[i] = 0.0; wy[i] = y;
                b = b1 - f * cc;
                cc = c1;
                y = y1 - f * y;
            } else {                    // interchange rows i and i+1
                const double f = b / a1;
                wb[i] = a1; wc[i] = b1; wd[i] = c1; wy[i] = y1;
                b = cc - f * b1;
                cc = -f * c1;
                y = y - f * y1;
            }
        }
        wb[n - 1] = b;
        // back substitution, x over wy
        double x2 = 0.0, x1 = y / b;
        wy[n - 1] = x1;
        for (long long i = n - 2; i >= 0; --i) {
            const double x = (wy[i] - wc[i] * x1 - wd[i] * x2) / wb[i];
            wy[i] = x;
            x2 = x1;
            x1 = x;
        }
    }
    __syncthreads();
    if (xout)
        for (long long i = threadIdx.x; i < n; i += blockDim.x) xout[i * L + l] = wy[i];
    double en = 0.0, ps = 0.0;
    double offs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double x = wy[i];
        en -= Y[i * ncol + l] * x;
        ps += x * x;
        for (int k = 0; k < nother && k < 8; ++k) offs[k] -= Y[i * ncol + (k + 1) * L + l] * x;
    }
    block_add(en, acc + 0);
    block_add(ps, acc + 1);
    for (int j = 0; j < nother && j < 8; ++j) block_add(offs[j], acc + 2 + j);
    for (int k = 0; k < nd; ++k) {
        double r = 0.0;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) r -= Y[i * ncol + dcol0 + k] * wy[i];
        block_add(r, rho + l * nd + k);
    }
}

// First-order density of a PC class on its eigenpairs: rho[l, k] =
// -sum_mu R[l, mu] V[k, mu] / (w_mu + base_l), one thread per (l, k).
__global__ void k_rho_pc(const double *R, const double *V, const double *w, const double *base, long long L,
                         long long nmu, int nd, double *rho) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L * nd) return;
    const long long l = t / nd;
    const int k = (int)(t % nd);
    double acc = 0.0;
    for (long long mu = 0; mu < nmu; ++mu) acc -= R[l * nmu + mu] * V[(long long)k * nmu + mu] / (w[mu] + base[l]);
    rho[t] = acc;
}

// The QD cross terms of the resolvent route in the original basis:
// acc[2 + k] -= sum_{l,i} Zo[(k L + l) n + i] X[l n + i] for the other states
// k < nother (blockIdx.y), X the labels' solutions (K + sig_l S)^-1 z_l.
__global__ void k_cross_dots(const double *Zo, const double *X, long long L, long long n, double *acc) {
    const int k = blockIdx.y;
    const long long tot = L * n;
    const double *z = Zo + (long long)k * tot;
    double s = 0.0;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x)
        s += z[t] * X[t];
    block_add(-s, acc + 2 + k);
}

// v0 (class 0): labels (ii <= ij) x (r <= s); G[i,r,j,s] = (i r | j s) wait: G = Rcv^T Rcv
__global__ void k_v0(const double *G, const double *eps, int nc, int nv, int voff, const unsigned char *fro,
                     double *acc) {
    long long npc = (long long)nc * (nc + 1) / 2, npv = (long long)nv * (nv + 1) / 2;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0.0, ps = 0.0;
    if (t < npc * npv) {
        long long pc = t / npv, pv = t % npv;
        // decode pair indices (ii <= ij), (r <= s) in row-major upper order
        int ii = 0;
        long long rem = pc;
        while (rem >= nc - ii) { rem -= nc - ii; ++ii; }
        int ij = ii + (int)rem;
        int r = 0;
        rem = pv;
        while (rem >= nv - r) { rem -= nv - r; ++r; }
        int s = r + (int)rem;
        if (!(fro && (fro[ii] || fro[ij]))) {
            long long NV = nv;
            // (ij r | s ii) = G[ij, r, ii, s];  (ij s | r ii) = G[ij, s, ii, r]
            double ab1 = G[((ij * NV + r) * nc + ii) * NV + s];
            double ab2 = G[((ij * NV + s) * nc + ii) * NV + r];
            bool zrs = r == s, zij = ii == ij;
            double dint;
            if (zrs && zij) dint = ab1;
            else if (zrs != zij) dint = sqrt(2.0) * ab1;
            else dint = 2.0 * sqrt(ab1 * ab1 + ab2 * ab2 - ab1 * ab2);
            double co = -dint / (eps[voff + r] + eps[voff + s] - eps[ii] - eps[ij]);
            e = dint * co;
            ps = co * co;
        }
    }
    block_add(e, acc + 0);
    block_add(ps, acc + 1);
}

// ---------------------------------------------------------------- host state
struct State {
    Ctx &c;
    int nc, na, nv, norb, M, s;
    long long Q;
    T eps;                      // (norb) device
    std::vector<double> eps_h;  // host copy
    T h;                        // transformed one-electron integrals [norb, norb]
    T Rcc, Rca, Rcv, Raa, Rav;  // transformed DF blocks [Q, p, q]
    State(Ctx &cc) : c(cc) {}
};

// Dense (p q | r s) block contraction over Q: out[(p,q),(r,s)] = X^T Y with
// X [Q, |pq|], Y [Q, |rs|].
T eri(Ctx &c, const T &X, const T &Y) {
    long long Q = X.sh[0], m = X.size() / Q, n = Y.size() / Q;
    T out = alloc(c, {m, n}, false);
    if (X.p == Y.p) gram(c, X.p, Q, m, out.p);  // (pq|rs) = (rs|pq): one triangle
    else gemm(c, true, false, m, n, Q, 1.0, X.p, m, Y.p, n, 0.0, out.p, n);
    return out;
}

struct PcResult {
    T C;       // [nd, nd]: columns mu < nnew are the PC coefficients, rest zero
    T w;       // [nd] reference layout (first nnew: K~ eigenvalues)
    int nnew;
};

// src/qdnevpt.F:1963-2033 and siblings: the PC metric sequence.
// Metrics of at least this order take the generalised-eigenproblem route
// when every metric eigenvalue is above the threshold.
constexpr long long kPcCholMin = 512;

PcResult pc_transform(Ctx &c, const T &S, const T &K, long long nd, double thr) {
    PcResult r;
    if (nd >= kPcCholMin && metric_above(c, S.p, nd, thr)) {
        // Every eigenvalue of S is kept (nnew = nd), so the orthonormalised
        // Koopmans eigenproblem X^T K X y = w y, X = U w_S^-1/2, is the pencil
        // K v = w S v with v = X y: same eigenvalues and, up to rotations
        // inside degenerate eigenspaces, the same PC coefficients C = X Y.
        // One Cholesky-based solve replaces the metric eigensolve and the
        // three order-nd GEMMs around it.
        T w = alloc(c, {nd}, false), V = alloc(c, {nd, nd}, false);
        if (sygvd_upper(c, K.p, S.p, nd, w.p, V.p)) {
            r.nnew = (int)nd;
            r.w = std::move(w);
            r.C = permuted(c, V, {1, 0});  // C[i][mu] = V[mu][i]
            return r;
        }
    }
    T w = alloc(c, {nd}, false), V = alloc(c, {nd, nd}, false);
    eigh_upper(c, S.p, nd, w.p, V.p);
    std::vector<double> wh(nd);
    ck(cudaMemcpyAsync(wh.data(), w.p, sizeof(double) * nd, cudaMemcpyDeviceToHost, c.st), "w copy");
    ck(cudaStreamSynchronize(c.st), "sync");
    // caux0p keeps w >= thr (negative eigenvalues are dependencies too);
    // eigenvalues are ascending, so the kept ones are a contiguous tail.
    long long first = 0;
    while (first < nd && !(wh[first] >= thr)) ++first;
    int nnew = (int)(nd - first);
    for (long long k = first; k < nd; ++k)
        if (!(wh[k] >= thr)) throw Error(2, "metric eigenvalues are not ascending");
    r.nnew = nnew;
    r.C = alloc(c, {nd, nd}, true);
    r.w = alloc(c, {nd}, false);
    ck(cudaMemcpyAsync(r.w.p, w.p, sizeof(double) * nd, cudaMemcpyDeviceToDevice, c.st), "w copy");
    if (nnew == 0) return r;
    // caux[i, k] = V[first+k][i] / sqrt(w[first+k])   (nd x nnew, row-major)
    std::vector<double> sc(nnew);
    for (int k = 0; k < nnew; ++k) sc[k] = 1.0 / std::sqrt(wh[first + k]);
    T cauxT = alloc(c, {nnew, nd}, false);  // cauxT[k][i]
    ck(cudaMemcpyAsync(cauxT.p, V.p + first * nd, sizeof(double) * nnew * nd, cudaMemcpyDeviceToDevice, c.st), "copy");
    T scale = alloc(c, {nnew}, false);
    ck(cudaMemcpyAsync(scale.p, sc.data(), sizeof(double) * nnew, cudaMemcpyHostToDevice, c.st), "copy");
    // scale rows of cauxT: use a GEMM-free row scaling via gather-free kernel
    {
        T tmp = alloc(c, {nnew, nd}, false);
        // tmp = diag(scale) cauxT via gemm_batched trick: C[k, :] = scale[k] * cauxT[k, :]
        gemm_batched(c, false, false, 1, nd, 1, 1.0, scale.p, 1, 1, cauxT.p, nd, nd, 0.0, tmp.p, nd, nd, nnew);
        cauxT = std::move(tmp);
    }
    T Ks = alloc(c, {nd, nd}, false);
    symmetrize_upper(c, K.p, nd, Ks.p);
    // Y = K caux  (nd x nnew);  Tm = caux^T Y  (nnew x nnew)
    T Y = alloc(c, {nd, nnew}, false);
    gemm(c, false, true, nd, nnew, nd, 1.0, Ks.p, nd, cauxT.p, nd, 0.0, Y.p, nnew);
    T Tm = alloc(c, {nnew, nnew}, false);
    gemm(c, false, false, nnew, nnew, nd, 1.0, cauxT.p, nd, Y.p, nnew, 0.0, Tm.p, nnew);
    T w2 = alloc(c, {nnew}, false), V2 = alloc(c, {nnew, nnew}, false);
    eigh_upper(c, Tm.p, nnew, w2.p, V2.p);
    ck(cudaMemcpyAsync(r.w.p, w2.p, sizeof(double) * nnew, cudaMemcpyDeviceToDevice, c.st), "w copy");
    // C[i, mu] = sum_k caux[i,k] V2col[k, mu] = sum_k cauxT[k][i] V2[mu][k]
    // C (nd x nd) with the first nnew columns: write C[:, :nnew] via ldc = nd
    gemm(c, true, true, nd, nnew, nnew, 1.0, cauxT.p, nd, V2.p, nnew, 0.0, r.C.p, nd);
    return r;
}

// Reference's state/pair index rules.
inline int pair_index(int big, int small) { return big * (big - 1) / 2 + small; }

// Labels over index pairs (p <= q, or p < q when strict) of a range of N,
// times an extra index e < E:  L = pair * E + e.  Each output row k = (k1,k2):
//   p != q:  c1 * src[base + p*sp + q*sq + e*se + k1*sk1 + k2*sk2] + c2 * (p <-> q)
//   p == q:  cdiag * src[base + p*(sp+sq) + e*se + ...]
struct PairGather {
    long long base, sp, sq, se, sk1, sk2;
    int N, E, K1, K2, strict;
    double c1, c2, cdiag;
};

__global__ void k_pair_gather(const double *src, PairGather g, double *out, long long L) {
    long long K = (long long)g.K1 * g.K2;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L * K) return;
    long long l = t / K, k = t % K;
    long long pair = l / g.E;
    int e = (int)(l % g.E);
    int p = 0;
    long long rem = pair;
    while (rem >= g.N - p - g.strict) { rem -= g.N - p - g.strict; ++p; }
    int q = p + g.strict + (int)rem;
    int k1 = (int)(k / g.K2), k2 = (int)(k % g.K2);
    long long ko = g.base + e * g.se + k1 * g.sk1 + k2 * g.sk2;
    double v;
    if (p != q) v = g.c1 * src[ko + p * g.sp + q * g.sq] + (g.c2 != 0.0 ? g.c2 * src[ko + q * g.sp + p * g.sq] : 0.0);
    else v = g.cdiag * src[ko + p * (g.sp + g.sq)];
    out[t] = v;
}

T pair_gather(Ctx &c, const T &src, PairGather g) {
    long long np = g.strict ? (long long)g.N * (g.N - 1) / 2 : (long long)g.N * (g.N + 1) / 2;
    long long L = np * g.E;
    T out = alloc(c, {L, (long long)g.K1 * g.K2}, false);
    if (L > 0) {
        k_pair_gather<<<nblk(L * g.K1 * g.K2), TPB, 0, c.st>>>(src.p, g, out.p, L);
        LAUNCHED();
        ck(cudaGetLastError(), "pair_gather");
    }
    return out;
}

// Zero the rows of labels whose orbitals are frozen (mask over labels).
__global__ void k_zero_rows(double *A, long long L, long long m, const unsigned char *mask) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < L * m && mask[t / m]) A[t] = 0.0;
}

// q[L] = sum V1[L,u] X[u,v] V2[L,v]
T bilin(Ctx &c, const T &V1, const double *X, long long m, const T &V2, double alpha = 1.0) {
    long long L = V1.sh[0];
    T q = alloc(c, {L}, true);
    if (L == 0) return q;
    T Y = alloc(c, {L, m}, false);
    gemm(c, false, false, L, m, m, 1.0, V1.p, m, X, m, 0.0, Y.p, m);
    k_rowdot<<<nblk(L * 32), TPB, 0, c.st>>>(Y.p, V2.p, L, m, q.p, alpha, 0);
    LAUNCHED();
    return q;
}

void rowdot_acc(Ctx &c, const T &A, const T &B, double *q, double alpha) {
    long long L = A.sh[0], m = A.size() / (L ? L : 1);
    if (L == 0) return;
    k_rowdot<<<nblk(L * 32), TPB, 0, c.st>>>(A.p, B.p, L, m, q, alpha, 1);
    LAUNCHED();
}

T upload(Ctx &c, const std::vector<double> &h) {
    T t = alloc(c, {(long long)h.size()}, false);
    if (!h.empty())
        ck(cudaMemcpyAsync(t.p, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, c.st), "upload");
    return t;
}

std::vector<double> download(Ctx &c, const double *p, long long n) {
    std::vector<double> h(n);
    if (n) {
        ck(cudaMemcpyAsync(h.data(), p, sizeof(double) * n, cudaMemcpyDeviceToHost, c.st), "download");
        ck(cudaStreamSynchronize(c.st), "sync");
    }
    return h;
}

T matmul(Ctx &c, const T &A, bool ta, const T &B, bool tb) {
    long long m = ta ? A.sh[1] : A.sh[0], k = ta ? A.sh[0] : A.sh[1];
    long long n = tb ? B.sh[0] : B.sh[1];
    T C = alloc(c, {m, n}, false);
    gemm(c, ta, tb, m, n, k, 1.0, A.p, A.sh[1], B.p, B.sh[1], 0.0, C.p, n);
    return C;
}

T view2(T &&t, long long r, long long cols) {
    t.nd = 2;
    t.sh[0] = r;
    t.sh[1] = cols;
    return std::move(t);
}

T copy_of(Ctx &c, const double *p, std::initializer_list<long long> shape) {
    T t = alloc(c, shape, false);
    ck(cudaMemcpyAsync(t.p, p, sizeof(double) * t.size(), cudaMemcpyDeviceToDevice, c.st), "copy");
    return t;
}

// Per-state RDM / Koopmans inputs on the device, C-ordered, plus transition
// arrays of the pairs this state takes part in.
struct StateData {
    T g1, g2, g3, hrdm, ipko1, eako1, ipko2, eako2, gk0pa, gk0pd, gk0pf;
    T aIP, aEA, bIP, bEA, cIP, cEA, dIP, dEA;
};
struct PairData {
    T d1, d2, d3;
};

struct Accum {  // host mirror of the reference's energy holders
    int M;
    std::vector<double> e2mpp, psimpp, e2enp, psienep, e2mp, e2en, psimp, psien;
    std::vector<long long> nnew;
    // first-order density blocks (compute_rho1st), Fortran order with the
    // state last: rhoir (nc, nv, M), rhoid (nc, na, M), rhodr (na, nv, M)
    bool rho = false;
    int nc = 0, na = 0, nv = 0;
    std::vector<double> rhoir, rhoid, rhodr;
    Accum(int m, int nc_ = 0, int na_ = 0, int nv_ = 0, bool rho_ = false)
        : M(m), e2mpp(8 * m), psimpp(8 * m), e2enp(8 * m), psienep(8 * m), e2mp(m * m), e2en(m * m), psimp(m),
          psien(m), nnew(10 * m, -1), rho(rho_), nc(nc_), na(na_), nv(nv_) {
        if (rho) {
            rhoir.assign((size_t)nc * nv * m, 0.0);
            rhoid.assign((size_t)nc * na * m, 0.0);
            rhodr.assign((size_t)na * nv * m, 0.0);
        }
    }
    double &E(std::vector<double> &v, int cls, int s) { return v[cls + 8 * s]; }   // (8, M) column-major
    double &H(std::vector<double> &v, int j, int s) { return v[j + M * s]; }       // (M, M) column-major
    // Adds the contributions a class collected in its own (zero-started)
    // accumulator.  Every slot a class assigns is zero before that class runs,
    // so adding reproduces the reference's sequence of stores.
    void merge(const Accum &o) {
        auto add = [](std::vector<double> &d, const std::vector<double> &x) {
            for (size_t i = 0; i < d.size(); ++i) d[i] += x[i];
        };
        add(e2mpp, o.e2mpp); add(psimpp, o.psimpp); add(e2enp, o.e2enp); add(psienep, o.psienep);
        add(e2mp, o.e2mp); add(e2en, o.e2en); add(psimp, o.psimp); add(psien, o.psien);
        if (rho && o.rho) {
            add(rhoir, o.rhoir); add(rhoid, o.rhoid); add(rhodr, o.rhodr);
        }
        for (size_t i = 0; i < nnew.size(); ++i)
            if (o.nnew[i] != -1) nnew[i] = o.nnew[i];
    }
};

// Non-blocking streams, each with its own cuBLAS/cuSOLVER handles, kept for
// the life of the process (one pool per device) and lent to the concurrent
// state / class tasks of a call; events order them against the caller's
// stream.
class CtxPool {
  public:
    static std::vector<Ctx> acquire(size_t n, int dev) {
        CtxPool &p = get();
        std::lock_guard<std::mutex> g(p.mu_);
        std::vector<Ctx> out;
        auto &free = p.free_[dev];
        while (out.size() < n && !free.empty()) {
            out.push_back(free.back());
            free.pop_back();
        }
        while (out.size() < n) {
            Ctx c{nullptr, nullptr, nullptr};
            ck(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking), "cudaStreamCreate");
            ck(cublasCreate(&c.blas), "cublasCreate");
            ck(cublasSetStream(c.blas, c.st), "cublasSetStream");
            ck(cusolverDnCreate(&c.sol), "cusolverDnCreate");
            ck(cusolverDnSetStream(c.sol, c.st), "cusolverDnSetStream");
            out.push_back(c);
        }
        return out;
    }
    static void release(std::vector<Ctx> &v, int dev) {
        CtxPool &p = get();
        std::lock_guard<std::mutex> g(p.mu_);
        for (auto &c : v) p.free_[dev].push_back(c);
        v.clear();
    }

  private:
    static CtxPool &get() {
        static CtxPool pool;
        return pool;
    }
    std::mutex mu_;
    std::map<int, std::vector<Ctx>> free_;
};

// The reduction of one pencil K v = w S v on a helper stream and host thread:
// the Cholesky check of the metric, its factorisation, the reduction to
// standard form and the tridiagonalisation need only S and K, so they overlap
// the caller's work on its own stream.  join() waits for them, orders the
// caller's stream after the helper's and hands the pencil's buffers to the
// caller's stream (where they are used and freed from then on).
class PencilFork {
  public:
    PencilFork(Ctx &caller, const T &S, const T &K, long long n, double thr, PencilTridiag &pt) : c_(caller), pt_(pt) {
        ck(cudaGetDevice(&dev_), "cudaGetDevice");
        aux_ = CtxPool::acquire(1, dev_);
        Ctx &a = aux_[0];
        a.split = c_.split;
        a.oz_err = c_.oz_err;
        a.sm_share = c_.sm_share;
        a.wait_limit = c_.wait_limit;
        a.all_pc_resolvent = c_.all_pc_resolvent;
        try {
            ck(cudaEventCreateWithFlags(&ready_, cudaEventDisableTiming), "cudaEventCreate");
            ck(cudaEventCreateWithFlags(&done_, cudaEventDisableTiming), "cudaEventCreate");
            ck(cudaEventRecord(ready_, c_.st), "cudaEventRecord");
            ck(cudaStreamWaitEvent(a.st, ready_, 0), "cudaStreamWaitEvent");
        } catch (...) {  // no thread yet: hand the helper context back before failing
            finish();
            throw;
        }
        const double *Sp = S.p, *Kp = K.p;
        th_ = std::thread([this, Sp, Kp, n, thr]() {
            try {
                ck(cudaSetDevice(dev_), "cudaSetDevice");
                ok_ = metric_above(aux_[0], Sp, n, thr) && pencil_tridiag(aux_[0], Kp, Sp, n, pt_);
            } catch (...) {
                err_ = std::current_exception();
            }
        });
    }
    PencilFork(const PencilFork &) = delete;
    PencilFork &operator=(const PencilFork &) = delete;
    // true when the metric kept every eigenvalue and the pencil is reduced
    bool join() {
        finish();
        if (err_) std::rethrow_exception(err_);
        return ok_;
    }
    ~PencilFork() { finish(); }

  private:
    void finish() {
        if (th_.joinable()) th_.join();
        if (aux_.empty()) return;
        Ctx &a = aux_[0];
        if (done_) {
            cudaEventRecord(done_, a.st);
            cudaStreamWaitEvent(c_.st, done_, 0);
        } else {
            cudaStreamSynchronize(a.st);
        }
        for (T *t : {&pt_.U, &pt_.A, &pt_.d, &pt_.e, &pt_.tau}) t->st = c_.st;
        a.split = false;
        a.oz_err = nullptr;
        a.sm_share = 1;
        a.wait_limit = 0;
        a.all_pc_resolvent = false;
        CtxPool::release(aux_, dev_);
        if (ready_) cudaEventDestroy(ready_);
        if (done_) cudaEventDestroy(done_);
        ready_ = done_ = nullptr;
    }
    Ctx &c_;
    PencilTridiag &pt_;
    int dev_ = 0;
    std::vector<Ctx> aux_;
    cudaEvent_t ready_ = nullptr, done_ = nullptr;
    std::thread th_;
    std::exception_ptr err_;
    bool ok_ = false;
};

class Runner {
  public:
    Ctx &c;
    int nc, na, nv, norb, M;
    long long Q;
    double thr;
    const unsigned char *fro_h;  // host mask (norb) or nullptr
    std::vector<StateData> &sd;
    std::vector<PairData> &pd;
    T B, h;  // dense DF tensor [Q,norb,norb], one-electron [norb,norb]
    Accum &acc;
    // per state
    int s;
    std::vector<double> eps;
    T Rcc, Rca, Rcv, Raa, Rav, hcv, hca, hav;
    T Jcc;  // [Q] sum_j Rcc[x,j,j]

    Runner(Ctx &cc, int nc_, int na_, int nv_, int M_, long long Q_, double thr_, const unsigned char *fro,
           std::vector<StateData> &sd_, std::vector<PairData> &pd_, Accum &a)
        : c(cc), nc(nc_), na(na_), nv(nv_), norb(nc_ + na_ + nv_), M(M_), Q(Q_), thr(thr_), fro_h(fro), sd(sd_),
          pd(pd_), acc(a) {}

    // A runner for one class of the current state: its own stream/handles and
    // accumulator, read-only views of b's per-state tensors.
    Runner(const Runner &b, Ctx &cc, Accum &a)
        : c(cc), nc(b.nc), na(b.na), nv(b.nv), norb(b.norb), M(b.M), Q(b.Q), thr(b.thr), fro_h(b.fro_h), sd(b.sd),
          pd(b.pd), acc(a), s(b.s), eps(b.eps) {
        B = T::view(b.B); h = T::view(b.h);
        Rcc = T::view(b.Rcc); Rca = T::view(b.Rca); Rcv = T::view(b.Rcv); Raa = T::view(b.Raa);
        Rav = T::view(b.Rav); hcv = T::view(b.hcv); hca = T::view(b.hca); hav = T::view(b.hav);
        Jcc = T::view(b.Jcc);
    }

    bool frozen(int orb) const { return fro_h && fro_h[orb]; }
    std::vector<int> others() const {
        std::vector<int> o;
        for (int j = 0; j < M; ++j)
            if (j != s) o.push_back(j);
        return o;
    }
    // (transition data of pair (s, j), true if j < s)
    std::pair<PairData *, bool> off(int j) {
        if (j < s) return {&pd[pair_index(s, j)], true};
        return {&pd[pair_index(j, s)], false};
    }

    // ------------------------------------------------ orbitals + integrals
    void prepare_state(int st) {
        s = st;
        StateData &D = sd[s];
        int n = na;
        // J vectors
        T Jc = alloc(c, {Q}, true);
        if (nc) {
            k_diag_sum<<<nblk(Q), TPB, 0, c.st>>>(B.p, Q, norb, 0, nc, Jc.p);
            LAUNCHED();
        }
        T Baa = alloc(c, {Q, (long long)n * n}, false);
        gather(c, B.p, (long long)nc * norb + nc, {Q, n, n}, {(long long)norb * norb, norb, 1}, Baa.p);
        T g1T = permuted(c, D.g1, {1, 0});
        T Ja = alloc(c, {Q}, false);
        gemm(c, false, false, Q, 1, (long long)n * n, 1.0, Baa.p, (long long)n * n, g1T.p, 1, 0.0, Ja.p, 1);
        T Jt = alloc(c, {Q}, false);
        axpby(c, Q, 2.0, Jc.p, 1.0, Ja.p, Jt.p);
        eps.assign(norb, 0.0);
        T Vc, Vv;
        auto fock = [&](int o, int ns, T &V) {
            T F = alloc(c, {ns, ns}, false);
            gather(c, h.p, (long long)o * norb + o, {ns, ns}, {norb, 1}, F.p);
            T Bss = alloc(c, {Q, (long long)ns * ns}, false);
            gather(c, B.p, (long long)o * norb + o, {Q, ns, ns}, {(long long)norb * norb, norb, 1}, Bss.p);
            gemm(c, false, false, 1, (long long)ns * ns, Q, 1.0, Jt.p, Q, Bss.p, (long long)ns * ns, 1.0, F.p,
                 (long long)ns * ns);
            if (nc) {
                T G = alloc(c, {ns, Q * nc}, false);
                gather(c, B.p, (long long)o * norb, {ns, Q, nc}, {norb, (long long)norb * norb, 1}, G.p);
                gemm(c, false, true, ns, ns, Q * nc, -1.0, G.p, Q * nc, G.p, Q * nc, 1.0, F.p, ns);
            }
            T Gp = alloc(c, {ns, Q * n}, false);
            gather(c, B.p, (long long)o * norb + nc, {ns, Q, n}, {norb, (long long)norb * norb, 1}, Gp.p);
            T H = alloc(c, {ns, Q * n}, false);  // H[p,(x,a)] = sum_b B[x,p,b] g1[b,a]
            gemm(c, false, false, (long long)ns * Q, n, n, 1.0, Gp.p, n, D.g1.p, n, 0.0, H.p, n);
            gemm(c, false, true, ns, ns, Q * n, -0.5, H.p, Q * n, Gp.p, Q * n, 1.0, F.p, ns);
            T w = alloc(c, {ns}, false);
            V = alloc(c, {ns, ns}, false);
            eigh_upper(c, F.p, ns, w.p, V.p);
            auto wh = download(c, w.p, ns);
            for (int k = 0; k < ns; ++k) eps[o + k] = wh[k];
        };
        if (nc) fock(0, nc, Vc);
        fock(nc + na, nv, Vv);
        // transformed DF blocks.  V rows are eigenvectors: U = V^T.
        long long NN = (long long)norb * norb;
        auto block = [&](int po, int np, int qo, int nq) {
            T b = alloc(c, {Q, np, nq}, false);
            gather(c, B.p, (long long)po * norb + qo, {Q, np, nq}, {NN, norb, 1}, b.p);
            return b;
        };
        auto left = [&](T &X, T &V, int np, int nq) {  // X[x] = V X[x]
            T Y = alloc(c, {Q, np, nq}, false);
            gemm_batched(c, false, false, np, nq, np, 1.0, V.p, np, 0, X.p, nq, (long long)np * nq, 0.0, Y.p, nq,
                         (long long)np * nq, Q);
            X = std::move(Y);
        };
        auto right = [&](T &X, T &V, int np, int nq) {  // X[x] = X[x] V^T
            T Y = alloc(c, {Q, np, nq}, false);
            gemm_batched(c, false, true, np, nq, nq, 1.0, X.p, nq, (long long)np * nq, V.p, nq, 0, 0.0, Y.p, nq,
                         (long long)np * nq, Q);
            X = std::move(Y);
        };
        int vo = nc + na;
        Raa = block(nc, na, nc, na);
        Rav = block(nc, na, vo, nv);
        right(Rav, Vv, na, nv);
        if (nc) {
            Rcc = block(0, nc, 0, nc);
            left(Rcc, Vc, nc, nc);
            right(Rcc, Vc, nc, nc);
            Rca = block(0, nc, nc, na);
            left(Rca, Vc, nc, na);
            Rcv = block(0, nc, vo, nv);
            left(Rcv, Vc, nc, nv);
            right(Rcv, Vv, nc, nv);
        } else {
            Rcc = alloc(c, {Q, 0, 0});
            Rca = alloc(c, {Q, 0, na});
            Rcv = alloc(c, {Q, 0, nv});
        }
        // one-electron blocks h' = U^T h U
        auto hblk = [&](int po, int np, int qo, int nq) {
            T b = alloc(c, {np, nq}, false);
            gather(c, h.p, (long long)po * norb + qo, {np, nq}, {norb, 1}, b.p);
            return b;
        };
        hav = hblk(nc, na, vo, nv);
        hav = matmul(c, hav, false, Vv, true);
        if (nc) {
            hcv = matmul(c, matmul(c, Vc, false, hblk(0, nc, vo, nv), false), false, Vv, true);
            hca = matmul(c, Vc, false, hblk(0, nc, nc, na), false);
        } else {
            hcv = alloc(c, {0, nv});
            hca = alloc(c, {0, na});
        }
        Jcc = alloc(c, {Q}, true);
        if (nc) {
            // sum_j Rcc[x,j,j]
            T tmp = alloc(c, {Q, nc}, false);
            gather(c, Rcc.p, 0, {Q, nc}, {(long long)nc * nc, nc + 1}, tmp.p);
            T ones = upload(c, std::vector<double>(nc, 1.0));
            gemm(c, false, false, Q, 1, nc, 1.0, tmp.p, nc, ones.p, 1, 0.0, Jcc.p, 1);
        }
    }

    T eri2(const T &X, const T &Y) {  // X [Q,p,q], Y [Q,r,s] -> [(p,q),(r,s)]
        return eri(c, X, Y);
    }
    T dev_eps() { return upload(c, eps); }

    // ---------------------------------------------------------- finishing
    std::vector<double> sc_finish(const T &dn, const T &dk, const std::vector<double> &base, const T &dnj, int mode) {
        long long L = dn.size();
        int no = M - 1;
        T bs = upload(c, base);
        T a = alloc(c, {2 + 8}, true);
        if (L > 0) {
            k_sc_finish<<<nblk(L), TPB, 0, c.st>>>(dn.p, dk.p, bs.p, dnj.p, no, L, mode, a.p);
            LAUNCHED();
        }
        return download(c, a.p, 2 + 8);
    }
    void sc_store(int cls, const std::vector<double> &r) {
        acc.H(acc.e2mp, s, s) += r[0];
        acc.psimp[s] += r[1];
        acc.E(acc.e2mpp, cls, s) += r[0];
        acc.E(acc.psimpp, cls, s) += r[1];
        auto o = others();
        for (size_t k = 0; k < o.size(); ++k) acc.H(acc.e2mp, o[k], s) += r[2 + k];
    }
    // PC: R [L,nmu] own, Rj [M-1, L, nmu]; Rp/Rpj for type 1.
    std::vector<double> pc_finish(const T &R, const T *Rp, const T &Rj, const T *Rpj, const T &w,
                                  const std::vector<double> &base, long long nmu, int type) {
        long long L = (long long)base.size();
        T bs = upload(c, base);
        T a = alloc(c, {2 + 8}, true);
        if (L * nmu > 0) {
            k_pc_finish<<<nblk(L * nmu), TPB, 0, c.st>>>(R.p, Rp ? Rp->p : nullptr, Rj.p, Rpj ? Rpj->p : nullptr,
                                                          M - 1, w.p, bs.p, L, nmu, type, a.p);
            LAUNCHED();
        }
        return download(c, a.p, 2 + 8);
    }
    // PC sums from the tridiagonal form of a pencil: Yt row-major [n][M L]
    // (column k L + l: state block k of label l), shifts per label.
    std::vector<double> resolvent_sums(const PencilTridiag &PT, const T &Yt, const std::vector<double> &shift,
                                       int nd = 0, long long dcol0 = 0, double *rho = nullptr, int nother = -1,
                                       double *xout = nullptr) {
        const long long L = (long long)shift.size(), n = PT.n;
        T sg = upload(c, shift);
        T a = alloc(c, {2 + 8}, true);
        if (L > 0 && n > 0) {
            const size_t smem = sizeof(double) * 6 * (size_t)n;
            // one limit for every caller: pencils of different orders are
            // solved concurrently on other host threads
            const int lim = raise_dynamic_smem((const void *)k_tridiag_resolvent);
            if ((long long)smem > lim) throw Error(NVPT_EINVAL, "resolvent: pencil order above the shared-memory limit");
            ProfSpan sp;
            sp.begin("pencil_solve", c.st, 0);
            k_tridiag_resolvent<<<(unsigned)L, 128, smem, c.st>>>(PT.d.p, PT.e.p, n, Yt.p, Yt.sh[1], L,
                                                                   nother < 0 ? M - 1 : nother, sg.p, a.p, nd, dcol0,
                                                                   rho, xout);
            sp.end();
            LAUNCHED();
        }
        return download(c, a.p, 2 + 8);
    }
    // The resolvent route of a PC class whose metric keeps every eigenvalue
    // (nnew = nd): sum_mu r_mu^2 / (w_mu + s_l) = z_l^T (K + s_l S)^-1 z_l.
    // fill(Z) writes the numerator rows z before the PC basis change, Z
    // row-major [M L, nd]: own state first, then the other states in
    // others() order.  Returns false, with nothing accumulated and fill not
    // called, when a metric eigenvalue is below the threshold.
    bool pc_resolvent(const T &S, const T &K, long long nd, long long L, int nnew_slot,
                      const std::vector<double> &shift, std::vector<double> &e2, double &psi2,
                      const std::function<void(double *)> &fill) {
        if (nd == 0 || L == 0 || !c.all_pc_resolvent) return false;
        PencilTridiag PT;
        if (!(metric_above(c, S.p, nd, thr) && pencil_tridiag(c, K.p, S.p, nd, PT))) return false;
        acc.nnew[nnew_slot + 10 * s] = (int)nd;
        const long long rows = (long long)M * L;
        T Z = alloc(c, {rows, nd}, false);
        fill(Z.p);
        // rows of Z are the columns of a column-major [nd, M L]
        pencil_rhs(c, PT, Z.p, rows);
        T Yt = permuted(c, Z, {1, 0});  // [nd][M L]
        pc_accum(e2, psi2, resolvent_sums(PT, Yt, shift));
        return true;
    }
    // First-order density on the eigenpairs: [L, nd] = -sum_mu R[l,mu] V[k,mu] / (w_mu + base_l)
    std::vector<double> rho_pc(const T &R, const T &V, const T &w, const std::vector<double> &base, long long nmu,
                               int nd) {
        const long long L = (long long)base.size();
        T bs = upload(c, base);
        T out = alloc(c, {L, (long long)nd}, true);
        if (L * nd > 0) {
            k_rho_pc<<<nblk(L * nd), TPB, 0, c.st>>>(R.p, V.p, w.p, bs.p, L, nmu, nd, out.p);
            LAUNCHED();
        }
        return download(c, out.p, L * nd);
    }
    void pc_accum(std::vector<double> &e2, double &psi2, const std::vector<double> &r) {
        e2[s + M * s] += r[0];
        psi2 += r[1];
        auto o = others();
        for (size_t k = 0; k < o.size(); ++k) e2[o[k] + M * s] += r[2 + k];
    }
    void pc_store(int cls, const std::vector<double> &e2, double psi2, bool assign) {
        if (assign) {
            acc.E(acc.e2enp, cls, s) = e2[s + M * s];
            acc.E(acc.psienep, cls, s) = psi2;
            acc.psien[s] += psi2;
        } else {
            acc.E(acc.e2enp, cls, s) += e2[s + M * s];
            acc.E(acc.psienep, cls, s) += psi2;
            acc.psien[s] += acc.E(acc.psienep, cls, s);
        }
        acc.H(acc.e2en, s, s) += e2[s + M * s];
        for (int j : others()) acc.H(acc.e2en, j, s) += e2[j + M * s];
    }

    // Stack per-other-state rows: out[j] = f(j) for the M-1 other states.
    T stack_others(long long L, long long m, const std::function<void(int, double *)> &f) {
        int no = M - 1;
        T out = alloc(c, {(long long)(no > 0 ? no : 1), L, m}, true);
        auto o = others();
        for (int k = 0; k < no; ++k) f(o[k], out.p + (long long)k * L * m);
        return out;
    }
    T mask_labels(const std::vector<unsigned char> &m) {
        T t = alloc(c, {(long long)m.size()}, false);
        // store as bytes inside a double buffer (enough room)
        if (!m.empty())
            ck(cudaMemcpyAsync(t.p, m.data(), m.size(), cudaMemcpyHostToDevice, c.st), "mask upload");
        return t;
    }
    void zero_rows(T &A, const std::vector<unsigned char> &mask) {
        bool any = false;
        for (auto v : mask) any |= v != 0;
        if (!any) return;
        T m = mask_labels(mask);
        long long L = A.sh[0], w = A.size() / (L ? L : 1);
        k_zero_rows<<<nblk(L * w), TPB, 0, c.st>>>(A.p, L, w, (const unsigned char *)m.p);
        LAUNCHED();
    }

    // ============================================================ classes
    void class0() {  // v0 :1661
        if (!nc) {
            acc.H(acc.e2en, s, s) = acc.H(acc.e2mp, s, s);
            acc.psien[s] = acc.psimp[s];
            return;
        }
        T G = eri2(Rcv, Rcv);  // [(i,r),(j,s)]
        T e = dev_eps();
        T fm = alloc(c, {(long long)norb}, false);
        std::vector<unsigned char> fmask(norb, 0);
        if (fro_h)
            for (int k = 0; k < norb; ++k) fmask[k] = fro_h[k];
        ck(cudaMemcpyAsync(fm.p, fmask.data(), norb, cudaMemcpyHostToDevice, c.st), "fro");
        T a = alloc(c, {2}, true);
        long long labels = (long long)nc * (nc + 1) / 2 * ((long long)nv * (nv + 1) / 2);
        k_v0<<<nblk(labels), TPB, 0, c.st>>>(G.p, e.p, nc, nv, nc + na, (const unsigned char *)fm.p, a.p);
        LAUNCHED();
        auto r = download(c, a.p, 2);
        acc.H(acc.e2mp, s, s) += r[0];
        acc.psimp[s] += r[1];
        acc.E(acc.e2mpp, 0, s) += r[0];
        acc.E(acc.psimpp, 0, s) += r[1];
        acc.H(acc.e2en, s, s) = acc.H(acc.e2mp, s, s);
        acc.psien[s] = acc.psimp[s];
        acc.E(acc.e2enp, 0, s) = acc.E(acc.e2mpp, 0, s);
        acc.E(acc.psienep, 0, s) = acc.E(acc.psimpp, 0, s);
    }

    // v1k / vm1k share the structure: labels (pair, ext) with two vectors.
    void class_pm1(bool plus, bool pc) {
        int n = na;
        StateData &D = sd[s];
        // plus: T = (i a | j r) as [i,a,j,r]; minus: T = (i r | a s) as [i,r,a,s]
        T Tm = plus ? eri2(Rca, Rcv) : eri2(Rcv, Rav);
        if (plus && !nc) return;
        if (!plus && !nc) return;
        long long s0, s1, s2, s3;
        PairGather gj{}, gk{};
        int N, E;
        if (plus) {  // labels (ii <= ij) x virtual s; vector index a
            s3 = 1; s2 = nv; s1 = (long long)nc * nv; s0 = (long long)n * nc * nv;
            N = nc; E = nv;
            gj = PairGather{0, s0, s2, s3, s1, 0, N, E, n, 1, 0, 1.0, 0.0, 1.0};   // tj = T[ii,a,ij,s]
            gk = PairGather{0, s2, s0, s3, s1, 0, N, E, n, 1, 0, 1.0, 0.0, 1.0};   // tk = T[ij,a,ii,s]
        } else {     // labels (r <= s) x core i; vector index a.  T[i,r,a,s]
            s3 = 1; s2 = nv; s1 = (long long)n * nv; s0 = (long long)nv * n * nv;
            N = nv; E = nc;
            gj = PairGather{0, s1, s3, s0, s2, 0, N, E, n, 1, 0, 1.0, 0.0, 1.0};   // tj = T[i,r,a,s]
            gk = PairGather{0, s3, s1, s0, s2, 0, N, E, n, 1, 0, 1.0, 0.0, 1.0};   // tk = T[i,s,a,r]
        }
        T Vj = pair_gather(c, Tm, gj), Vk = pair_gather(c, Tm, gk);
        long long L = Vj.sh[0];
        // labels: pair (p,q), e
        std::vector<double> base(L);
        std::vector<unsigned char> same(L), fmask(L, 0);
        {
            long long l = 0;
            for (int p = 0; p < N; ++p)
                for (int q = p; q < N; ++q)
                    for (int e = 0; e < E; ++e, ++l) {
                        same[l] = p == q;
                        if (plus) {
                            base[l] = eps[p] + eps[q] - eps[nc + na + e];
                            fmask[l] = frozen(p) || frozen(q);
                        } else {
                            base[l] = eps[e] - eps[nc + na + p] - eps[nc + na + q];
                            fmask[l] = frozen(e);
                        }
                    }
        }
        // sum_ab X[a,b] cint[a,b] with cint = tj tj^T + tk tk^T - (tj tk^T + tk tj^T)/2
        // (p != q) or tj tj^T / 2 (p == q).  Zero tk on p == q and halve tj there:
        // (tj/sqrt2)^T X (tj/sqrt2) = tj^T X tj / 2.
        T Vj2 = copy_of(c, Vj.p, {L, n}), Vk2 = copy_of(c, Vk.p, {L, n});
        {
            std::vector<double> sj(L), sk(L);
            for (long long l = 0; l < L; ++l) {
                sj[l] = same[l] ? std::sqrt(0.5) : 1.0;
                sk[l] = same[l] ? 0.0 : 1.0;
            }
            scale_rows(Vj2, sj);
            scale_rows(Vk2, sk);
            zero_rows(Vj2, fmask);
            zero_rows(Vk2, fmask);
        }
        auto cform = [&](const double *X) {
            T q = bilin(c, Vj2, X, n, Vj2);
            T q2 = bilin(c, Vk2, X, n, Vk2);
            axpby(c, L, 1.0, q.p, 1.0, q2.p, q.p);
            T q3 = bilin(c, Vj2, X, n, Vk2);
            T q4 = bilin(c, Vk2, X, n, Vj2);
            axpby(c, L, 1.0, q.p, -0.5, q3.p, q.p);
            axpby(c, L, 1.0, q.p, -0.5, q4.p, q.p);
            return q;
        };
        // norms: plus: ro = 2 delta - g1 ; minus: g1
        T ro = copy_of(c, D.g1.p, {n, n});
        if (plus) {
            std::vector<double> I2(n * n, 0.0);
            for (int a = 0; a < n; ++a) I2[a * n + a] = 2.0;
            T Id = upload(c, I2);
            axpby(c, (long long)n * n, 1.0, Id.p, -1.0, D.g1.p, ro.p);
        }
        T dn = cform(ro.p);
        axpby(c, L, 2.0, dn.p, 0.0, nullptr, dn.p);
        const T &gk_ = plus ? D.eako1 : D.ipko1;
        T dk = cform(gk_.p);
        T dnj = stack_others(L, 1, [&](int j, double *out) {
            auto [P, lt] = off(j);
            // plus: ro_j[a,ap] = -daoff(iap,ia) (j<i) / -daoff(ia,iap); minus: daoff(ia,iap) / daoff(iap,ia)
            T X = plus ? (lt ? permuted(c, P->d1, {1, 0}, -1.0) : permuted(c, P->d1, {0, 1}, -1.0))
                       : (lt ? permuted(c, P->d1, {0, 1}) : permuted(c, P->d1, {1, 0}));
            T q = cform(X.p);
            axpby(c, L, 2.0, q.p, 0.0, nullptr, out);
        });
        auto r = sc_finish(dn, dk, base, dnj, plus ? 0 : 1);
        sc_store(plus ? 1 : 2, r);
        if (!pc) return;
        // PC (e2p1cont / e2m1cont)
        T S = copy_of(c, ro.p, {n, n});
        T Kk = alloc(c, {n, n}, false);
        axpby(c, (long long)n * n, 0.5, gk_.p, 0.0, nullptr, Kk.p);
        PcResult P = pc_transform(c, S, Kk, n, thr);
        acc.nnew[(plus ? 0 : 1) + 10 * s] = P.nnew;
        // own: s(a,mu) = sum_ap X[ap,a] C[ap,mu]  (X = 2-g1 or g1)
        T sm = matmul(c, ro, true, P.C, false);  // [n, n]
        // vectors: p != q: tj+tk and tj-tk; p == q: sqrt2 tj and 0
        T Vp = alloc(c, {L, n}, false), Vm = alloc(c, {L, n}, false);
        axpby(c, L * n, 1.0, Vj.p, 1.0, Vk.p, Vp.p);
        axpby(c, L * n, 1.0, Vj.p, -1.0, Vk.p, Vm.p);
        {
            std::vector<double> sp(L), sm_(L);
            for (long long l = 0; l < L; ++l) {
                sp[l] = 1.0;
                sm_[l] = same[l] ? 0.0 : 1.0;
            }
            // on p == q: Vp = tj + tk = 2 tj (tk == tj there); want sqrt2 tj
            for (long long l = 0; l < L; ++l)
                if (same[l]) sp[l] = std::sqrt(2.0) / 2.0;
            scale_rows(Vp, sp);
            scale_rows(Vm, sm_);
            zero_rows(Vp, fmask);
            zero_rows(Vm, fmask);
        }
        T R = matmul(c, Vp, false, sm, false), Rp = matmul(c, Vm, false, sm, false);
        T Rj = stack_others(L, n, [&](int j, double *out) {
            auto [PD, lt] = off(j);
            // plus: ro[a,ap] = -daoff(a,ap) (j<i) / -daoff(ap,a);  minus: daoff(ap,a) (j<i) / daoff(a,ap)
            T X = plus ? (lt ? permuted(c, PD->d1, {0, 1}, -1.0) : permuted(c, PD->d1, {1, 0}, -1.0))
                       : (lt ? permuted(c, PD->d1, {1, 0}) : permuted(c, PD->d1, {0, 1}));
            T sj = matmul(c, X, false, P.C, false);
            gemm(c, false, false, L, n, n, 1.0, Vp.p, n, sj.p, n, 0.0, out, n);
        });
        T Rpj = stack_others(L, n, [&](int j, double *out) {
            auto [PD, lt] = off(j);
            T X = plus ? (lt ? permuted(c, PD->d1, {0, 1}, -1.0) : permuted(c, PD->d1, {1, 0}, -1.0))
                       : (lt ? permuted(c, PD->d1, {1, 0}) : permuted(c, PD->d1, {0, 1}));
            T sj = matmul(c, X, false, P.C, false);
            gemm(c, false, false, L, n, n, 1.0, Vm.p, n, sj.p, n, 0.0, out, n);
        });
        std::vector<double> pbase(L);
        for (long long l = 0; l < L; ++l) pbase[l] = -base[l];  // w + eps_r - eps_i - eps_j  /  w + eps_r + eps_s - eps_i
        std::vector<double> e2(M * M, 0.0);
        double psi2 = 0.0;
        pc_accum(e2, psi2, pc_finish(R, &Rp, Rj, &Rpj, P.w, pbase, n, 1));
        pc_store(plus ? 1 : 2, e2, psi2, true);
    }

    void scale_rows(T &A, const std::vector<double> &f) {
        long long L = A.sh[0], m = A.size() / (L ? L : 1);
        if (!L) return;
        T fs = upload(c, f);
        T out = alloc(c, {L, m}, false);
        gemm_batched(c, false, false, 1, m, 1, 1.0, fs.p, 1, 1, A.p, m, m, 0.0, out.p, m, m, L);
        A = std::move(out);
        A.nd = 2;
        A.sh[0] = L;
        A.sh[1] = m;
    }

    // ------------------------------------------------------ classes (+-2)
    // Pair-restriction matrix P [n^2, np]: column pair(a<=b) picks row (a,b)
    // with weight w_diag on a == b and w_off on a < b.
    T pair_matrix(double w_diag, double w_off, bool transposed_rows) {
        int n = na;
        long long np = (long long)n * (n + 1) / 2;
        std::vector<double> P((size_t)n * n * np, 0.0);
        long long k = 0;
        for (int a = 0; a < n; ++a)
            for (int b = a; b < n; ++b, ++k) {
                long long row = transposed_rows ? (long long)b * n + a : (long long)a * n + b;
                P[row * np + k] = a == b ? w_diag : w_off;
            }
        T t = upload(c, P);
        return view2(std::move(t), (long long)n * n, np);
    }
    // restricted square: P0^T X P0 for an n^2 x n^2 matrix X
    T restrict_sq(const T &X) {
        T P0 = pair_matrix(1.0, 1.0, false);
        T Y = matmul(c, X, false, P0, false);
        return matmul(c, P0, true, Y, false);
    }

    void class_pm2(bool plus, bool pc) {
        int n = na, n2 = n * n;
        StateData &D = sd[s];
        const T &Dm = plus ? D.hrdm : D.g2;      // daat (+2) or daa (-2)
        const T &Km = plus ? D.eako2 : D.ipko2;  // gkp2aa / gkm2aa
        int N = plus ? nc : nv;
        if (N == 0) return;
        // integrals: plus T = (i a | j b) [i,a,j,b]; minus T = (a r | b s) [a,r,b,s]
        T Tm = plus ? eri2(Rca, Rca) : eri2(Rav, Rav);
        long long st0, st1, st2, st3;  // strides of the 4 axes
        if (plus) { st3 = 1; st2 = n; st1 = (long long)nc * n; st0 = (long long)n * nc * n; }
        else { st3 = 1; st2 = nv; st1 = (long long)n * nv; st0 = (long long)nv * n * nv; }
        // SC vectors v[c,d] per pair (p<=q): plus: T[p,c,q,d]; minus d1 = (q c | p d) = T[c,q,d,p]
        PairGather gne = plus ? PairGather{0, st0, st2, 0, st1, st3, N, 1, n, n, 1, 1.0, 0.0, 0.0}
                              : PairGather{0, st3, st1, 0, st0, st2, N, 1, n, n, 1, 1.0, 0.0, 0.0};
        T Vne = pair_gather(c, Tm, gne);
        // diagonal labels only (p == q): a strided gather with weight 0.5 (absorbs cint * 0.25)
        T Veq = alloc(c, {(long long)N, (long long)n2}, false);
        if (plus) gather(c, Tm.p, 0, {N, n, n}, {st0 + st2, st1, st3}, Veq.p, 0.5);
        else gather(c, Tm.p, 0, {N, n, n}, {st1 + st3, st0, st2}, Veq.p, 0.5);
        long long Lne = Vne.sh[0], Leq = N;
        std::vector<unsigned char> fne(Lne, 0), feq(Leq, 0);
        std::vector<double> bne(Lne), beq(Leq);
        {
            long long l = 0;
            int o = plus ? 0 : nc + na;
            for (int p = 0; p < N; ++p)
                for (int q = p + 1; q < N; ++q, ++l) {
                    bne[l] = plus ? eps[p] + eps[q] : -eps[o + p] - eps[o + q];
                    fne[l] = plus && (frozen(p) || frozen(q));
                }
            for (int p = 0; p < N; ++p) {
                beq[p] = plus ? 2.0 * eps[p] : -2.0 * eps[o + p];
                feq[p] = plus && frozen(p);
            }
        }
        zero_rows(Vne, fne);
        zero_rows(Veq, feq);
        // matrices [(cp,dp),(c,d)]
        T Deq = copy_of(c, Dm.p, {n2, n2});
        permute(c, Dm.p, {n, n, n, n}, {0, 1, 3, 2}, Deq.p, 1.0, true);
        T Keq = copy_of(c, Km.p, {n2, n2});
        permute(c, Km.p, {n, n, n, n}, {1, 0, 2, 3}, Keq.p, 1.0, true);
        // bilinear forms: q = v^T X v with X indexed [cp dp, c d] and v over both
        auto forms = [&](const T &V, const double *X) { return bilin(c, V, X, n2, V); };
        T dn = alloc(c, {Lne + Leq}, false), dk = alloc(c, {Lne + Leq}, false);
        {
            T a = forms(Vne, Dm.p), b = forms(Veq, Deq.p);
            ck(cudaMemcpyAsync(dn.p, a.p, sizeof(double) * Lne, cudaMemcpyDeviceToDevice, c.st), "cp");
            ck(cudaMemcpyAsync(dn.p + Lne, b.p, sizeof(double) * Leq, cudaMemcpyDeviceToDevice, c.st), "cp");
            T a2 = forms(Vne, Km.p), b2 = forms(Veq, Keq.p);
            ck(cudaMemcpyAsync(dk.p, a2.p, sizeof(double) * Lne, cudaMemcpyDeviceToDevice, c.st), "cp");
            ck(cudaMemcpyAsync(dk.p + Lne, b2.p, sizeof(double) * Leq, cudaMemcpyDeviceToDevice, c.st), "cp");
        }
        long long L = Lne + Leq;
        T dnj = stack_others(L, 1, [&](int j, double *out) {
            auto [P, lt] = off(j);
            T rt = alloc(c, {n, n, n, n}, false);
            if (plus) build_ro2toff(c, P->d2.p, P->d1.p, n, rt.p);
            else ck(cudaMemcpyAsync(rt.p, P->d2.p, sizeof(double) * rt.size(), cudaMemcpyDeviceToDevice, c.st), "cp");
            // plus:  lt: rt (+ rt^(1,0,2,3));  else rt^(2,3,0,1) (+ rt^(3,2,0,1))
            // minus: lt: d^(2,3,0,1) (+ d^(3,2,0,1));  else d (+ d^(1,0,2,3))
            bool firstform = plus ? lt : !lt;
            T Xn = firstform ? copy_of(c, rt.p, {n2, n2}) : permuted(c, rt, {2, 3, 0, 1});
            T Xe = copy_of(c, Xn.p, {n2, n2});
            if (firstform) permute(c, rt.p, {n, n, n, n}, {1, 0, 2, 3}, Xe.p, 1.0, true);
            else permute(c, rt.p, {n, n, n, n}, {3, 2, 0, 1}, Xe.p, 1.0, true);
            T a = forms(Vne, Xn.p), b = forms(Veq, Xe.p);
            ck(cudaMemcpyAsync(out, a.p, sizeof(double) * Lne, cudaMemcpyDeviceToDevice, c.st), "cp");
            ck(cudaMemcpyAsync(out + Lne, b.p, sizeof(double) * Leq, cudaMemcpyDeviceToDevice, c.st), "cp");
        });
        // plus: den = eps_r + eps_s - dk/dn ; minus: den = -dk/dn - eps_r - eps_s (base carries the signs)
        std::vector<double> base(bne);
        base.insert(base.end(), beq.begin(), beq.end());
        auto r = sc_finish(dn, dk, base, dnj, 1);
        sc_store(plus ? 3 : 4, r);
        if (!pc) return;
        std::vector<double> e2(M * M, 0.0);
        double psi2 = 0.0;
        // ---- (a) r != s: metric fillcm2 (row (i,j), j fastest) ----
        {
            T S = copy_of(c, Dm.p, {n2, n2}), K = copy_of(c, Km.p, {n2, n2});
            // labels: plus (i<j core): dint[ab] = (i b | j a) = T[i,b,j,a];
            //         minus (r<s virt): dint[ab] = d1(b,a), d1 = (r a | s b) -> T[b,r,a,s]
            PairGather g = plus ? PairGather{0, st0, st2, 0, st3, st1, N, 1, n, n, 1, 1.0, 0.0, 0.0}
                                : PairGather{0, st1, st3, 0, st2, st0, N, 1, n, n, 1, 1.0, 0.0, 0.0};
            T V = pair_gather(c, Tm, g);
            zero_rows(V, fne);
            // the transition metric of another state j, [(ap,bp), (a,b)]
            auto xmet = [&](int j) {
                auto [PD, lt] = off(j);
                T rt = alloc(c, {n, n, n, n}, false);
                if (plus) build_ro2toff(c, PD->d2.p, PD->d1.p, n, rt.p);
                else ck(cudaMemcpyAsync(rt.p, PD->d2.p, sizeof(double) * rt.size(), cudaMemcpyDeviceToDevice, c.st), "cp");
                // plus: lt rt^(1,0,3,2) else rt^(3,2,1,0); minus: lt d^(3,2,1,0) else d^(1,0,3,2)
                bool a1 = plus ? lt : !lt;
                T X = a1 ? permuted(c, rt, {1, 0, 3, 2}) : permuted(c, rt, {3, 2, 1, 0});
                return view2(std::move(X), n2, n2);
            };
            std::vector<double> pb(Lne);  // deno = w - eps_i - eps_j  /  w + eps_r + eps_s
            for (long long l = 0; l < Lne; ++l) pb[l] = -bne[l];
            // numerators before the PC basis change: own z = S^T v (R = V S^T C), other z = X_j^T v
            const bool res = pc_resolvent(S, K, n2, Lne, plus ? 2 : 4, pb, e2, psi2, [&](double *Z) {
                gemm(c, false, true, Lne, n2, n2, 1.0, V.p, n2, S.p, n2, 0.0, Z, n2);
                auto o = others();
                for (size_t k = 0; k < o.size(); ++k) {
                    T Xm = xmet(o[k]);
                    gemm(c, false, false, Lne, n2, n2, 1.0, V.p, n2, Xm.p, n2, 0.0, Z + (long long)(k + 1) * Lne * n2,
                         n2);
                }
            });
            if (!res) {
                PcResult P = pc_transform(c, S, K, n2, thr);
                acc.nnew[(plus ? 2 : 4) + 10 * s] = P.nnew;
                T sm = matmul(c, S, true, P.C, false);  // s(ab,mu) = sum_{pq} D[pq,ab] C[pq,mu]
                T R = matmul(c, V, false, sm, false);
                T Rj = stack_others(Lne, n2, [&](int j, double *out) {
                    T Xm = xmet(j);
                    T sj = matmul(c, Xm, false, P.C, false);
                    gemm(c, false, false, Lne, n2, n2, 1.0, V.p, n2, sj.p, n2, 0.0, out, n2);
                });
                pc_accum(e2, psi2, pc_finish(R, nullptr, Rj, nullptr, P.w, pb, n2, 0));
            }
        }
        // ---- (b) r == s: metric fillcm2p on pairs a <= b ----
        {
            long long np = (long long)n * (n + 1) / 2;
            T Sf = copy_of(c, Dm.p, {n2, n2});
            permute(c, Dm.p, {n, n, n, n}, {0, 1, 3, 2}, Sf.p, 1.0, true);
            T Kf = copy_of(c, Km.p, {n2, n2});
            permute(c, Km.p, {n, n, n, n}, {0, 1, 3, 2}, Kf.p, 1.0, true);
            T Sp = restrict_sq(Sf), Kp = restrict_sq(Kf);
            // labels: plus core i: dint[pair(a,b)] = w T[i,b,i,a]; minus virt r: w T[a,r,b,r]
            T Vf = alloc(c, {(long long)N, (long long)n2}, false);
            if (plus) gather(c, Tm.p, 0, {N, n, n}, {st0 + st2, st3, st1}, Vf.p);  // [i, a, b] = T[i,b,i,a]
            else gather(c, Tm.p, 0, {N, n, n}, {st1 + st3, st0, st2}, Vf.p);      // [r, a, b] = T[a,r,b,r]
            zero_rows(Vf, feq);
            T Pw = pair_matrix(1.0, 2.0, false);
            T V = matmul(c, Vf, false, Pw, false);  // [N, np]
            // the transition metric of another state j on pairs, [pair ab, pair abp]
            auto xmet = [&](int j) {
                auto [PD, lt] = off(j);
                T rt = alloc(c, {n, n, n, n}, false);
                if (plus) build_ro2toff(c, PD->d2.p, PD->d1.p, n, rt.p);
                else ck(cudaMemcpyAsync(rt.p, PD->d2.p, sizeof(double) * rt.size(), cudaMemcpyDeviceToDevice, c.st), "cp");
                // plus lt: 0.5(rt^(1,0,3,2)+rt^(1,0,2,3)) else 0.5(rt^(3,2,1,0)+rt^(3,2,0,1))
                // minus lt: 0.5(d^(3,2,1,0)+d^(3,2,0,1)) else 0.5(d^(1,0,2,3)+d^(1,0,3,2))
                bool a1 = plus ? lt : !lt;
                T X = alloc(c, {n2, n2}, false);
                if (a1) {
                    permute(c, rt.p, {n, n, n, n}, {1, 0, 3, 2}, X.p, 0.5, false);
                    permute(c, rt.p, {n, n, n, n}, {1, 0, 2, 3}, X.p, 0.5, true);
                } else {
                    permute(c, rt.p, {n, n, n, n}, {3, 2, 1, 0}, X.p, 0.5, false);
                    permute(c, rt.p, {n, n, n, n}, {3, 2, 0, 1}, X.p, 0.5, true);
                }
                return restrict_sq(X);
            };
            std::vector<double> pb(Leq);
            for (long long l = 0; l < Leq; ++l) pb[l] = -beq[l];
            // numerators before the PC basis change: own z = 0.5 Sp^T v, other z = X_j^T v
            const bool res = pc_resolvent(Sp, Kp, np, Leq, plus ? 3 : 5, pb, e2, psi2, [&](double *Z) {
                gemm(c, false, true, Leq, np, np, 0.5, V.p, np, Sp.p, np, 0.0, Z, np);
                auto o = others();
                for (size_t k = 0; k < o.size(); ++k) {
                    T Xr = xmet(o[k]);
                    gemm(c, false, false, Leq, np, np, 1.0, V.p, np, Xr.p, np, 0.0, Z + (long long)(k + 1) * Leq * np,
                         np);
                }
            });
            if (!res) {
                PcResult P = pc_transform(c, Sp, Kp, np, thr);
                acc.nnew[(plus ? 3 : 5) + 10 * s] = P.nnew;
                // s(ab,mu) = sum_{abp} 0.5 Sf[abp, ab] C[abp, mu]
                T smp = matmul(c, Sp, true, P.C, false);
                axpby(c, np * np, 0.5, smp.p, 0.0, nullptr, smp.p);
                T R = matmul(c, V, false, smp, false);
                T Rj = stack_others(Leq, np, [&](int j, double *out) {
                    T Xr = xmet(j);
                    T sj = matmul(c, Xr, false, P.C, false);
                    gemm(c, false, false, Leq, np, np, 1.0, V.p, np, sj.p, np, 0.0, out, np);
                });
                pc_accum(e2, psi2, pc_finish(R, nullptr, Rj, nullptr, P.w, pb, np, 0));
            }
        }
        pc_store(plus ? 3 : 4, e2, psi2, false);
    }

    // ------------------------------------------------------ class (0')
    void class0p(bool pc) {  // v0pmod :4326, fillc0p :4195, e20pcont :4771
        int n = na, nn = n * n;
        StateData &D = sd[s];
        if (!nc) return;
        long long L = (long long)nc * nv;  // labels (i, r)
        // heffd(i,r) = h'(i,r) + sum_j [2 (jj|ir) - (ji|jr)]
        T hd = copy_of(c, hcv.p, {nc, nv});
        gemm(c, false, false, 1, L, Q, 2.0, Jcc.p, Q, Rcv.p, L, 1.0, hd.p, L);
        gemm(c, true, false, nc, nv, Q * nc, -1.0, Rcc.p, nc, Rcv.p, nv, 1.0, hd.p, nv);
        T DJ = eri2(Rcv, Raa);                        // [(i,r),(a,b)]
        T DKr = eri2(Rca, Rav);                       // [(i,a),(b,r)]
        T DK = alloc(c, {L, nn}, false);             // [(i,r),(a,b)] = DKr[i,a,b,r]
        permute(c, DKr.p, {nc, n, n, nv}, {0, 3, 1, 2}, DK.p);
        DJ = view2(std::move(DJ), L, nn);
        T E2 = alloc(c, {n, n, n, n}, false);
        build_ee2L(c, D.g2.p, D.g1.p, n, E2.p);
        T E2tr = alloc(c, {n, n, n, n}, false);
        build_ee2trL(c, E2.p, D.g1.p, n, E2tr.p);
        // dum1[ap,bp,a,b] = ee2(bp,ap,a,b); dum2 = ee2tr(bp,b,ap,a) + [a==b] da(bp,ap)
        T dum1 = permuted(c, E2, {1, 0, 2, 3});
        T dum2 = permuted(c, E2tr, {2, 0, 3, 1});
        add_diag_pairs(c, dum2.p, n, 2, 3, D.g1.p, true, 1.0);
        T dk1 = permuted(c, D.gk0pa, {1, 0, 2, 3});
        T dk2 = permuted(c, D.gk0pd, {1, 0, 2, 3});
        std::vector<unsigned char> fm(L, 0);
        for (int i = 0; i < nc; ++i)
            for (int r = 0; r < nv; ++r) fm[(long long)i * nv + r] = frozen(i);
        zero_rows(DJ, fm);
        zero_rows(DK, fm);
        // dn = 2 dj'D1dj - dj'D1dk - dk'D1dj + dk'D2dk  (x' X y = sum x[pq] X[pq,ab] y[ab])
        auto quad = [&](const double *X1, const double *X2, double c11, double c12, double c21, double c22,
                        double *out) {
            T q = bilin(c, DJ, X1, nn, DJ, c11);
            T y = alloc(c, {L, (long long)nn}, false);
            gemm(c, false, false, L, nn, nn, 1.0, DJ.p, nn, X1, nn, 0.0, y.p, nn);  // y = dj' X1
            rowdot_acc(c, y, DK, q.p, c12);                                          // dj' X1 dk
            gemm(c, false, false, L, nn, nn, 1.0, DK.p, nn, X1, nn, 0.0, y.p, nn);  // dk' X1
            rowdot_acc(c, y, DJ, q.p, c21);                                          // dk' X1 dj
            gemm(c, false, false, L, nn, nn, 1.0, DK.p, nn, X2, nn, 0.0, y.p, nn);
            rowdot_acc(c, y, DK, q.p, c22);                                          // dk' X2 dk
            ck(cudaMemcpyAsync(out, q.p, sizeof(double) * L, cudaMemcpyDeviceToDevice, c.st), "cp");
        };
        T dn = alloc(c, {L}, false), dkoo = alloc(c, {L}, false);
        quad(dum1.p, dum2.p, 2.0, -1.0, -1.0, 1.0, dn.p);
        quad(dk1.p, dk2.p, 1.0, -0.5, -0.5, 1.0, dkoo.p);
        // di = 2 dj - dk; dummy = sum g1[b,a] di[a,b]; dummyk = 1/2 sum gf[a,b] di[a,b]
        T di = alloc(c, {L, (long long)nn}, false);
        axpby(c, L * nn, 2.0, DJ.p, -1.0, DK.p, di.p);
        T g1T = permuted(c, D.g1, {1, 0});
        T dummy = alloc(c, {L}, false), dummyk = alloc(c, {L}, false);
        gemm(c, false, false, L, 1, nn, 1.0, di.p, nn, g1T.p, 1, 0.0, dummy.p, 1);
        gemm(c, false, false, L, 1, nn, 0.5, di.p, nn, D.gk0pf.p, 1, 0.0, dummyk.p, 1);
        // dn += 2 h dummy + 2 h^2 ; dkoo += h dummyk   (elementwise over labels)
        auto hv = download(c, hd.p, L);
        auto dumh = download(c, dummy.p, L), dumkh = download(c, dummyk.p, L);
        auto dnh = download(c, dn.p, L), dkh = download(c, dkoo.p, L);
        for (long long l = 0; l < L; ++l) {
            if (fm[l]) hv[l] = 0.0;
            dnh[l] += 2.0 * hv[l] * dumh[l] + 2.0 * hv[l] * hv[l];
            dkh[l] += hv[l] * dumkh[l];
        }
        T dnd = upload(c, dnh), dkd = upload(c, dkh);
        T dnj = stack_others(L, 1, [&](int j, double *out) {
            auto [P, lt] = off(j);
            (void)lt;
            T E2o = alloc(c, {n, n, n, n}, false), E2tro = alloc(c, {n, n, n, n}, false);
            build_ee2L(c, P->d2.p, P->d1.p, n, E2o.p);
            build_ee2trL(c, E2o.p, P->d1.p, n, E2tro.p);
            T o1 = permuted(c, E2o, {1, 0, 2, 3});
            T o2 = permuted(c, E2tro, {2, 0, 3, 1});
            add_diag_pairs(c, o2.p, n, 2, 3, P->d1.p, false, 1.0);
            quad(o1.p, o2.p, 2.0, -1.0, -1.0, 1.0, out);
            // + h * sum (daoff(b,a) + daoff(a,b)) di[a,b]
            T dsum = copy_of(c, P->d1.p, {n, n});
            permute(c, P->d1.p, {n, n}, {1, 0}, dsum.p, 1.0, true);
            T t = alloc(c, {L}, false);
            gemm(c, false, false, L, 1, nn, 1.0, di.p, nn, dsum.p, 1, 0.0, t.p, 1);
            auto th = download(c, t.p, L);
            auto oh = download(c, out, L);
            for (long long l = 0; l < L; ++l) oh[l] += hv[l] * th[l];
            ck(cudaMemcpyAsync(out, oh.data(), sizeof(double) * L, cudaMemcpyHostToDevice, c.st), "up");
            ck(cudaStreamSynchronize(c.st), "sync");
        });
        std::vector<double> base(L);
        for (int i = 0; i < nc; ++i)
            for (int r = 0; r < nv; ++r) base[(long long)i * nv + r] = eps[i] - eps[nc + na + r];
        auto res = sc_finish(dnd, dkd, base, dnj, 2);
        sc_store(7, res);
        if (!pc) return;
        // ---- PC: fillc0p (order 2 n^2) ----
        long long n2 = 2LL * nn;
        T S = alloc(c, {n2, n2}, false), K = alloc(c, {n2, n2}, false);
        T Snw = permuted(c, E2, {2, 3, 1, 0});  // ee2(bp,ap,a,b) at [a,b,ap,bp]
        T Sse = alloc(c, {n, n, n, n}, false);
        {   // -daa(bp,a,b,ap) at [a,b,ap,bp]  + [a==ap] 2 da(bp,b)
            gather(c, D.g2.p, 0, {n, n, n, n}, {(long long)n * n, n, 1, (long long)n * n * n}, Sse.p, -1.0);
            add_diag_pairs(c, Sse.p, n, 0, 2, D.g1.p, true, 2.0);
        }
        T Kga = permuted(c, D.gk0pa, {1, 0, 2, 3}), Kgd = permuted(c, D.gk0pd, {1, 0, 2, 3});
        // dst[(ro+i)*n2 + co + j] = alpha * src[i*nn + j]
        auto place = [&](T &dst, const T &src, long long ro, long long co, double alpha) {
            T tmp = alloc(c, {nn, nn}, false);
            gather(c, src.p, 0, {nn, nn}, {nn, 1}, tmp.p, alpha);
            ck(cudaMemcpy2DAsync(dst.p + ro * n2 + co, sizeof(double) * n2, tmp.p, sizeof(double) * nn,
                                 sizeof(double) * nn, nn, cudaMemcpyDeviceToDevice, c.st),
               "copy2d");
        };
        place(S, Snw, 0, 0, 2.0);
        place(S, Snw, 0, nn, -1.0);
        place(S, Snw, nn, 0, -1.0);
        place(S, Sse, nn, nn, 1.0);
        place(K, Kga, 0, 0, 1.0);
        place(K, Kga, 0, nn, -0.5);
        place(K, Kga, nn, 0, -0.5);
        place(K, Kgd, nn, nn, 1.0);
        T val = view2(copy_of(c, Snw.p, {nn, nn}), nn, nn);
        T val2 = alloc(c, {n, n, n, n}, false);  // -daa(ap,b,a,bp) at [a,b,ap,bp] + [ap==a] 2 da(b,bp)
        gather(c, D.g2.p, 0, {n, n, n, n}, {(long long)n, (long long)n * n, (long long)n * n * n, 1}, val2.p, -1.0);
        add_diag_pairs(c, val2.p, n, 0, 2, D.g1.p, false, 2.0);
        T val2m = view2(std::move(val2), nn, nn);
        T gba = permuted(c, D.g1, {1, 0});  // ro vector gba[ab] = da(b,a)
        T hdev = upload(c, hv);
        // the matrices of another state j: v ~ val, v2 ~ val2, ro ~ gba
        struct OtherMats { T v, v2, ro; };
        auto other_mats = [&](int j) {
            auto [PD, lt] = off(j);
            T E2o = alloc(c, {n, n, n, n}, false);
            build_ee2L(c, PD->d2.p, PD->d1.p, n, E2o.p);
            T v = lt ? permuted(c, E2o, {1, 0, 2, 3}) : permuted(c, E2o, {2, 3, 1, 0});
            T v2 = alloc(c, {n, n, n, n}, false);
            if (lt) {  // -daaoff(a,bp,ap,b) + [ap==a] 2 daoff(bp,b)
                gather(c, PD->d2.p, 0, {n, n, n, n},
                       {(long long)n * n * n, 1, (long long)n, (long long)n * n}, v2.p, -1.0);
                add_diag_pairs(c, v2.p, n, 0, 2, PD->d1.p, true, 2.0);
            } else {   // -daaoff(ap,b,a,bp) + [ap==a] 2 daoff(b,bp)
                gather(c, PD->d2.p, 0, {n, n, n, n},
                       {(long long)n, (long long)n * n, (long long)n * n * n, 1}, v2.p, -1.0);
                add_diag_pairs(c, v2.p, n, 0, 2, PD->d1.p, false, 2.0);
            }
            T ro = lt ? permuted(c, PD->d1, {1, 0}) : copy_of(c, PD->d1.p, {n, n});  // daoff(b,a) / daoff(a,b)
            return OtherMats{view2(std::move(v), nn, nn), view2(std::move(v2), nn, nn), std::move(ro)};
        };
        std::vector<double> pb(L);
        for (long long l = 0; l < L; ++l) pb[l] = -base[l];  // deno = w + eps_r - eps_i
        std::vector<double> e2(M * M, 0.0);
        double psi2 = 0.0;
        const int nrho = acc.rho ? 1 : 0;
        auto store_rho = [&](const std::vector<double> &rl) {
            for (int i = 0; i < nc; ++i)
                for (int r = 0; r < nv; ++r) acc.rhoir[i + (size_t)nc * (r + (size_t)nv * s)] += rl[(size_t)i * nv + r];
        };
        PencilTridiag PT;
        if (c.all_pc_resolvent && metric_above(c, S.p, n2, thr) && pencil_tridiag(c, K.p, S.p, n2, PT)) {
            // every metric eigenvalue is kept: resolvents of the pencil (as in
            // the (+-1') classes) on the numerators before the PC basis change,
            //   z = [di A1 + 2 h g1 | -dj A1 + dk A2 - h g1]   (R = z C),
            // and for the density the vector g = [2 da | -da] (vaux = g C)
            acc.nnew[8 + 10 * s] = (int)n2;
            const long long rows = (long long)M * L + nrho;
            T Z = alloc(c, {rows, n2}, false);
            auto zrows = [&](const T &A1, const T &A2, const double *g1, double *out) {
                gemm(c, false, false, L, nn, nn, 1.0, di.p, nn, A1.p, nn, 0.0, out, n2);
                gemm(c, false, false, L, nn, 1, 2.0, hdev.p, 1, g1, nn, 1.0, out, n2);
                gemm(c, false, false, L, nn, nn, -1.0, DJ.p, nn, A1.p, nn, 0.0, out + nn, n2);
                gemm(c, false, false, L, nn, nn, 1.0, DK.p, nn, A2.p, nn, 1.0, out + nn, n2);
                gemm(c, false, false, L, nn, 1, -1.0, hdev.p, 1, g1, nn, 1.0, out + nn, n2);
            };
            zrows(val, val2m, gba.p, Z.p);
            auto o = others();
            for (size_t k = 0; k < o.size(); ++k) {
                OtherMats m = other_mats(o[k]);
                zrows(m.v, m.v2, m.ro.p, Z.p + (long long)(k + 1) * L * n2);
            }
            if (nrho) {
                double *g = Z.p + (long long)M * L * n2;
                axpby(c, nn, 2.0, D.g1.p, 0.0, nullptr, g);
                axpby(c, nn, -1.0, D.g1.p, 0.0, nullptr, g + nn);
            }
            pencil_rhs(c, PT, Z.p, rows);
            T Yt = permuted(c, Z, {1, 0});  // [n2][M L + nrho]
            T rho = alloc(c, {L, 1}, true);
            pc_accum(e2, psi2, resolvent_sums(PT, Yt, pb, nrho, (long long)M * L, rho.p));
            pc_store(7, e2, psi2, true);
            if (nrho) store_rho(download(c, rho.p, L));
            return;
        }
        PcResult P = pc_transform(c, S, K, n2, thr);
        acc.nnew[8 + 10 * s] = P.nnew;
        // aux: s = val C_top, sp = val C_bot, spp = val2 C_bot (val = Snw as [ab,abp])
        T Ctop = alloc(c, {(long long)nn, n2}, false), Cbot = alloc(c, {(long long)nn, n2}, false);
        ck(cudaMemcpyAsync(Ctop.p, P.C.p, sizeof(double) * nn * n2, cudaMemcpyDeviceToDevice, c.st), "cp");
        ck(cudaMemcpyAsync(Cbot.p, P.C.p + nn * n2, sizeof(double) * nn * n2, cudaMemcpyDeviceToDevice, c.st), "cp");
        T sA = matmul(c, val, false, Ctop, false), sP = matmul(c, val, false, Cbot, false);
        T sPP = matmul(c, val2m, false, Cbot, false);
        T gtop = alloc(c, {1, n2}, false), gbot = alloc(c, {1, n2}, false);
        gemm(c, false, false, 1, n2, nn, 1.0, gba.p, nn, Ctop.p, n2, 0.0, gtop.p, n2);
        gemm(c, false, false, 1, n2, nn, 1.0, gba.p, nn, Cbot.p, n2, 0.0, gbot.p, n2);
        auto rim = [&](const T &s_, const T &sp_, const T &spp_, const T &gt, const T &gb, double *out) {
            // out[L,mu] = di s + (-dj) sp + dk spp + h (2 gt - gb)
            gemm(c, false, false, L, n2, nn, 1.0, di.p, nn, s_.p, n2, 0.0, out, n2);
            gemm(c, false, false, L, n2, nn, -1.0, DJ.p, nn, sp_.p, n2, 1.0, out, n2);
            gemm(c, false, false, L, n2, nn, 1.0, DK.p, nn, spp_.p, n2, 1.0, out, n2);
            T g = alloc(c, {1, n2}, false);
            axpby(c, n2, 2.0, gt.p, -1.0, gb.p, g.p);
            gemm(c, false, false, L, n2, 1, 1.0, hdev.p, 1, g.p, n2, 1.0, out, n2);
        };
        T R = alloc(c, {L, n2}, false);
        rim(sA, sP, sPP, gtop, gbot, R.p);
        T Rj = stack_others(L, n2, [&](int j, double *out) {
            OtherMats m = other_mats(j);
            T sj = matmul(c, m.v, false, Ctop, false), spj = matmul(c, m.v, false, Cbot, false);
            T sppj = matmul(c, m.v2, false, Cbot, false);
            T gt = alloc(c, {1, n2}, false), gb = alloc(c, {1, n2}, false);
            gemm(c, false, false, 1, n2, nn, 1.0, m.ro.p, nn, Ctop.p, n2, 0.0, gt.p, n2);
            gemm(c, false, false, 1, n2, nn, 1.0, m.ro.p, nn, Cbot.p, n2, 0.0, gb.p, n2);
            rim(sj, spj, sppj, gt, gb, out);
        });
        pc_accum(e2, psi2, pc_finish(R, nullptr, Rj, nullptr, P.w, pb, n2, 0));
        pc_store(7, e2, psi2, true);
        if (nrho) {
            // e20pcont :4854-4860, :4971-4975: rhoir(i,r) -= sum_mu c_mu vaux_mu with
            // vaux_mu = sum_ab da(a,b) (2 coef(ab,mu) - coef(ab+nn,mu))
            T v = alloc(c, {1, n2}, false);
            gemm(c, false, false, 1, n2, nn, 2.0, D.g1.p, nn, Ctop.p, n2, 0.0, v.p, n2);
            gemm(c, false, false, 1, n2, nn, -1.0, D.g1.p, nn, Cbot.p, n2, 1.0, v.p, n2);
            store_rho(rho_pc(R, v, P.w, pb, n2, 1));
        }
    }

    // ------------------------------------------------ classes (-1') and (+1')
    // minus: vmupE :5869 + fillcm1p :4266 + e2m1pcont :5214 (labels: virtual r)
    // plus:  vpupE :5437 + fillcp1p :4296 + e21pcont :5001 (labels: core i)
    void class_pm1p(bool minus, bool pc) {
        int n = na, n3 = n * n * n;
        StateData &D = sd[s];
        int Lx = minus ? nv : nc;
        if (Lx == 0) return;
        const T &A = minus ? D.aIP : D.aEA;
        const T &Bm = minus ? D.bIP : D.bEA;
        const T &Cm = minus ? D.cIP : D.cEA;
        const T &Dm = minus ? D.dIP : D.dEA;
        // heffd [Lx, n]
        T H = alloc(c, {(long long)Lx, (long long)n}, false);
        if (minus) {
            // heffd(a,r) = h'(a,r) + sum_j [2 (a r|jj) - (a j|r j)] - sum_b (a b|b r)
            T hr = copy_of(c, hav.p, {n, nv});  // [a, r]
            gemm(c, false, false, 1, (long long)n * nv, Q, 2.0, Jcc.p, Q, Rav.p, (long long)n * nv, 1.0, hr.p,
                 (long long)n * nv);
            if (nc) gemm(c, true, false, n, nv, Q * nc, -1.0, Rca.p, n, Rcv.p, nv, 1.0, hr.p, nv);
            T RaaP = permuted(c, Raa, {1, 0, 2});  // [a, x, b]
            gemm(c, false, false, n, nv, Q * n, -1.0, RaaP.p, Q * n, Rav.p, nv, 1.0, hr.p, nv);
            permute(c, hr.p, {n, nv}, {1, 0}, H.p);
        } else {
            // heffd(i,a) = h'(i,a) + sum_j [2 (jj|ia) - (ji|ja)]
            ck(cudaMemcpyAsync(H.p, hca.p, sizeof(double) * nc * n, cudaMemcpyDeviceToDevice, c.st), "cp");
            gemm(c, false, false, 1, (long long)nc * n, Q, 2.0, Jcc.p, Q, Rca.p, (long long)nc * n, 1.0, H.p,
                 (long long)nc * n);
            gemm(c, true, false, nc, n, Q * nc, -1.0, Rcc.p, nc, Rca.p, n, 1.0, H.p, n);
        }
        // label vectors Vd[L, (ap,bp,cp)] = dint1(ap,cp,bp)
        T Vd = alloc(c, {(long long)Lx, (long long)n3}, false);
        if (minus) {
            T X3 = eri2(Raa, Rav);  // [(a,b),(c,r)] = (a b | c r)
            permute(c, X3.p, {n, n, n, nv}, {3, 0, 2, 1}, Vd.p);
        } else {
            T X = eri2(Raa, Rca);   // [(a,b),(i,c)] = (a b | c i)
            permute(c, X.p, {n, n, nc, n}, {2, 0, 3, 1}, Vd.p);
        }
        std::vector<unsigned char> fm(Lx, 0);
        if (!minus)
            for (int i = 0; i < nc; ++i) fm[i] = frozen(i);
        zero_rows(Vd, fm);
        zero_rows(H, fm);
        // accessor tensors of this state
        T E2 = alloc(c, {n, n, n, n}, false), E3 = alloc(c, {n, n, n, n, n, n}, false);
        build_ee2L(c, D.g2.p, D.g1.p, n, E2.p);
        build_eee2L(c, D.g3.p, D.g2.p, D.g1.p, n, E3.p);
        T W2 = alloc(c, {n, n, n, n}, false), W3 = alloc(c, {n, n, n, n, n, n}, false);
        T rho = copy_of(c, D.g1.p, {n, n});  // [ap, a]
        if (minus) {
            permute(c, E2.p, {n, n, n, n}, {1, 2, 0, 3}, W2.p);           // ee2(cp,ap,bp,a)
            permute(c, E3.p, {n, n, n, n, n, n}, {1, 2, 0, 4, 3, 5}, W3.p);  // eee2(cp,ap,bp,b,a,c)
        } else {
            T E2tr = alloc(c, {n, n, n, n}, false), E3t = alloc(c, {n, n, n, n, n, n}, false);
            build_ee2trL(c, E2.p, D.g1.p, n, E2tr.p);
            build_eee2tL(c, E3.p, E2.p, n, E3t.p);
            permute(c, E2tr.p, {n, n, n, n}, {1, 2, 0, 3}, W2.p);
            permute(c, E3t.p, {n, n, n, n, n, n}, {1, 2, 0, 4, 3, 5}, W3.p);
            std::vector<double> I2(n * n, 0.0);
            for (int a = 0; a < n; ++a) I2[a * n + a] = 2.0;
            T Id = upload(c, I2);
            axpby(c, (long long)n * n, 1.0, Id.p, -1.0, D.g1.p, rho.p);  // 2 delta - da(ap,a)
        }
        T Bc = copy_of(c, Bm.p, {n, n, n, n});
        permute(c, Cm.p, {n, n, n, n}, {1, 2, 3, 0}, Bc.p, 1.0, true);  // + cmat(a,ap,bp,cp)
        long long L = Lx;
        // With PC, the order-n^3 products of the SC forms are the first terms
        // of the PC numerators, so they are formed once: own state
        // dp'W3 dp = diag(Vd S Vd^T) with the metric S = W3^T (the diagonal of
        // a quadratic form does not see the transpose); another state j:
        // Vd W3o_j is Vd S_j, S_j the transition metric of its numerators.
        T S, K, Yown;
        std::map<int, T> yoth;
        PencilTridiag PT;
        std::unique_ptr<PencilFork> fork;
        if (pc) {
            S = view2(permuted(c, W3, {3, 4, 5, 0, 1, 2}), n3, n3);  // [(a,b,c),(ap,bp,cp)]
            K = view2(permuted(c, A, {3, 4, 5, 0, 1, 2}), n3, n3);
            // the pencil's reduction overlaps the SC work below
            if (n3 >= kPcCholMin || c.all_pc_resolvent) fork.reset(new PencilFork(c, S, K, n3, thr, PT));
            Yown = alloc(c, {L, (long long)n3}, false);
            gemm(c, false, false, L, n3, n3, 1.0, Vd.p, n3, S.p, n3, 0.0, Yown.p, n3);
        }
        // dumm = h'rho h + 2 dp'W2 h + dp'W3 dp ; dumk = h'Dm h + dp'Bc h + dp'A dp
        // (y3pre: Vd W3 or a product with the same diagonal form; y3keep: keep Vd W3)
        auto form3 = [&](const double *rho_, const double *w2, double c2, const double *w3, double *out,
                         const T *y3pre, T *y3keep) {
            T q = bilin(c, H, rho_, n, H);
            T y = alloc(c, {L, (long long)n}, false);
            gemm(c, false, false, L, n, n3, 1.0, Vd.p, n3, w2, n, 0.0, y.p, n);  // dp' W2
            rowdot_acc(c, y, H, q.p, c2);
            if (y3pre) {
                rowdot_acc(c, *y3pre, Vd, q.p, 1.0);
            } else {
                T y3 = alloc(c, {L, (long long)n3}, false);
                gemm(c, false, false, L, n3, n3, 1.0, Vd.p, n3, w3, n3, 0.0, y3.p, n3);
                rowdot_acc(c, y3, Vd, q.p, 1.0);
                if (y3keep) *y3keep = std::move(y3);
            }
            ck(cudaMemcpyAsync(out, q.p, sizeof(double) * L, cudaMemcpyDeviceToDevice, c.st), "cp");
        };
        T dumm = alloc(c, {L}, false), dumk = alloc(c, {L}, false);
        form3(rho.p, W2.p, 2.0, W3.p, dumm.p, pc ? &Yown : nullptr, nullptr);
        form3(Dm.p, Bc.p, 1.0, A.p, dumk.p, nullptr, nullptr);
        T dnj = stack_others(L, 1, [&](int j, double *out) {
            auto [P, lt] = off(j);
            T E2o = alloc(c, {n, n, n, n}, false), E3o = alloc(c, {n, n, n, n, n, n}, false);
            build_ee2L(c, P->d2.p, P->d1.p, n, E2o.p);
            build_eee2L(c, P->d3.p, P->d2.p, P->d1.p, n, E3o.p);
            T ro = alloc(c, {n, n}, false), W2o = alloc(c, {n, n, n, n}, false);
            T W3o = alloc(c, {n, n, n, n, n, n}, false);
            const T *e3src = &E3o;
            T E2a, E2b, E3t;
            if (minus) {
                // h daoff(a,ap) h (j<i) / daoff(ap,a): [ap,a]
                permute(c, P->d1.p, {n, n}, lt ? std::vector<int>{1, 0} : std::vector<int>{0, 1}, ro.p);
                permute(c, E2o.p, {n, n, n, n}, {1, 2, 0, 3}, W2o.p);           // ee2(cp,ap,bp,a)
                permute(c, E2o.p, {n, n, n, n}, {2, 1, 3, 0}, W2o.p, 1.0, true);  // + ee2(a,bp,ap,cp)
            } else {
                // -daoff(ap,a) (j<i) / -daoff(a,ap): [ap,a]
                permute(c, P->d1.p, {n, n}, lt ? std::vector<int>{0, 1} : std::vector<int>{1, 0}, ro.p, -1.0);
                E2a = alloc(c, {n, n, n, n}, false);
                E2b = alloc(c, {n, n, n, n}, false);
                build_ee2trL(c, E2o.p, P->d1.p, n, E2a.p);
                build_ee2tlL(c, E2o.p, P->d1.p, n, E2b.p);
                permute(c, E2a.p, {n, n, n, n}, {1, 2, 0, 3}, W2o.p);
                permute(c, E2b.p, {n, n, n, n}, {2, 1, 3, 0}, W2o.p, 1.0, true);
                E3t = alloc(c, {n, n, n, n, n, n}, false);
                build_eee2tL(c, E3o.p, E2o.p, n, E3t.p);
                e3src = &E3t;
            }
            // j<i: (cp,ap,bp,b,a,c); j>i: (c,a,b,bp,ap,cp) at [ap,bp,cp,a,b,c]
            if (lt) permute(c, e3src->p, {n, n, n, n, n, n}, {1, 2, 0, 4, 3, 5}, W3o.p);
            else permute(c, e3src->p, {n, n, n, n, n, n}, {4, 3, 5, 1, 2, 0}, W3o.p);
            form3(ro.p, W2o.p, 1.0, W3o.p, out, nullptr, pc ? &yoth[j] : nullptr);
        });
        std::vector<double> base(L);
        for (long long l = 0; l < L; ++l) base[l] = minus ? -eps[nc + na + l] : eps[l];
        auto res = sc_finish(dumm, dumk, base, dnj, 0);
        sc_store(minus ? 6 : 5, res);
        if (!pc) return;
        // ---- PC: metric S and Koopmans matrix K of order n^3 (formed above) ----
        T W2t = permuted(c, W2, {3, 0, 1, 2});                 // [a, (ap,bp,cp)]
        W2t = view2(std::move(W2t), n, n3);
        // Z[l, x] = (Vd S + H W2t)[l, x]: the numerators of the reference
        // before the change to the PC basis (R = Z C); Y = Vd S was formed above.
        auto zm = [&](const T &Y, const T &W2_, double *out) {
            ck(cudaMemcpyAsync(out, Y.p, sizeof(double) * L * n3, cudaMemcpyDeviceToDevice, c.st), "cp");
            gemm(c, false, false, L, n3, n, 1.0, H.p, n, W2_.p, n3, 1.0, out, n3);
        };
        // the same rows with the transition metric of another state j
        // The first term Vd S_j, with S_j the transition metric [(a,b,c),(ap,bp,cp)]
        // of eee2(c,a,b,bp,ap,cp) (j<i) / eee2(cp,ap,bp,b,a,c) (j>i) -- eee2t
        // for (+1') -- is the product kept from the SC form of state j.
        auto other_z = [&](int j, double *out) {
            auto [PD, lt] = off(j);
            T E2o = alloc(c, {n, n, n, n}, false);
            build_ee2L(c, PD->d2.p, PD->d1.p, n, E2o.p);
            T W2o = alloc(c, {n, n, n, n}, false);
            if (lt) {  // minus ee2(a,bp,ap,cp) / plus ee2tl(a,bp,ap,cp)
                if (minus) permute(c, E2o.p, {n, n, n, n}, {2, 1, 3, 0}, W2o.p);
                else {
                    T E2b = alloc(c, {n, n, n, n}, false);
                    build_ee2tlL(c, E2o.p, PD->d1.p, n, E2b.p);
                    permute(c, E2b.p, {n, n, n, n}, {2, 1, 3, 0}, W2o.p);
                }
            } else {   // minus ee2(cp,ap,bp,a) / plus ee2tr(cp,ap,bp,a)
                if (minus) permute(c, E2o.p, {n, n, n, n}, {1, 2, 0, 3}, W2o.p);
                else {
                    T E2a = alloc(c, {n, n, n, n}, false);
                    build_ee2trL(c, E2o.p, PD->d1.p, n, E2a.p);
                    permute(c, E2a.p, {n, n, n, n}, {1, 2, 0, 3}, W2o.p);
                }
            }
            T W2ot = permuted(c, W2o, {3, 0, 1, 2});
            W2ot = view2(std::move(W2ot), n, n3);
            zm(yoth.at(j), W2ot, out);
        };
        std::vector<double> pb(L);  // deno = w + eps_r  /  w - eps_i
        for (long long l = 0; l < L; ++l) pb[l] = -base[l];
        std::vector<double> e2(M * M, 0.0);
        double psi2 = 0.0;
        // compute_rho1st: vaux(d,mu) = sum_abc coef(mu,abc) g_d[abc] with g_d[abc] =
        // ee2(d,b,a,c) for (-1') (e2m1pcont :5326-5343, into rhodr) and ee2tl(d,b,a,c)
        // for (+1') (e21pcont :5113-5125, into rhoid); rho -= sum_mu c_mu vaux(d,mu)
        const int nd = acc.rho ? n : 0;
        T Ed;
        if (nd) {
            Ed = alloc(c, {(long long)n, (long long)n3}, false);
            if (minus) {
                permute(c, E2.p, {n, n, n, n}, {0, 2, 1, 3}, Ed.p);
            } else {
                T E2tl = alloc(c, {n, n, n, n}, false);
                build_ee2tlL(c, E2.p, D.g1.p, n, E2tl.p);
                permute(c, E2tl.p, {n, n, n, n}, {0, 2, 1, 3}, Ed.p);
            }
        }
        auto store_rho = [&](const std::vector<double> &rl) {
            for (long long l = 0; l < L; ++l)
                for (int d = 0; d < n; ++d) {
                    const double v = rl[(size_t)l * n + d];
                    if (minus) acc.rhodr[d + (size_t)na * (l + (size_t)nv * s)] += v;
                    else acc.rhoid[l + (size_t)nc * (d + (size_t)na * s)] += v;
                }
        };
        if (fork && fork->join()) {
            // Every metric eigenvalue is kept (nnew = n3): the PC sums over
            // the eigenpairs of K v = w S v are resolvents of the pencil,
            //   sum_mu r_mu^2 / (w_mu + s) = z^T (K + s S)^-1 z,
            // evaluated in the pencil's tridiagonal form (no eigenvectors).
            acc.nnew[(minus ? 7 : 6) + 10 * s] = (int)n3;
            // The QD cross terms and the densities need z_j^T x and g_d^T x
            // with x = (K + s S)^-1 z.  Mapping every z_j and g_d into the
            // tridiagonal basis costs M L + nd vector transforms; mapping the L
            // solutions back (x = U^-1 Q x~) and taking the dots in the original
            // basis costs 2 L.  The cheaper of the two is used.
            if (2 * L < (long long)M * L + nd) {
                T Zo = alloc(c, {L, (long long)n3}, false);
                zm(Yown, W2t, Zo.p);
                auto o = others();
                T Zx = alloc(c, {(long long)std::max<size_t>(o.size(), 1) * L, (long long)n3}, false);
                for (size_t k = 0; k < o.size(); ++k) other_z(o[k], Zx.p + (long long)k * L * n3);
                pencil_rhs(c, PT, Zo.p, L);
                T Yt = permuted(c, Zo, {1, 0});  // [n3][L]
                T Xt = alloc(c, {(long long)n3, L}, false);
                std::vector<double> r = resolvent_sums(PT, Yt, pb, 0, 0, nullptr, 0, Xt.p);
                T X = permuted(c, Xt, {1, 0});   // [L][n3]: the columns of a column-major [n3, L]
                pencil_back(c, PT, X.p, L);      // x = U^-1 Q x~
                if (!o.empty()) {
                    T a = alloc(c, {2 + 8}, true);
                    k_cross_dots<<<dim3((unsigned)std::min<long long>(nblk(L * n3), 1024), (unsigned)o.size()), TPB,
                                   0, c.st>>>(Zx.p, X.p, L, n3, a.p);
                    LAUNCHED();
                    auto cr = download(c, a.p, 2 + 8);
                    for (size_t k = 0; k < o.size(); ++k) r[2 + k] += cr[2 + k];
                }
                pc_accum(e2, psi2, r);
                if (nd) {  // rho[l, d] = -g_d . x_l
                    T rho = alloc(c, {L, (long long)nd}, false);
                    gemm(c, false, true, L, nd, n3, -1.0, X.p, n3, Ed.p, n3, 0.0, rho.p, nd);
                    store_rho(download(c, rho.p, L * nd));
                }
                pc_store(minus ? 6 : 5, e2, psi2, true);
                return;
            }
            // own state, then the others, then the nd density vectors g_d
            T Z = alloc(c, {(long long)M * L + nd, (long long)n3}, false);
            zm(Yown, W2t, Z.p);
            auto o = others();
            for (size_t k = 0; k < o.size(); ++k) other_z(o[k], Z.p + (long long)(k + 1) * L * n3);
            if (nd)
                ck(cudaMemcpyAsync(Z.p + (long long)M * L * n3, Ed.p, sizeof(double) * nd * n3,
                                   cudaMemcpyDeviceToDevice, c.st), "cp");
            // rows of Z are the columns of a column-major [n3, M L + nd]
            pencil_rhs(c, PT, Z.p, (long long)M * L + nd);
            Z = view2(std::move(Z), (long long)M * L + nd, n3);
            T Yt = permuted(c, Z, {1, 0});  // [n3][M L + nd]
            T rho = alloc(c, {L, (long long)(nd ? nd : 1)}, true);
            pc_accum(e2, psi2, resolvent_sums(PT, Yt, pb, nd, (long long)M * L, rho.p));
            if (nd) store_rho(download(c, rho.p, L * nd));
        } else {
            PcResult P = pc_transform(c, S, K, n3, thr);
            acc.nnew[(minus ? 7 : 6) + 10 * s] = P.nnew;
            // R[l, mu] = sum_x Z[l, x] C[x, mu]: the order-n3 products S C and
            // W2t C of the reference are reassociated onto the L rows.
            T Z = alloc(c, {L, (long long)n3}, false), R = alloc(c, {L, (long long)n3}, false);
            zm(Yown, W2t, Z.p);
            gemm(c, false, false, L, n3, n3, 1.0, Z.p, n3, P.C.p, n3, 0.0, R.p, n3);
            T Rj = stack_others(L, n3, [&](int j, double *out) {
                other_z(j, Z.p);
                gemm(c, false, false, L, n3, n3, 1.0, Z.p, n3, P.C.p, n3, 0.0, out, n3);
            });
            pc_accum(e2, psi2, pc_finish(R, nullptr, Rj, nullptr, P.w, pb, n3, 0));
            if (nd) {
                T V = alloc(c, {(long long)nd, (long long)n3}, false);
                gemm(c, false, false, nd, n3, n3, 1.0, Ed.p, n3, P.C.p, n3, 0.0, V.p, n3);
                store_rho(rho_pc(R, V, P.w, pb, n3, nd));
            }
        }
        pc_store(minus ? 6 : 5, e2, psi2, true);
    }
};  // class Runner

}  // namespace
}  // namespace s2
}  // namespace nvpt

// ===================================================================== C ABI
using namespace nvpt;
using namespace nvpt::s2;

namespace {

// Device copy of a host array (or a device array when on_device).
T stage_in(Ctx &c, const double *src, long long count, bool on_device) {
    T t = alloc(c, {count}, false);
    if (count > 0)
        ck(cudaMemcpyAsync(t.p, src, sizeof(double) * count, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                           c.st),
           "stage in");
    return t;
}

// C-ordered [i1..ik] slice `slot` of a Fortran (P, n, ..., n) array.
T fortran_slice(Ctx &c, const T &F, long long P, long long slot, int n, int k) {
    std::vector<long long> shape(k, n), stride(k);
    long long s = P;
    for (int i = 0; i < k; ++i) {
        stride[i] = s;
        s *= n;
    }
    T out = alloc_v(c, shape, false);
    gather(c, F.p, slot, shape, stride, out.p);
    return out;
}

struct ClassStreams {
    int dev = 0;
    std::vector<Ctx> c;
    std::vector<cudaEvent_t> done;
    cudaEvent_t prep = nullptr;
    explicit ClassStreams(size_t n) : done(n, nullptr) {
        ck(cudaGetDevice(&dev), "cudaGetDevice");
        c = CtxPool::acquire(n, dev);
        ck(cudaEventCreateWithFlags(&prep, cudaEventDisableTiming), "cudaEventCreate");
        for (size_t k = 0; k < n; ++k) ck(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming), "cudaEventCreate");
    }
    ~ClassStreams() {
        for (size_t k = 0; k < c.size(); ++k) {
            cudaStreamSynchronize(c[k].st);
            if (done[k]) cudaEventDestroy(done[k]);
        }
        if (prep) cudaEventDestroy(prep);
        for (auto &x : c) {
            x.split = false;
            x.oz_err = nullptr;
            x.sm_share = 1;
            x.wait_limit = 0;
            x.all_pc_resolvent = false;
        }
        CtxPool::release(c, dev);
    }
};

int run_qdnevpt(nvpt_context *ctx, cudaStream_t st, const nvpt_qdnevpt_in *in, nvpt_qdnevpt_out *out,
                bool on_device, std::string &err) {
    const int nc = (int)in->ncore, na = (int)in->nact, nv = (int)in->nvirt, M = (int)in->metat;
    const long long Q = in->nchovec;
    const int norb = nc + na + nv;
    if (na < 1 || na > 16 || nc < 0 || nv < 1 || M < 1 || M > 9 || Q < 1) {
        err = "qdnevpt: bad sizes (need 1 <= nact <= 16, nvirt >= 1, 1 <= metat <= 9)";
        return NVPT_EINVAL;
    }
    if (in->class_mask == 0) {
        err = "qdnevpt: empty class mask";
        return NVPT_EINVAL;
    }
    Ctx c{st, nullptr, nullptr};
    ck(cublasCreate(&c.blas), "cublasCreate");
    ck(cublasSetStream(c.blas, st), "cublasSetStream");
    ck(cusolverDnCreate(&c.sol), "cusolverDnCreate");
    ck(cusolverDnSetStream(c.sol, st), "cusolverDnSetStream");
    struct Handles {
        Ctx &c;
        ~Handles() {
            cublasDestroy(c.blas);
            cusolverDnDestroy(c.sol);
        }
    } guard{c};
    // split precision: the stage's large products run as Ozaki digit products
    c.split = nvpt_get_precision(ctx) == NVPT_PRECISION_SPLIT;
    T ozerr;
    if (c.split) {
        ozerr = alloc(c, {1}, true);
        c.oz_err = (int *)ozerr.p;
    }
    int n = na;
    long long n2 = (long long)n * n, n4 = n2 * n2, n6 = n4 * n2;
    long long npair = (long long)norb * (norb + 1) / 2;
    auto need = [&](const double *p, const char *name) {
        if (!p) throw Error(NVPT_EINVAL, std::string("qdnevpt: missing dataset ") + name);
    };
    need(in->oneint, "oneint"); need(in->cholesky_array, "cholesky_array");
    need(in->rdm1, "1-RDM"); need(in->rdm2, "2-RDM"); need(in->rdm3, "3-RDM"); need(in->hrdm2, "2-HRDM");
    need(in->ipko1, "1-IPKO"); need(in->eako1, "1-EAKO"); need(in->ipko2, "2-IPKO"); need(in->eako2, "2-EAKO");
    need(in->gk0pa, "gk0pa"); need(in->gk0pd, "gk0pd"); need(in->gk0pf, "gk0pf");
    bool four = (in->class_mask & 0x60) != 0;  // (+1') and (-1') need the A-D matrices
    if (four) {
        need(in->amat_ip, "amatIP"); need(in->amat_ea, "amatEA"); need(in->bmat_ip, "bmatIP");
        need(in->bmat_ea, "bmatEA"); need(in->cmat_ip, "cmatIP"); need(in->cmat_ea, "cmatEA");
        need(in->dmat_ip, "dmatIP"); need(in->dmat_ea, "dmatEA");
    }
    int P = M * (M - 1) / 2;
    if (P > 0) { need(in->trdm1, "1-TRDM"); need(in->trdm2, "2-TRDM"); need(in->trdm3, "3-TRDM"); }
    // stage inputs
    auto S = [&](const double *p, long long cnt) { return stage_in(c, p, cnt, on_device); };
    T F1 = S(in->rdm1, M * n2), F2 = S(in->rdm2, M * n4), F3 = S(in->rdm3, M * n6), FH = S(in->hrdm2, M * n4);
    T Fip1 = S(in->ipko1, M * n2), Fea1 = S(in->eako1, M * n2), Fip2 = S(in->ipko2, M * n4), Fea2 = S(in->eako2, M * n4);
    T Fa = S(in->gk0pa, M * n4), Fd = S(in->gk0pd, M * n4), Ff = S(in->gk0pf, M * n2);
    std::vector<StateData> sd(M);
    for (int s = 0; s < M; ++s) {
        StateData &D = sd[s];
        D.g1 = fortran_slice(c, F1, M, s, n, 2); D.g2 = fortran_slice(c, F2, M, s, n, 4);
        D.g3 = fortran_slice(c, F3, M, s, n, 6); D.hrdm = fortran_slice(c, FH, M, s, n, 4);
        D.ipko1 = fortran_slice(c, Fip1, M, s, n, 2); D.eako1 = fortran_slice(c, Fea1, M, s, n, 2);
        D.ipko2 = fortran_slice(c, Fip2, M, s, n, 4); D.eako2 = fortran_slice(c, Fea2, M, s, n, 4);
        D.gk0pa = fortran_slice(c, Fa, M, s, n, 4); D.gk0pd = fortran_slice(c, Fd, M, s, n, 4);
        D.gk0pf = fortran_slice(c, Ff, M, s, n, 2);
    }
    if (four) {
        const double *srcs[8] = {in->amat_ip, in->amat_ea, in->bmat_ip, in->bmat_ea,
                                 in->cmat_ip, in->cmat_ea, in->dmat_ip, in->dmat_ea};
        int ks[8] = {6, 6, 4, 4, 4, 4, 2, 2};
        for (int q = 0; q < 8; ++q) {
            long long cnt = M * (ks[q] == 6 ? n6 : ks[q] == 4 ? n4 : n2);
            T Fq = S(srcs[q], cnt);
            for (int s = 0; s < M; ++s) {
                T t = fortran_slice(c, Fq, M, s, n, ks[q]);
                StateData &D = sd[s];
                T *dst[8] = {&D.aIP, &D.aEA, &D.bIP, &D.bEA, &D.cIP, &D.cEA, &D.dIP, &D.dEA};
                *dst[q] = std::move(t);
            }
        }
    }
    std::vector<PairData> pd(P);
    if (P > 0) {
        T T1 = S(in->trdm1, P * n2), T2 = S(in->trdm2, P * n4), T3 = S(in->trdm3, P * n6);
        for (int k = 0; k < P; ++k) {
            pd[k].d1 = fortran_slice(c, T1, P, k, n, 2);
            pd[k].d2 = fortran_slice(c, T2, P, k, n, 4);
            pd[k].d3 = fortran_slice(c, T3, P, k, n, 6);
        }
    }
    // compute_rho1st: the first-order density blocks when the caller asks for them
    const bool want_rho = out->rhoir || out->rhoid || out->rhodr;
    Accum acc(M, nc, na, nv, want_rho);
    Runner R(c, nc, na, nv, M, Q, in->thr_lindep, in->frozen, sd, pd, acc);
    {
        T chol = S(in->cholesky_array, Q * npair);
        R.B = alloc(c, {Q, norb, norb}, false);
        k_unpack_B<<<nblk(Q * norb * norb), TPB, 0, c.st>>>(chol.p, Q, norb, R.B.p);
        LAUNCHED();
        T one = S(in->oneint, npair);
        R.h = alloc(c, {norb, norb}, false);
        k_unpack_tri<<<nblk((long long)norb * norb), TPB, 0, c.st>>>(one.p, norb, R.h.p);
        LAUNCHED();
    }
    bool pc = !in->no_pc;
    std::vector<double> epsnew((size_t)norb * M, 0.0);
    unsigned m = (unsigned)in->class_mask;
    // The classes of one state only read the state's orbitals and integrals,
    // so each runs on its own stream, handles and host thread; their
    // accumulators are merged afterwards in the reference's class order
    // (0, +1, -1, +2, -2, 0', -1', +1').
    using Job = std::function<void(Runner &)>;
    std::vector<Job> jobs;
    std::vector<const char *> tags;  // live-timing tags (nvpt_profile_read)
    if (m & 1u) { jobs.push_back([](Runner &r) { r.class0(); }); tags.push_back("s2_class_0"); }
    if (m & 2u) { jobs.push_back([pc](Runner &r) { r.class_pm1(true, pc); }); tags.push_back("s2_class_+1"); }
    if (m & 4u) { jobs.push_back([pc](Runner &r) { r.class_pm1(false, pc); }); tags.push_back("s2_class_-1"); }
    if (m & 8u) { jobs.push_back([pc](Runner &r) { r.class_pm2(true, pc); }); tags.push_back("s2_class_+2"); }
    if (m & 16u) { jobs.push_back([pc](Runner &r) { r.class_pm2(false, pc); }); tags.push_back("s2_class_-2"); }
    if (m & 128u) { jobs.push_back([pc](Runner &r) { r.class0p(pc); }); tags.push_back("s2_class_0p"); }
    if (m & 64u) { jobs.push_back([pc](Runner &r) { r.class_pm1p(true, pc); }); tags.push_back("s2_class_+1p"); }
    if (m & 32u) { jobs.push_back([pc](Runner &r) { r.class_pm1p(false, pc); }); tags.push_back("s2_class_-1p"); }
    const size_t nj = jobs.size();
    // The states are independent too: every state is prepared on its own
    // stream, then every (state, class) pair runs concurrently.  The
    // accumulators are merged state by state in the reference's class order.
    int dev = 0;
    ck(cudaGetDevice(&dev), "cudaGetDevice");
    ClassStreams ps((size_t)M), cs((size_t)M * nj);
    // order-n^3 pencils in flight at once: one per state and (+-1') class
    const int pencils = M * (((m & 64u) ? 1 : 0) + ((m & 32u) ? 1 : 0));
    for (auto *pool : {&ps, &cs})
        for (auto &pc_ : pool->c) {
            pc_.split = c.split;
            pc_.oz_err = c.oz_err;
            // measured: 8 pencils (4 states) fastest on quarters; 2 pencils on the whole GPU each
            pc_.sm_share = pc && pencils >= 4 ? 4 : 1;
            pc_.wait_limit = nvpt_context_wait_limit(ctx);
            pc_.all_pc_resolvent = nvpt_context_pc_route(ctx) == 1;
        }
    ck(cudaEventRecord(ps.prep, c.st), "event");  // B and h ready
    std::vector<std::unique_ptr<Runner>> SR(M);
    {
        std::vector<std::exception_ptr> fail(M);
        auto prep = [&](int st_) {
            try {
                ck(cudaSetDevice(dev), "cudaSetDevice");
                ck(cudaStreamWaitEvent(ps.c[st_].st, ps.prep, 0), "wait");
                SR[st_].reset(new Runner(R, ps.c[st_], acc));
                ProfSpan span;
                span.begin("s2_prepare", ps.c[st_].st, 0);
                SR[st_]->prepare_state(st_);
                span.end();
            } catch (...) {
                fail[st_] = std::current_exception();
            }
            cudaEventRecord(ps.done[st_], ps.c[st_].st);
        };
        std::vector<std::thread> th;
        for (int st_ = 1; st_ < M; ++st_) th.emplace_back(prep, st_);
        prep(0);
        for (auto &t : th) t.join();
        for (int st_ = 0; st_ < M; ++st_)
            if (fail[st_]) std::rethrow_exception(fail[st_]);
    }
    for (int st_ = 0; st_ < M; ++st_)
        for (int k = 0; k < norb; ++k) epsnew[k + (size_t)norb * st_] = SR[st_]->eps[k];
    {
        const size_t nt = (size_t)M * nj;
        std::vector<Accum> local(nt, Accum(M, nc, na, nv, want_rho));
        std::vector<std::exception_ptr> fail(nt);
        auto work = [&](size_t idx) {
            const size_t st_ = idx / nj, k = idx % nj;
            try {
                ck(cudaSetDevice(dev), "cudaSetDevice");
                ck(cudaStreamWaitEvent(cs.c[idx].st, ps.done[st_], 0), "wait");
                Runner W(*SR[st_], cs.c[idx], local[idx]);
                ProfSpan span;
                span.begin(tags[k], cs.c[idx].st, 0);
                jobs[k](W);
                span.end();
            } catch (...) {
                fail[idx] = std::current_exception();
            }
            cudaEventRecord(cs.done[idx], cs.c[idx].st);
        };
        std::vector<std::thread> th;
        for (size_t idx = 1; idx < nt; ++idx) th.emplace_back(work, idx);
        if (nt) work(0);
        for (auto &t : th) t.join();
        for (size_t idx = 0; idx < nt; ++idx) {
            ck(cudaStreamWaitEvent(c.st, cs.done[idx], 0), "wait");
            // the state tensors are freed on their prepare stream: after their readers
            ck(cudaStreamWaitEvent(ps.c[idx / nj].st, cs.done[idx], 0), "wait");
        }
        for (size_t idx = 0; idx < nt; ++idx)
            if (fail[idx]) std::rethrow_exception(fail[idx]);
        for (size_t idx = 0; idx < nt; ++idx) acc.merge(local[idx]);
    }
    SR.clear();
    ck(cudaStreamSynchronize(c.st), "qdnevpt sync");
    if (c.split) {
        int h = 0;
        ck(cudaMemcpy(&h, c.oz_err, sizeof(int), cudaMemcpyDeviceToHost), "error flag");
        if (h) {
            err = "qdnevpt: a split-precision product timed out waiting on its pipeline";
            return NVPT_ETIMEDOUT;
        }
    }
    auto put = [](double *dst, const std::vector<double> &v) {
        if (dst) std::memcpy(dst, v.data(), sizeof(double) * v.size());
    };
    put(out->e2mpp, acc.e2mpp); put(out->psimpp, acc.psimpp); put(out->e2enp, acc.e2enp);
    put(out->psienep, acc.psienep); put(out->e2mp, acc.e2mp); put(out->e2en, acc.e2en);
    put(out->psimp, acc.psimp); put(out->psien, acc.psien); put(out->epsnew, epsnew);
    if (out->nnew) std::memcpy(out->nnew, acc.nnew.data(), sizeof(int64_t) * acc.nnew.size());
    if (want_rho) {
        put(out->rhoir, acc.rhoir); put(out->rhoid, acc.rhoid); put(out->rhodr, acc.rhodr);
    }
    return NVPT_OK;
}

}  // namespace

extern "C" const char *nvpt_context_error_set(nvpt_context *ctx, const char *msg);
extern "C" void *nvpt_context_stream(nvpt_context *ctx);

extern "C" int nvpt_qdnevpt(nvpt_context *ctx, const nvpt_qdnevpt_in *in, nvpt_qdnevpt_out *out) {
    if (!ctx || !in || !out) return NVPT_EINVAL;
    std::string err;
    try {
        int rc = run_qdnevpt(ctx, (cudaStream_t)nvpt_context_stream(ctx), in, out, false, err);
        if (rc != NVPT_OK) nvpt_context_error_set(ctx, err.c_str());
        return rc;
    } catch (const Error &e) {
        nvpt_context_error_set(ctx, e.what());
        return e.code == 3 ? NVPT_ENOMEM : e.code == 4 ? NVPT_ETIMEDOUT : (e.code == NVPT_EINVAL ? NVPT_EINVAL : NVPT_ECUDA);
    }
}

extern "C" int nvpt_qdnevpt_d(nvpt_context *ctx, const nvpt_qdnevpt_in *in, nvpt_qdnevpt_out *out, void *stream) {
    if (!ctx || !in || !out) return NVPT_EINVAL;
    std::string err;
    try {
        cudaStream_t st = stream ? (cudaStream_t)stream : (cudaStream_t)nvpt_context_stream(ctx);
        int rc = run_qdnevpt(ctx, st, in, out, true, err);
        if (rc != NVPT_OK) nvpt_context_error_set(ctx, err.c_str());
        return rc;
    } catch (const Error &e) {
        nvpt_context_error_set(ctx, e.what());
        return e.code == 3 ? NVPT_ENOMEM : e.code == 4 ? NVPT_ETIMEDOUT : (e.code == NVPT_EINVAL ? NVPT_EINVAL : NVPT_ECUDA);
    }
}
