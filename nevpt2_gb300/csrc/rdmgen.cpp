// Exact spin-free reduced density matrices of a determinant-expanded CI
// vector, written in the layouts the Koopmans/NEVPT2 path consumes.
//
// This is the synthetic-input generator.  It replaces the reference's
// CI-vector builders (src/koopro4QD.F90:921-3013 rofour / ro3 / ro2 / ro1 and
// the *off transition variants) with a different algorithm:
//
//   Gamma_k(P;Q) = sum_sigma < Phi_{P,sigma} | Phi_{Q,sigma} >,
//   |Phi_{q}> = a_{q_k} ... a_{q_1} |Psi>,
//
// i.e. every k-RDM is a Gram matrix of k-fold annihilated vectors.  The
// spin-orbital Gram blocks D_r (r = number of alpha annihilations) are built
// exactly from the sparse annihilation images grouped by the (N-k)-electron
// determinant they land on, then folded into the spin-free tensors:
//   Gamma_k(P;Q) = sum_{sigma in {a,b}^k} sgn(p) sgn(q) D_r(sort p, sort q),
//   p_m = (P_m, sigma_m), q_m = (Q_m, sigma_m).
//
// Conventions (identical to the reference's arrays):
//   dal(s,i,j)          = <E_ij>
//   taa(s,i,j,k,l)      = sum <a+_i a+_j a_l a_k>      (pairs i-k, j-l)
//   daaa(s,i,j,k,l,m,n) = sum <a+_i a+_j a+_k a_n a_m a_l>
//   ro4(ind,L1..L4,s)   = Gamma_4(K;L) with K the descending-sorted key
//                         quadruple, ind = lindice(K), src/indices_norm.F90:64
//   all Fortran column-major, state index first (ro4: state last).
// Transition matrices use bra = root `s`, ket = root `t`.
//
// Spin orbitals: alpha orbital p -> bit p, beta orbital p -> bit n+p; a
// determinant is the ordered product a+_{i1} ... a+_{iN}|0> with ascending
// spin-orbital indices.  n <= 16 (2n <= 32 bits).
#include <algorithm>
#include <numeric>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
#endif

namespace {

typedef int64_t I;

I binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    I r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

struct Binom {
    I t[40][40];
    Binom() {
        for (int n = 0; n < 40; ++n)
            for (int k = 0; k < 40; ++k) t[n][k] = binom(n, k);
    }
};
const Binom BIN;

// colex rank of an ascending 0-based subset
inline I subset_rank(const int *x, int r) {
    I s = 0;
    for (int j = 0; j < r; ++j) s += BIN.t[x[j]][j + 1];
    return s;
}

inline I mask_rank(uint32_t m, int n) {
    I s = 0;
    int j = 0;
    for (int p = 0; p < n; ++p)
        if (m >> p & 1u) { s += BIN.t[p][j + 1]; ++j; }
    return s;
}

inline int popc(uint32_t x) { return __builtin_popcount(x); }

// A zero-filled buffer whose pages are first touched by all threads (the
// Gram blocks reach 1.7 GB at n = 16; a serial fill costs a second).
struct ZeroBuf {
    double *p;
    explicit ZeroBuf(size_t count) : p(new double[count]) {
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)count; ++i) p[i] = 0.0;
    }
    ~ZeroBuf() { delete[] p; }
    ZeroBuf(const ZeroBuf &) = delete;
    ZeroBuf &operator=(const ZeroBuf &) = delete;
    double *data() { return p; }
};

struct Entry {
    uint64_t key;   // (xid << 24) | S
    int32_t det;    // +-(det+1): sign of the annihilation string
    int32_t pad;
};

// One spin block: k annihilations, r of them alpha.
struct Block {
    int n, k, r;
    I dimA, dimB, dim;  // C(n,r), C(n,k-r), product
};

// Build the Gram block D (dim x dim) for bra root s and ket root t.
// coef is (ndet x nroot) column-major.
void gram_block(const Block &blk, I ndet, const uint32_t *amask, const uint32_t *bmask, const double *coef,
                int s, int t, double *D) {
    const int n = blk.n, k = blk.k, r = blk.r;
    std::vector<Entry> ent;
    // count entries
    std::vector<I> cnt(ndet + 1, 0);
    for (I I0 = 0; I0 < ndet; ++I0) cnt[I0 + 1] = BIN.t[popc(amask[I0])][r] * BIN.t[popc(bmask[I0])][k - r];
    for (I I0 = 0; I0 < ndet; ++I0) cnt[I0 + 1] += cnt[I0];
    ent.resize(cnt[ndet]);
    if (ent.empty()) return;
#pragma omp parallel for schedule(dynamic, 64)
    for (I I0 = 0; I0 < ndet; ++I0) {
        uint32_t am = amask[I0], bm = bmask[I0];
        int aocc[32], bocc[32], na = 0, nb = 0;
        for (int p = 0; p < n; ++p) if (am >> p & 1u) aocc[na++] = p;
        for (int p = 0; p < n; ++p) if (bm >> p & 1u) bocc[nb++] = p;
        I pos = cnt[I0];
        // enumerate r-subsets of aocc (indices into aocc) and (k-r)-subsets of bocc
        int ia[8], ib[8];
        for (int j = 0; j < r; ++j) ia[j] = j;
        bool amore = (r <= na);
        while (amore) {
            for (int j = 0; j < k - r; ++j) ib[j] = j;
            bool bmore = (k - r <= nb);
            while (bmore) {
                // spin orbitals ascending: alpha part then beta part
                uint32_t xa = am, xb = bm;
                int sorbs[8], cntbelow = 0, sgnexp = 0;
                int asub[8], bsub[8];
                for (int j = 0; j < r; ++j) {
                    int p = aocc[ia[j]];
                    asub[j] = p;
                    xa &= ~(1u << p);
                    sorbs[j] = p;
                    cntbelow = ia[j];  // occupied alphas below p
                    sgnexp += cntbelow - j;
                }
                for (int j = 0; j < k - r; ++j) {
                    int p = bocc[ib[j]];
                    bsub[j] = p;
                    xb &= ~(1u << p);
                    sorbs[r + j] = n + p;
                    cntbelow = na + ib[j];
                    sgnexp += cntbelow - (r + j);
                }
                (void)sorbs;
                I S = subset_rank(asub, r) * blk.dimB + subset_rank(bsub, k - r);
                I xid = mask_rank(xa, n) * BIN.t[n][nb - (k - r)] + mask_rank(xb, n);
                Entry e;
                e.key = ((uint64_t)xid << 24) | (uint64_t)S;
                e.det = (sgnexp & 1) ? -(int32_t)(I0 + 1) : (int32_t)(I0 + 1);
                e.pad = 0;
                ent[pos++] = e;
                // next beta subset
                int j = k - r - 1;
                while (j >= 0 && ib[j] == nb - (k - r) + j) --j;
                if (j < 0) bmore = false;
                else { ++ib[j]; for (int m = j + 1; m < k - r; ++m) ib[m] = ib[m - 1] + 1; }
            }
            int j = r - 1;
            while (j >= 0 && ia[j] == na - r + j) --j;
            if (j < 0) amore = false;
            else { ++ia[j]; for (int m = j + 1; m < r; ++m) ia[m] = ia[m - 1] + 1; }
        }
    }
    // keys are unique (one entry per source determinant and annihilation
    // set), so any sort gives the same order
#ifdef _OPENMP
    __gnu_parallel::sort(ent.begin(), ent.end(), [](const Entry &a, const Entry &b) { return a.key < b.key; });
#else
    std::sort(ent.begin(), ent.end(), [](const Entry &a, const Entry &b) { return a.key < b.key; });
#endif
    // groups by xid (a group starts where xid changes), then the entries
    // bucketed by S, ascending e inside a bucket, for a race-free,
    // deterministic row-parallel update.  Both passes run over contiguous
    // chunks of the entries: per-chunk counts, an exclusive scan over the
    // chunks, then each chunk writes its own part -- the same arrays a
    // sequential pass would produce.
    const I ne = (I)ent.size();
    const int nch = std::max(1, std::min(256, (int)(ne / 65536) + 1));
    auto chunk_lo = [&](int c) { return ne * c / nch; };
    std::vector<I> heads(nch + 1, 0);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nch; ++c) {
        I h = 0;
        for (I e = chunk_lo(c); e < chunk_lo(c + 1); ++e)
            if (e == 0 || (ent[e].key >> 24) != (ent[e - 1].key >> 24)) ++h;
        heads[c + 1] = h;
    }
    for (int c = 0; c < nch; ++c) heads[c + 1] += heads[c];
    std::vector<I> gstart((size_t)heads[nch] + 1);
    std::vector<I> gid(ne);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nch; ++c) {
        I g = heads[c] - 1;
        for (I e = chunk_lo(c); e < chunk_lo(c + 1); ++e) {
            if (e == 0 || (ent[e].key >> 24) != (ent[e - 1].key >> 24)) gstart[++g] = e;
            gid[e] = g;
        }
    }
    gstart[heads[nch]] = ne;
    // counting sort by S: per-chunk histograms, bucket starts, chunk offsets
    const I dim = blk.dim;
    std::vector<I> hist((size_t)nch * dim, 0);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nch; ++c) {
        I *hc = hist.data() + (size_t)c * dim;
        for (I e = chunk_lo(c); e < chunk_lo(c + 1); ++e) hc[ent[e].key & 0xFFFFFFull]++;
    }
    std::vector<I> sstart(dim + 1, 0);
    for (I q = 0; q < dim; ++q) {
        I acc = sstart[q];
        for (int c = 0; c < nch; ++c) {  // hist becomes each chunk's write offset in bucket q
            const I h = hist[(size_t)c * dim + q];
            hist[(size_t)c * dim + q] = acc;
            acc += h;
        }
        sstart[q + 1] = acc;
    }
    std::vector<I> sorder(ne);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < nch; ++c) {
        I *off = hist.data() + (size_t)c * dim;
        for (I e = chunk_lo(c); e < chunk_lo(c + 1); ++e) sorder[off[ent[e].key & 0xFFFFFFull]++] = e;
    }
    auto val = [&](I e, int root) {
        int32_t d = ent[e].det;
        I det = (d > 0 ? d : -d) - 1;
        double v = coef[det + ndet * root];
        return d > 0 ? v : -v;
    };
#pragma omp parallel for schedule(dynamic, 16)
    for (I S = 0; S < blk.dim; ++S) {
        double *row = D + S * blk.dim;
        for (I q = sstart[S]; q < sstart[S + 1]; ++q) {
            I e = sorder[q];
            double vs = val(e, s);
            if (vs == 0.0) continue;
            I g = gid[e];
            for (I f = gstart[g]; f < gstart[g + 1]; ++f) row[ent[f].key & 0xFFFFFFull] += vs * val(f, t);
        }
    }
}

// Map an orbital tuple with spins to (rank within its block, sign); returns
// false if two entries coincide.  spins: bit m set = beta.
inline bool spin_tuple_rank(const int *orb, unsigned spins, int k, int r, I dimB, I *rank, int *sgn) {
    // spin-orbital indices
    int so[8];
    for (int m = 0; m < k; ++m) so[m] = orb[m] + ((spins >> m & 1u) ? 64 : 0);
    // insertion sort with parity
    int par = 0;
    for (int i = 1; i < k; ++i) {
        int v = so[i], j = i - 1;
        while (j >= 0 && so[j] > v) { so[j + 1] = so[j]; --j; ++par; }
        so[j + 1] = v;
    }
    for (int i = 1; i < k; ++i)
        if (so[i] == so[i - 1]) return false;
    int a[8], b[8];
    for (int i = 0; i < r; ++i) a[i] = so[i];
    for (int i = 0; i < k - r; ++i) b[i] = so[r + i] - 64;
    *rank = subset_rank(a, r) * dimB + subset_rank(b, k - r);
    *sgn = (par & 1) ? -1 : 1;
    return true;
}

inline I lind(int i1, int i2, int i3, int i4) {  // 1-based descending quadruple
    return (I)(i1 - 1) * i1 * (i1 + 1) * (i1 + 2) / 24 + (I)(i2 - 1) * i2 * (i2 + 1) / 6 + (I)(i3 - 1) * i3 / 2 + i4;
}

inline I normind(int a, int b, int c, int d) {
    int v[4] = {a, b, c, d};
    std::sort(v, v + 4, [](int x, int y) { return x > y; });
    return lind(v[0], v[1], v[2], v[3]);
}

}  // namespace

extern "C" {

// Dense spin-free k-RDM (k = 1, 2, 3) for the (bra s, ket t) root pair,
// accumulated into out at stride `ldo` over the pair index `slot`:
// out[slot + ldo*(P1 + n P2 + ... + n^{2k-1} Q_k)] with P = upper, Q = lower
// indices in the reference's (P..., Q...) argument order.
int rdmgen_dense(int n, int k, long ndet, const uint32_t *amask, const uint32_t *bmask, const double *coef,
                 int s, int t, double *out, long ldo, long slot) {
    if (n < 1 || n > 16 || k < 1 || k > 3) return 1;
    I nk = 1;
    for (int i = 0; i < k; ++i) nk *= n;
    for (int r = 0; r <= k; ++r) {
        Block blk{n, k, r, BIN.t[n][r], BIN.t[n][k - r], BIN.t[n][r] * BIN.t[n][k - r]};
        ZeroBuf D((size_t)(blk.dim * blk.dim));
        gram_block(blk, ndet, amask, bmask, coef, s, t, D.data());
        // (rank, sign) of every index tuple under every spin pattern of this block
        const unsigned nsp = 1u << k;
        std::vector<int32_t> trk((size_t)nsp * nk, -1);
        std::vector<int8_t> tsg((size_t)nsp * nk, 0);
#pragma omp parallel for schedule(static)
        for (I Q = 0; Q < nk; ++Q) {
            int qo[4];
            I y = Q;
            for (int m = 0; m < k; ++m) { qo[m] = (int)(y % n); y /= n; }
            for (unsigned sp = 0; sp < nsp; ++sp) {
                if (k - popc(sp) != r) continue;
                I Trank;
                int sg2;
                if (!spin_tuple_rank(qo, sp, k, r, blk.dimB, &Trank, &sg2)) continue;
                trk[sp * nk + Q] = (int32_t)Trank;
                tsg[sp * nk + Q] = (int8_t)sg2;
            }
        }
#pragma omp parallel for schedule(dynamic, 4)
        for (I P = 0; P < nk; ++P) {
            for (unsigned sp = 0; sp < nsp; ++sp) {
                const int32_t Srank = trk[sp * nk + P];
                if (Srank < 0) continue;
                const int sg1 = tsg[sp * nk + P];
                const double *row = D.data() + (I)Srank * blk.dim;
                const int32_t *tr = trk.data() + sp * nk;
                const int8_t *ts = tsg.data() + sp * nk;
                for (I Q = 0; Q < nk; ++Q) {
                    if (tr[Q] < 0) continue;
                    double v = row[tr[Q]];
                    if (v == 0.0) continue;
                    out[slot + ldo * (P + nk * Q)] += (sg1 * ts[Q]) * v;
                }
            }
        }
    }
    return 0;
}

// Packed spin-free 4-RDM of root s into ro4_s (W x n^4 block of one state),
// filling every slot (K descending, L) with normind(L) <= normind(K); the
// remaining slots are never addressed by ord8 and stay as they are.
int rdmgen_ro4(int n, long ndet, const uint32_t *amask, const uint32_t *bmask, const double *coef, int s,
               double *ro4_s) {
    if (n < 1 || n > 16) return 1;
    const int k = 4;
    const I W = (I)n * (n + 1) * (n + 2) * (n + 3) / 24;
    // list of descending keys
    std::vector<int> keys;
    for (int i1 = 1; i1 <= n; ++i1)
        for (int i2 = 1; i2 <= i1; ++i2)
            for (int i3 = 1; i3 <= i2; ++i3)
                for (int i4 = 1; i4 <= i3; ++i4) {
                    keys.push_back(i1); keys.push_back(i2); keys.push_back(i3); keys.push_back(i4);
                }
    const I nkeys = (I)keys.size() / 4;
    const I n4 = (I)n * n * n * n;
    std::vector<I> nm(n4);
    for (I L = 0; L < n4; ++L) {
        I y = L;
        int q[4];
        for (int m = 0; m < 4; ++m) { q[m] = (int)(y % n) + 1; y /= n; }
        nm[L] = normind(q[0], q[1], q[2], q[3]);
    }
    // L in ascending normind order; the slots of key `ind` are the first
    // upto[ind] of them
    std::vector<I> lord(n4);
    std::iota(lord.begin(), lord.end(), (I)0);
    std::stable_sort(lord.begin(), lord.end(), [&](I a, I b) { return nm[a] < nm[b]; });
    std::vector<I> upto(W + 1, 0);
    for (I L = 0; L < n4; ++L) upto[nm[L]]++;
    for (I v = 1; v <= W; ++v) upto[v] += upto[v - 1];
    std::vector<int32_t> trk((size_t)16 * n4);
    std::vector<int8_t> tsg((size_t)16 * n4);
    for (int r = 0; r <= k; ++r) {
        Block blk{n, k, r, BIN.t[n][r], BIN.t[n][k - r], BIN.t[n][r] * BIN.t[n][k - r]};
        ZeroBuf D((size_t)(blk.dim * blk.dim));
        gram_block(blk, ndet, amask, bmask, coef, s, s, D.data());
        // (rank, sign) of every L under every spin pattern of this block
#pragma omp parallel for schedule(static)
        for (I L = 0; L < n4; ++L) {
            I y = L;
            int q[4];
            for (int m = 0; m < 4; ++m) { q[m] = (int)(y % n); y /= n; }
            for (unsigned sp = 0; sp < 16u; ++sp) {
                I Trank;
                int sg2;
                const bool ok = (k - popc(sp) == r) && spin_tuple_rank(q, sp, k, r, blk.dimB, &Trank, &sg2);
                trk[sp * n4 + L] = ok ? (int32_t)Trank : -1;
                tsg[sp * n4 + L] = ok ? (int8_t)sg2 : 0;
            }
        }
#pragma omp parallel for schedule(dynamic, 8)
        for (I kk = 0; kk < nkeys; ++kk) {
            int K[4] = {keys[4 * kk] - 1, keys[4 * kk + 1] - 1, keys[4 * kk + 2] - 1, keys[4 * kk + 3] - 1};
            I ind = lind(K[0] + 1, K[1] + 1, K[2] + 1, K[3] + 1);
            const I lim = upto[ind];
            for (unsigned sp = 0; sp < 16u; ++sp) {
                if (k - popc(sp) != r) continue;
                I Srank;
                int sg1;
                if (!spin_tuple_rank(K, sp, k, r, blk.dimB, &Srank, &sg1)) continue;
                const double *row = D.data() + Srank * blk.dim;
                const int32_t *tr = trk.data() + sp * n4;
                const int8_t *ts = tsg.data() + sp * n4;
                for (I i = 0; i < lim; ++i) {
                    const I L = lord[i];
                    if (tr[L] < 0) continue;
                    double v = row[tr[L]];
                    if (v == 0.0) continue;
                    ro4_s[(ind - 1) + W * L] += (sg1 * ts[L]) * v;
                }
            }
        }
    }
    return 0;
}

int rdmgen_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
