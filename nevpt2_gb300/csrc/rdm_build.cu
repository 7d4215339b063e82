// Spin-free 1-4-RDMs of a determinant-expanded CI vector on the device: the
// role of the reference's CI-vector builders (src/koopro4QD.F90:921-1569
// rofour, :1571 ro3, :2412 ro2, :2861 ro1 and the *off transition variants
// :1978, :2620, :2936), computed as Gram matrices of annihilated vectors:
//
//   Gamma_k(P;Q) = sum_sigma < Phi_{P,sigma} | Phi_{Q,sigma} >,
//   |Phi_q> = a_{q_k} ... a_{q_1} |Psi>.
//
// Per spin block (k annihilations, r of them alpha) every determinant emits
// one entry per choice of r occupied alpha and k-r occupied beta orbitals:
// the (N-k)-electron determinant it lands on (xid), the annihilated set's
// rank S within the block and the sign of the annihilation string.  The
// entries are sorted by (xid, S) (device radix sort); entries of one xid form
// a group and every pair in a group adds c_bra(e) c_ket(f) to D[S_e, S_f]
// (FP64 atomics).  The spin-free tensors are then gathered from D with the
// (rank, sign) of every orbital tuple under every spin pattern.
//
// Conventions (those of the reference's arrays): dal(s,i,j) = <E_ij>;
// taa(s,i,j,k,l) = sum <a+_i a+_j a_l a_k>; daaa(s,i,j,k,l,m,n) =
// sum <a+_i a+_j a+_k a_n a_m a_l>; ro4(ind,L1..L4,s) = Gamma_4(K;L) with K
// the descending-sorted key quadruple, ind = lindice(K) (src/indices_norm.F90
// :64), filled for normind(L) <= normind(K) (the slots ord8 addresses).
// Spin orbitals: alpha p -> bit p, beta p -> bit n+p; a determinant is the
// product of creators in ascending spin-orbital order.  n <= 16.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <vector>

#include "nvpt2_internal.h"

namespace nvpt {
namespace {

__constant__ long long c_binom[33][33];

struct BinomHost {
    long long t[33][33];
    BinomHost() {
        for (int n = 0; n < 33; ++n)
            for (int k = 0; k < 33; ++k) {
                long long r = (k < 0 || k > n) ? 0 : 1;
                for (int i = 1; i <= k && r; ++i) r = r * (n - k + i) / i;
                t[n][k] = r;
            }
    }
};

__device__ __forceinline__ long long subset_rank(const int *x, int r) {  // colex rank, ascending 0-based
    long long s = 0;
    for (int j = 0; j < r; ++j) s += c_binom[x[j]][j + 1];
    return s;
}
__device__ __forceinline__ long long mask_rank(unsigned m, int n) {
    long long s = 0;
    int j = 0;
    for (int p = 0; p < n; ++p)
        if (m >> p & 1u) s += c_binom[p][++j];
    return s;
}

// entries per determinant: C(na, r) C(nb, k - r)
__global__ void k_entry_counts(const unsigned *amask, const unsigned *bmask, long long ndet, int k, int r,
                               long long *cnt) {
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= ndet) return;
    cnt[I] = c_binom[__popc(amask[I])][r] * c_binom[__popc(bmask[I])][k - r];
}

// One thread per determinant: its annihilation images, key = xid << 24 | S,
// value = +-(I + 1) (sign of the annihilation string).
__global__ void k_entries(const unsigned *amask, const unsigned *bmask, long long ndet, int n, int k, int r,
                          long long dimB, const long long *off, unsigned long long *key, int *val) {
    const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= ndet) return;
    const unsigned am = amask[I], bm = bmask[I];
    int aocc[16], bocc[16], na = 0, nb = 0;
    for (int p = 0; p < n; ++p) {
        if (am >> p & 1u) aocc[na++] = p;
        if (bm >> p & 1u) bocc[nb++] = p;
    }
    if (r > na || k - r > nb) return;
    long long pos = off[I];
    const long long nbt = c_binom[n][nb - (k - r)];
    int ia[4], ib[4];
    for (int j = 0; j < r; ++j) ia[j] = j;
    for (bool amore = true; amore;) {
        for (int j = 0; j < k - r; ++j) ib[j] = j;
        for (bool bmore = true; bmore;) {
            unsigned xa = am, xb = bm;
            int sgnexp = 0, asub[4], bsub[4];
            for (int j = 0; j < r; ++j) {
                const int p = aocc[ia[j]];
                asub[j] = p;
                xa &= ~(1u << p);
                sgnexp += ia[j] - j;  // occupied spin orbitals below p, less those already removed
            }
            for (int j = 0; j < k - r; ++j) {
                const int p = bocc[ib[j]];
                bsub[j] = p;
                xb &= ~(1u << p);
                sgnexp += na + ib[j] - (r + j);
            }
            const long long S = subset_rank(asub, r) * dimB + subset_rank(bsub, k - r);
            const long long xid = mask_rank(xa, n) * nbt + mask_rank(xb, n);
            key[pos] = ((unsigned long long)xid << 24) | (unsigned long long)S;
            val[pos] = (sgnexp & 1) ? -(int)(I + 1) : (int)(I + 1);
            ++pos;
            int j = k - r - 1;
            while (j >= 0 && ib[j] == nb - (k - r) + j) --j;
            if (j < 0) bmore = false;
            else {
                ++ib[j];
                for (int m = j + 1; m < k - r; ++m) ib[m] = ib[m - 1] + 1;
            }
        }
        int j = r - 1;
        while (j >= 0 && ia[j] == na - r + j) --j;
        if (j < 0) amore = false;
        else {
            ++ia[j];
            for (int m = j + 1; m < r; ++m) ia[m] = ia[m - 1] + 1;
        }
    }
}

// group heads of the sorted entries (xid changes)
__global__ void k_heads(const unsigned long long *key, long long ne, long long *flag) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    flag[e] = (e == 0 || (key[e] >> 24) != (key[e - 1] >> 24)) ? 1 : 0;
}
// group end of every entry: the next head at or after e + 1
__global__ void k_group_end(const long long *head_pos, long long ngroups, const long long *gid_excl,
                            const long long *flag, long long ne, long long *gend) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const long long g = gid_excl[e] + flag[e] - 1;  // group index of e
    gend[e] = g + 1 < ngroups ? head_pos[g + 1] : ne;
}
__global__ void k_head_pos(const long long *flag, const long long *gid_excl, long long ne, long long *head_pos) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne || !flag[e]) return;
    head_pos[gid_excl[e]] = e;
}
__global__ void k_group_start(const long long *head_pos, const long long *gid_excl, const long long *flag,
                              long long ne, long long *gbeg) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    gbeg[e] = head_pos[gid_excl[e] + flag[e] - 1];
}

__device__ __forceinline__ double entry_coef(int v, const double *coef, long long ndet, int root) {
    const long long det = (v > 0 ? v : -v) - 1;
    const double c = coef[det + ndet * root];
    return v > 0 ? c : -c;
}

// D[S_e, S_f] += c_s(e) c_t(f) for every pair of one group; one thread per e
__global__ void k_gram(const unsigned long long *key, const int *val, const long long *gbeg, const long long *gend,
                       long long ne, const double *coef, long long ndet, int s, int t, long long dim, double *D) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const double vs = entry_coef(val[e], coef, ndet, s);
    if (vs == 0.0) return;
    double *row = D + (long long)(key[e] & 0xFFFFFFull) * dim;
    for (long long f = gbeg[e]; f < gend[e]; ++f) atomicAdd(row + (key[f] & 0xFFFFFFull), vs * entry_coef(val[f], coef, ndet, t));
}

// (rank, sign) of orbital tuple `orb` under spin pattern `spins` (bit m =
// beta) in block (k, r); false if two spin orbitals coincide
__device__ __forceinline__ bool spin_tuple_rank(const int *orb, unsigned spins, int k, int r, long long dimB,
                                                long long *rank, int *sgn) {
    int so[4];
    for (int m = 0; m < k; ++m) so[m] = orb[m] + ((spins >> m & 1u) ? 64 : 0);
    int par = 0;
    for (int i = 1; i < k; ++i) {
        const int v = so[i];
        int j = i - 1;
        while (j >= 0 && so[j] > v) {
            so[j + 1] = so[j];
            --j;
            ++par;
        }
        so[j + 1] = v;
    }
    for (int i = 1; i < k; ++i)
        if (so[i] == so[i - 1]) return false;
    int a[4], b[4];
    for (int i = 0; i < r; ++i) a[i] = so[i];
    for (int i = 0; i < k - r; ++i) b[i] = so[r + i] - 64;
    *rank = subset_rank(a, r) * dimB + subset_rank(b, k - r);
    *sgn = (par & 1) ? -1 : 1;
    return true;
}

// rank/sign tables of every tuple (n^k) under every spin pattern of block r
__global__ void k_tuple_tables(int n, int k, int r, long long dimB, long long nk, int *trk, signed char *tsg) {
    const long long Q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (Q >= nk) return;
    int q[4];
    long long y = Q;
    for (int m = 0; m < k; ++m) {
        q[m] = (int)(y % n);
        y /= n;
    }
    for (unsigned sp = 0; sp < (1u << k); ++sp) {
        long long rk;
        int sg;
        const bool ok = (k - __popc(sp) == r) && spin_tuple_rank(q, sp, k, r, dimB, &rk, &sg);
        trk[sp * nk + Q] = ok ? (int)rk : -1;
        tsg[sp * nk + Q] = ok ? (signed char)sg : 0;
    }
}

// dense k-RDM (k <= 3): out[slot + ldo (P + n^k Q)] += sum_sp sg(P) sg(Q) D[rk(P), rk(Q)]
__global__ void k_fold_dense(const double *D, long long dim, const int *trk, const signed char *tsg, int k,
                             long long nk, double *out, long long ldo, long long slot) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nk * nk) return;
    const long long P = t % nk, Q = t / nk;
    double acc = 0.0;
    for (unsigned sp = 0; sp < (1u << k); ++sp) {
        const int a = trk[sp * nk + P], b = trk[sp * nk + Q];
        if (a < 0 || b < 0) continue;
        acc += (double)(tsg[sp * nk + P] * tsg[sp * nk + Q]) * D[(long long)a * dim + b];
    }
    if (acc != 0.0) out[slot + ldo * t] += acc;
}

// packed 4-RDM: slot (ind(K), L) for every descending key K and every L with
// normind(L) <= normind(K); one thread per (key, L)
__global__ void k_fold_ro4(const double *D, long long dim, const int *trk, const signed char *tsg, int n,
                           long long W, double *ro4) {
    const long long n4 = (long long)n * n * n * n;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= W * n4) return;
    const long long L = t / W, kk = t % W;  // kk = ind - 1
    // decode the key: the kk-th descending quadruple in lindice order
    int K[4];
    {
        long long rem = kk + 1;
        int i1 = 1;
        while ((long long)i1 * (i1 + 1) * (i1 + 2) * (i1 + 3) / 24 < rem) ++i1;
        rem -= (long long)(i1 - 1) * i1 * (i1 + 1) * (i1 + 2) / 24;
        int i2 = 1;
        while ((long long)i2 * (i2 + 1) * (i2 + 2) / 6 < rem) ++i2;
        rem -= (long long)(i2 - 1) * i2 * (i2 + 1) / 6;
        int i3 = 1;
        while ((long long)i3 * (i3 + 1) / 2 < rem) ++i3;
        rem -= (long long)(i3 - 1) * i3 / 2;
        K[0] = i1 - 1; K[1] = i2 - 1; K[2] = i3 - 1; K[3] = (int)rem - 1;
    }
    int q[4];
    long long y = L;
    for (int m = 0; m < 4; ++m) {
        q[m] = (int)(y % n);
        y /= n;
    }
    if (normind4(q[0] + 1, q[1] + 1, q[2] + 1, q[3] + 1) > kk + 1) return;  // never addressed by ord8
    double acc = 0.0;
    for (unsigned sp = 0; sp < 16u; ++sp) {
        const int b = trk[sp * n4 + L];
        if (b < 0) continue;
        long long a;
        int sg;
        if (!spin_tuple_rank(K, sp, 4, 4 - __popc(sp), c_binom[n][__popc(sp)], &a, &sg)) continue;
        acc += (double)(sg * tsg[sp * n4 + L]) * D[a * dim + b];
    }
    if (acc != 0.0) ro4[kk + W * L] += acc;
}

}  // namespace

// Builds D of block (k, r) for roots (s, t) and folds it: fold(D, dim, dimB)
// is called with D on the device and returns 0 or an error.  Returns 0, 2 on
// an allocation failure.
template <class Fold>
static int rdm_block(int n, int k, int r, long long ndet, const unsigned *amask, const unsigned *bmask,
                     const double *coef, int s, int t, cudaStream_t st, Fold &&fold) {
    static const BinomHost host_binom;
    cudaMemcpyToSymbolAsync(c_binom, host_binom.t, sizeof(host_binom.t), 0, cudaMemcpyHostToDevice, st);
    const long long dimA = host_binom.t[n][r], dimB = host_binom.t[n][k - r], dim = dimA * dimB;
    std::vector<void *> bufs;
    struct Release {
        std::vector<void *> &b;
        cudaStream_t st;
        ~Release() {
            for (void *p : b) cudaFreeAsync(p, st);
        }
    } rel{bufs, st};
    auto get = [&](void **p, size_t bytes) {
        if (cudaMallocAsync(p, bytes ? bytes : 1, st) != cudaSuccess) return false;
        bufs.push_back(*p);
        return true;
    };
    // exclusive prefix sums (device scan) of m counts into out[0..m]
    auto scan = [&](const long long *in, long long m, long long *out) {
        size_t bytes = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (int64_t)m, st);
        void *tmp;
        if (!get(&tmp, bytes)) return false;
        cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, (int64_t)m, st);
        return true;
    };
    long long *cnt, *off;
    double *D;
    if (!get((void **)&cnt, sizeof(long long) * (ndet + 1)) || !get((void **)&off, sizeof(long long) * (ndet + 1)) ||
        !get((void **)&D, sizeof(double) * dim * dim))
        return 2;
    cudaMemsetAsync(D, 0, sizeof(double) * dim * dim, st);
    cudaMemsetAsync(cnt + ndet, 0, sizeof(long long), st);
    const unsigned nb = (unsigned)((ndet + 255) / 256);
    k_entry_counts<<<nb, 256, 0, st>>>(amask, bmask, ndet, k, r, cnt);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (!scan(cnt, ndet + 1, off)) return 2;  // off[ndet] = the entry count
    long long ne = 0;
    cudaMemcpyAsync(&ne, off + ndet, sizeof(long long), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (ne > 0) {
        unsigned long long *key, *key2;
        int *val, *val2;
        long long *flag, *gex, *hpos, *gbeg, *gend;
        if (!get((void **)&key, 8 * ne) || !get((void **)&key2, 8 * ne) || !get((void **)&val, 4 * ne) ||
            !get((void **)&val2, 4 * ne) || !get((void **)&flag, 8 * (ne + 1)) || !get((void **)&gex, 8 * (ne + 1)) ||
            !get((void **)&gbeg, 8 * ne) || !get((void **)&gend, 8 * ne))
            return 2;
        k_entries<<<nb, 256, 0, st>>>(amask, bmask, ndet, n, k, r, dimB, off, key, val);
        size_t tmp_bytes = 0;
        cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key, key2, val, val2, (int64_t)ne, 0, 64, st);
        void *tmp;
        if (!get(&tmp, tmp_bytes)) return 2;
        cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key, key2, val, val2, (int64_t)ne, 0, 64, st);
        const unsigned ge = (unsigned)((ne + 255) / 256);
        cudaMemsetAsync(flag + ne, 0, sizeof(long long), st);
        k_heads<<<ge, 256, 0, st>>>(key2, ne, flag);
        if (!scan(flag, ne + 1, gex)) return 2;  // gex[ne] = the group count
        long long ng = 0;
        cudaMemcpyAsync(&ng, gex + ne, sizeof(long long), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        if (!get((void **)&hpos, 8 * (ng + 1))) return 2;
        k_head_pos<<<ge, 256, 0, st>>>(flag, gex, ne, hpos);
        k_group_start<<<ge, 256, 0, st>>>(hpos, gex, flag, ne, gbeg);
        k_group_end<<<ge, 256, 0, st>>>(hpos, ng, gex, flag, ne, gend);
        k_gram<<<ge, 256, 0, st>>>(key2, val2, gbeg, gend, ne, coef, ndet, s, t, dim, D);
        g_launches.fetch_add(6, std::memory_order_relaxed);
    }
    return fold(D, dim, dimB);
}

int launch_rdm_dense(int n, int k, long long ndet, const unsigned *amask, const unsigned *bmask, const double *coef,
                     int s, int t, double *out, long long ldo, long long slot, cudaStream_t st) {
    long long nk = 1;
    for (int i = 0; i < k; ++i) nk *= n;
    for (int r = 0; r <= k; ++r) {
        int rc = rdm_block(n, k, r, ndet, amask, bmask, coef, s, t, st, [&](const double *D, long long dim,
                                                                           long long dimB) {
            int *trk = nullptr;
            signed char *tsg = nullptr;
            if (cudaMallocAsync((void **)&trk, sizeof(int) * (16 * nk), st) != cudaSuccess) return 2;
            if (cudaMallocAsync((void **)&tsg, 16 * nk, st) != cudaSuccess) {
                cudaFreeAsync(trk, st);
                return 2;
            }
            k_tuple_tables<<<(unsigned)((nk + 255) / 256), 256, 0, st>>>(n, k, r, dimB, nk, trk, tsg);
            k_fold_dense<<<(unsigned)((nk * nk + 255) / 256), 256, 0, st>>>(D, dim, trk, tsg, k, nk, out, ldo, slot);
            g_launches.fetch_add(2, std::memory_order_relaxed);
            cudaFreeAsync(tsg, st);
            cudaFreeAsync(trk, st);
            return 0;
        });
        if (rc) return rc;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

int launch_rofour(int n, long long ndet, const unsigned *amask, const unsigned *bmask, const double *coef, int s,
                  double *ro4_s, cudaStream_t st) {
    const long long n4 = (long long)n * n * n * n, W = (long long)n * (n + 1) * (n + 2) * (n + 3) / 24;
    for (int r = 0; r <= 4; ++r) {
        int rc = rdm_block(n, 4, r, ndet, amask, bmask, coef, s, s, st, [&](const double *D, long long dim,
                                                                          long long dimB) {
            int *trk = nullptr;
            signed char *tsg = nullptr;
            if (cudaMallocAsync((void **)&trk, sizeof(int) * (16 * n4), st) != cudaSuccess) return 2;
            if (cudaMallocAsync((void **)&tsg, 16 * n4, st) != cudaSuccess) {
                cudaFreeAsync(trk, st);
                return 2;
            }
            k_tuple_tables<<<(unsigned)((n4 + 255) / 256), 256, 0, st>>>(n, 4, r, dimB, n4, trk, tsg);
            k_fold_ro4<<<(unsigned)((W * n4 + 255) / 256), 256, 0, st>>>(D, dim, trk, tsg, n, W, ro4_s);
            g_launches.fetch_add(2, std::memory_order_relaxed);
            cudaFreeAsync(tsg, st);
            cudaFreeAsync(trk, st);
            return 0;
        });
        if (rc) return rc;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace nvpt
