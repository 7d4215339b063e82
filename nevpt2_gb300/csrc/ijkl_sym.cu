// Symmetry-packed two-electron integrals: the irrep tables of
// src/infsym.F90:16-69 (initialize_infsym), the addressing tables of
// src/ijkl_utils.F90:111-170 (determine_n2int) and :173-207 (reijkl), the
// lookup ai_twoint (:690-756), and get_aj_atwo (src/koopro4QD.F90:3900-3971)
// on that integral path.
//
// Integer tables, 1-based values as in the reference (int64, the reference's
// default integer kind), built on the device:
//   its(i,j)  = ((i-1) xor (j-1)) + 1, the D2h-subgroup product table
//   itsym(k)  irrep of orbital k, ordered inactive (irrep by irrep), active,
//             virtual
//   num(k)    = k(k-1)/2 for k = 1..norb(norb+1)/2
//   indic(ij) irrep of the pair ij = num(i)+j (i >= j); jndic(ij) its rank
//             among the pairs of that irrep (in ij order)
//   ndeb(r)   offset of the pair-irrep r block of twoint; ni4 its length
//   nad/kt    per irrep pair (is >= js, position num(is)+js): nad = is and
//             kt = 1 when js == is, else 0 (the integral vanishes)
// twoint holds, per pair irrep r, the triangle of (ij|kl) over the pairs of
// that irrep, (ij|kl) at ndeb(r) + num(max(jndic)) + min(jndic).
#include "nvpt2_internal.h"

namespace nvpt {

// One CTA: the per-irrep ranks jndic are a running count over the pairs in
// ij order, formed chunk by chunk with warp ballots and a block prefix.
__global__ void __launch_bounds__(256) k_ijkl_tables(int nsym, const ll *nish, const ll *nash, const ll *nssh,
                                                     int norb, ll *its, ll *itsym, ll *num, ll *indic, ll *jndic,
                                                     ll *ndeb, ll *nad, ll *kt, ll *ni4, int *bad) {
    __shared__ int s_itsym[4096];
    __shared__ ll s_base[8];
    __shared__ int s_warp[8][8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < nsym * nsym; i += blockDim.x) its[i] = ((i % nsym) ^ (i / nsym)) + 1;
    if (tid == 0) {
        int k = 0;
        const ll *cnt[3] = {nish, nash, nssh};
        for (int sp = 0; sp < 3; ++sp)
            for (int r = 0; r < nsym; ++r)
                for (ll j = 0; j < cnt[sp][r]; ++j) {
                    if (k < norb) {
                        itsym[k] = r + 1;
                        s_itsym[k] = r + 1;
                    }
                    ++k;
                }
        *bad = (k != norb);
        for (int r = 0; r < 8; ++r) s_base[r] = 0;
    }
    __syncthreads();
    if (*bad) return;
    const ll npair = (ll)norb * (norb + 1) / 2;
    for (ll k = tid; k < npair; k += blockDim.x) num[k] = k * (k + 1) / 2;  // num(k+1) = k(k+1)/2
    for (ll c0 = 0; c0 < npair; c0 += blockDim.x) {
        const ll t = c0 + tid;
        int r = -1;
        if (t < npair) {
            // pair t (0-based) = num(i) + j - 1 with i >= j
            int i = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) / 2.0);
            while ((ll)i * (i + 1) / 2 > t) --i;
            while ((ll)(i + 1) * (i + 2) / 2 <= t) ++i;
            const int j = (int)(t - (ll)i * (i + 1) / 2);  // 0-based j <= i
            r = (s_itsym[i] - 1) ^ (s_itsym[j] - 1);          // pair irrep, 0-based
            indic[t] = r + 1;
        }
        int my_prefix = 0;
        for (int q = 0; q < nsym; ++q) {
            const unsigned m = __ballot_sync(0xffffffffu, r == q);
            if (lane == 0) s_warp[q][warp] = __popc(m);
            if (r == q) my_prefix = __popc(m & ((1u << lane) - 1u));
        }
        __syncthreads();
        if (r >= 0) {
            int before = 0;
            for (int w = 0; w < warp; ++w) before += s_warp[r][w];
            jndic[t] = s_base[r] + before + my_prefix + 1;
        }
        __syncthreads();
        if (tid < nsym) {
            int tot = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s_warp[tid][w];
            s_base[tid] += tot;
        }
        __syncthreads();
    }
    if (tid == 0) {
        // s_base[r] = nos(r+1), the pair count of each irrep
        ll off = 0;
        for (int r = 0; r < nsym; ++r) {
            ndeb[r] = off;
            off += s_base[r] * (s_base[r] + 1) / 2;
        }
        *ni4 = off;
        int p = 0;
        for (int is = 1; is <= nsym; ++is)
            for (int js = 1; js <= is; ++js, ++p) {
                nad[p] = js == is ? is : 0;
                kt[p] = js == is ? 1 : 0;
            }
    }
}

// src/ijkl_utils.F90:690-756 ai_twoint, with the tables above.
__device__ __forceinline__ double ai_twoint(const IjklTables &T, int i, int j, int k, int l) {
    ll ij = i >= j ? T.num[i - 1] + j : T.num[j - 1] + i;
    ll kl = k >= l ? T.num[k - 1] + l : T.num[l - 1] + k;
    const ll ijs = T.indic[ij - 1], kls = T.indic[kl - 1];
    ll ijkls;
    if (ijs > kls) {
        ijkls = T.num[ijs - 1] + kls;
    } else {
        ijkls = T.num[kls - 1] + ijs;
        const ll tmp = ij;
        ij = kl;
        kl = tmp;
    }
    const ll nadv = T.nad[ijkls - 1];
    if (nadv == 0) return 0.0;
    const bool zsig = nadv < 0;
    const ll nadi = zsig ? -nadv : nadv;
    if (T.kt[ijkls - 1] != 1) return 0.0;  // kt is 0 or 1 here; 0 pairs with nad = 0 above
    const ll nij = T.jndic[ij - 1], nkl = T.jndic[kl - 1];
    const ll ijkl = nij > nkl ? T.num[nij - 1] + nkl : T.num[nkl - 1] + nij;
    const double v = T.twoint[T.ndeb[nadi - 1] + ijkl - 1];
    return zsig ? -v : v;
}

__global__ void k_ai_twoint_list(IjklTables T, ll count, const int64_t *ijkl, double *out) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t *q = ijkl + 4 * t;
    out[t] = ai_twoint(T, (int)q[0], (int)q[1], (int)q[2], (int)q[3]);
}

// get_aj_atwo on the twoint path: atwo(i,j,k,l) = (i+nc j+nc | k+nc l+nc)
// and aj(active upper triangle) = oneint + sum_{j<=ncore} [2(ab|jj) - (aj|jb)]
// (the rest of aj is the caller's copy of oneint).
__global__ void k_atwo_twoint(IjklTables T, int n, int ncore, double *atwo) {
    const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (ll)n * n * n * n) return;
    const int i = (int)(t % n), j = (int)((t / n) % n), k = (int)((t / ((ll)n * n)) % n),
              l = (int)(t / ((ll)n * n * n));
    atwo[t] = ai_twoint(T, i + 1 + ncore, j + 1 + ncore, k + 1 + ncore, l + 1 + ncore);
}

__global__ void k_aj_twoint(IjklTables T, const double *oneint, int n, int ncore, double *aj) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int a = t % n + 1, b = t / n + 1;
    if (b < a) return;
    const int ac = a + ncore, bc = b + ncore;
    const ll jab = tri_index(ac, bc) - 1;
    double v = oneint[jab];
    for (int j = 1; j <= ncore; ++j) v = v + 2.0 * ai_twoint(T, ac, bc, j, j) - ai_twoint(T, ac, j, j, bc);
    aj[jab] = v;
}

// Output screens of the symmetry branches: an element whose orbitals'
// irreps multiply to a non-symmetric irrep is set to zero -- bamat's
// isatot /= 1 (src/koopro4QD.F90:4105-4133: all six indices of
// amat/atmat(s,ap,bp,cp,a,b,c)) and koop2E's its(isab,iscd) /= 1
// (src/koop_matrices.F90:289-304,336-351: the four indices of the 2-IP/2-EA
// matrices).  irr = itsym of the first active orbital onward (1-based).
__global__ void k_sym_screen(double *x, double *y, int M, int n, int k, const ll *irr) {
    ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    ll total = M;
    for (int i = 0; i < k; ++i) total *= n;
    if (t >= total) return;
    ll r = t / M;
    int g = 0;
    for (int i = 0; i < k; ++i) {
        g ^= (int)irr[r % n] - 1;
        r /= n;
    }
    if (g != 0) {
        x[t] = 0.0;
        if (y) y[t] = 0.0;
    }
}

void launch_sym_screen(double *x, double *y, int M, int n, int k, const long long *irr, cudaStream_t st) {
    ll total = M;
    for (int i = 0; i < k; ++i) total *= n;
    k_sym_screen<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(x, y, M, n, k, irr);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

int launch_ijkl_tables(int nsym, const ll *nish, const ll *nash, const ll *nssh, int norb, ll *its, ll *itsym,
                       ll *num, ll *indic, ll *jndic, ll *ndeb, ll *nad, ll *kt, ll *ni4, int *bad, cudaStream_t st) {
    k_ijkl_tables<<<1, 256, 0, st>>>(nsym, nish, nash, nssh, norb, its, itsym, num, indic, jndic, ndeb, nad, kt, ni4,
                                     bad);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 1;
}

void launch_ai_twoint(const IjklTables &T, ll count, const int64_t *ijkl, double *out, cudaStream_t st) {
    if (count <= 0) return;
    k_ai_twoint_list<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(T, count, ijkl, out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

void launch_aj_atwo_twoint(const IjklTables &T, const double *oneint, int n, int ncore, int norb, double *atwo,
                           double *aj, cudaStream_t st) {
    cudaMemcpyAsync(aj, oneint, sizeof(double) * (size_t)norb * (norb + 1) / 2, cudaMemcpyDeviceToDevice, st);
    k_aj_twoint<<<(unsigned)((n * n + 63) / 64), 64, 0, st>>>(T, oneint, n, ncore, aj);
    const ll n4 = (ll)n * n * n * n;
    k_atwo_twoint<<<(unsigned)((n4 + 127) / 128), 128, 0, st>>>(T, n, ncore, atwo);
    g_launches.fetch_add(2, std::memory_order_relaxed);
}

}  // namespace nvpt
