// Unfolding of QCMaquis RDM label/value lists into the dense arrays of the
// path: src/rdm_utils.F90:236-464 permute_4rdm (into the packed 4-RDM
// ro4(W,n,n,n,n) of one state) and :470-511 permute_3rdm (into a 3-RDM
// (n,n,n,n,n,n) of one state or root pair), as hdf5_read_rdm_from_resfile
// (src/rdm_utils.F90:193-226) applies them: labels + 1, one call per entry in
// file order, every image an assignment (a later entry overwrites an earlier
// one on the same element; within one entry a later image overwrites an
// earlier one).
//
// GPU form: every entry is a thread.  Pass 1 claims each destination element
// with atomicMax of the key (entry << 4 | image); pass 2 writes the value of
// the image whose key won.  The result is the one of the sequential loop,
// bit for bit, independent of thread order.
#include "eexx.cuh"
#include "nvpt2_internal.h"

namespace nvpt {

namespace {

constexpr double kRdmThresh = 1.0e-12;  // src/rdm_utils.F90:241 / :479

struct Img {
    int a, b, c, d;  // permuted (m,n,o,p)
    signed char w;   // 0: val, 1: -val/2, 2: -2 val
};

// The image table of permute_4rdm for one label (1-based indices), in the
// reference's order.  Returns the number of images (0..12).
__device__ int images4(int i, int j, int k, int l, int m, int n, int o, int p, Img *im) {
    int c = 0;
    auto put = [&](int a, int b, int cc, int d, signed char w) { im[c++] = Img{a, b, cc, d, w}; };
    const signed char V = 0, H = 1, T = 2;
    if (i == j && k == l) {  // case 1
        if (m == n && o == p) {
            put(m, n, o, o, V); put(o, o, m, m, V);
            put(m, o, o, m, H); put(m, o, m, o, H); put(o, m, m, o, H); put(o, m, o, m, H);
        } else if (m == n && o != p) {
            put(m, n, o, p, V); put(m, m, p, o, V); put(o, p, m, m, V); put(p, o, m, m, V);
            put(o, m, m, p, H); put(o, m, p, m, H); put(p, m, m, o, H); put(p, m, o, m, H);
            put(m, o, p, m, H); put(m, p, o, m, H); put(m, p, m, o, H); put(m, o, m, p, H);
        } else if (m != n && o == p) {
            put(m, n, o, p, V); put(n, m, o, o, V); put(o, o, m, n, V); put(o, o, n, m, V);
            put(m, o, o, n, H); put(n, o, o, m, H); put(o, m, o, n, H); put(o, n, o, m, H);
            put(o, m, n, o, H); put(o, n, m, o, H); put(m, o, n, o, H); put(n, o, m, o, H);
        } else {  // m != n, o != p
            if (n == o) {
                put(m, n, o, p, V);
                put(n, n, m, p, T); put(n, n, p, m, T); put(m, p, n, n, T); put(p, m, n, n, T);
                put(p, n, n, m, V); put(p, n, m, n, V); put(m, n, p, n, V); put(n, p, m, n, V);
                put(n, m, p, n, V); put(n, m, n, p, V); put(n, p, n, m, V);
            } else {  // both remaining branches of the reference write the same eight images
                put(m, n, o, p, V); put(m, n, p, o, V); put(n, m, p, o, V); put(n, m, o, p, V);
                put(o, p, m, n, V); put(o, p, n, m, V); put(p, o, n, m, V); put(p, o, m, n, V);
            }
        }
    } else if (i == j && k != l) {  // case 2
        if (m == n && o == p) {
            put(m, n, o, p, V); put(o, o, m, m, V);
            put(m, o, o, m, H); put(o, m, m, o, H); put(o, m, o, m, H); put(m, o, m, o, H);
        }
        if (m == n && o != p) {
            put(m, n, o, p, V);
            put(m, o, m, p, H); put(m, p, o, m, H); put(o, m, m, p, H); put(p, m, o, m, H);
        }
        if (m != n && o == p) {
            put(m, n, o, p, V); put(n, m, o, o, V);
        }
        if (m != n && n != o && o != p && m != p) {
            put(m, n, o, p, V); put(n, m, o, p, V);
        }
    } else if (i != j && j == k && k != l) {  // case 3
        if (m == n && o == p) {
            put(m, n, o, p, V); put(o, o, m, m, V); put(o, m, o, m, V); put(m, o, m, o, V);
            put(m, o, o, m, T); put(o, m, m, o, T);
        }
        if (m != n && o == p) {
            put(m, n, o, p, V); put(o, o, m, n, V); put(o, m, o, n, V); put(m, o, n, o, V);
            put(m, o, o, n, T);
        }
        if (m != n && o != p && m == p) {
            put(m, n, o, p, V); put(m, o, n, m, V);
        }
        if (m != n && n != o && o != p && m != p) {
            put(m, n, o, p, V); put(m, o, n, p, V);
        }
    } else if (i != j && k == l) {  // case 4
        if (m == n && o == p) {
            put(m, n, o, p, V); put(o, o, m, m, V);
            put(m, o, o, m, H); put(o, m, m, o, H); put(o, m, o, m, H); put(m, o, m, o, H);
        }
        if (m == n && o != p) {
            put(m, n, o, p, V); put(m, m, p, o, V);
        }
        if (m != n && o == p) {
            put(m, n, o, p, V);
            put(m, o, n, o, H); put(m, o, o, n, H); put(o, n, o, m, H); put(o, n, m, o, H);
        }
        if (m != n && n != o && o != p && m != p) {
            put(m, n, o, p, V); put(m, n, p, o, V);
        }
    } else if (i != j && k != l && j != k) {  // case 5
        if ((m == o && n == p) || (m == p && n == o)) {
            put(m, n, o, p, V); put(n, m, p, o, V);
        } else if (m == n && o == p) {
            put(m, n, o, p, V); put(o, o, m, m, V);
        } else {
            put(m, n, o, p, V);
        }
    }
    return c;
}

__device__ __forceinline__ double weighted(double v, signed char w) {
    return w == 0 ? v : (w == 1 ? v * (-0.5) : v * (-2.0));
}

__device__ __forceinline__ bool label_ok(const int *L, int k, int n) {
    for (int q = 0; q < k; ++q)
        if (L[q] < 0 || L[q] >= n) return false;
    return true;
}

// ro4 offset (0-based) of norm(i,j,k,l), (a,b,c,d) for 1-based indices.
__device__ __forceinline__ ll ro4_at(ll W, int n, int i, int j, int k, int l, int a, int b, int c, int d) {
    return (normind4(i, j, k, l) - 1) + W * ((a - 1) + (ll)n * ((b - 1) + (ll)n * ((c - 1) + (ll)n * (d - 1))));
}

__global__ void k_unfold4(const int32_t *lab, const double *val, ll ne, int n, ll W, double *ro4,
                          unsigned long long *owner, int pass, int *bad) {
    ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int32_t *L = lab + 8 * e;
    int q[8];
    for (int t = 0; t < 8; ++t) q[t] = L[t];
    if (!label_ok(q, 8, n)) {
        atomicExch(bad, 1);
        return;
    }
    const double v = val[e];
    if (fabs(v) < kRdmThresh) return;
    Img im[12];
    const int cnt = images4(q[0] + 1, q[1] + 1, q[2] + 1, q[3] + 1, q[4] + 1, q[5] + 1, q[6] + 1, q[7] + 1, im);
    for (int t = 0; t < cnt; ++t) {
        const ll at = ro4_at(W, n, q[0] + 1, q[1] + 1, q[2] + 1, q[3] + 1, im[t].a, im[t].b, im[t].c, im[t].d);
        const unsigned long long key = ((unsigned long long)e << 4) | (unsigned long long)t;
        if (pass == 0) atomicMax(owner + at, key + 1);  // 0 = unclaimed
        else if (owner[at] == key + 1) ro4[at] = weighted(v, im[t].w);
    }
}

__global__ void k_unfold3(const int32_t *lab, const double *val, ll ne, int n, double *r3, ll ld, int trans,
                          unsigned long long *owner, int pass, int *bad) {
    ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int32_t *L = lab + 6 * e;
    int q[6];
    for (int t = 0; t < 6; ++t) q[t] = L[t];
    if (!label_ok(q, 6, n)) {
        atomicExch(bad, 1);
        return;
    }
    const double v = val[e];
    if (fabs(v) < kRdmThresh) return;
    const int i = q[0], j = q[1], k = q[2], l = q[3], m = q[4], nn = q[5];
    if (i == j && i == k) return;
    if (l == m && l == nn) return;
    const double tmp = trans ? v : -v;  // src/rdm_utils.F90:486
    const int P[12][6] = {{i, j, k, l, m, nn}, {i, k, j, l, nn, m}, {j, i, k, m, l, nn}, {j, k, i, m, nn, l},
                          {k, i, j, nn, l, m}, {k, j, i, nn, m, l}, {l, m, nn, i, j, k}, {l, nn, m, i, k, j},
                          {m, l, nn, j, i, k}, {m, nn, l, j, k, i}, {nn, l, m, k, i, j}, {nn, m, l, k, j, i}};
    const int cnt = trans ? 6 : 12;
    for (int t = 0; t < cnt; ++t) {
        const ll lin = P[t][0] + (ll)n * (P[t][1] + (ll)n * (P[t][2] + (ll)n * (P[t][3] + (ll)n * (P[t][4] + (ll)n * P[t][5]))));
        const unsigned long long key = ((unsigned long long)e << 4) | (unsigned long long)t;
        if (pass == 0) atomicMax(owner + lin, key + 1);
        else if (owner[lin] == key + 1) r3[lin * ld] = tmp;
    }
}

}  // namespace

int launch_unfold4(const int32_t *labels, const double *values, long long nentries, int n, double *ro4,
                   unsigned long long *owner, int *bad, cudaStream_t st) {
    const ll W = (ll)n * (n + 1) * (n + 2) * (n + 3) / 24, slots = W * n * n * n * n;
    if (cudaMemsetAsync(owner, 0, sizeof(unsigned long long) * slots, st) != cudaSuccess) return 1;
    if (nentries == 0) return 0;
    const unsigned g = (unsigned)((nentries + 255) / 256);
    for (int pass = 0; pass < 2; ++pass) {
        k_unfold4<<<g, 256, 0, st>>>(labels, values, nentries, n, W, ro4, owner, pass, bad);
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    return 0;
}

int launch_unfold3(const int32_t *labels, const double *values, long long nentries, int n, double *rdm3,
                   long long ld, bool trans, unsigned long long *owner, int *bad, cudaStream_t st) {
    const ll slots = (ll)n * n * n * n * n * n;
    if (cudaMemsetAsync(owner, 0, sizeof(unsigned long long) * slots, st) != cudaSuccess) return 1;
    if (nentries == 0) return 0;
    const unsigned g = (unsigned)((nentries + 255) / 256);
    for (int pass = 0; pass < 2; ++pass) {
        k_unfold3<<<g, 256, 0, st>>>(labels, values, nentries, n, rdm3, ld, trans ? 1 : 0, owner, pass, bad);
        g_launches.fetch_add(1, std::memory_order_relaxed);
    }
    return 0;
}

}  // namespace nvpt
