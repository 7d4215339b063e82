// Device-side index maps and normal-ordered <E..E> accessors.
//
// Index arithmetic of src/indices_norm.F90:31-106 and src/ord_utils.F90:71-129
// (ord8) and the accessor formulas of src/eexx_functions.F90:25-225, evaluated
// on the fly from the spin-free RDMs.  All orbital indices are 1-based and
// every array uses the reference's column-major, state-first layout
// (ro4 is state-last), so that device results address exactly the same
// elements as the Fortran code.
#pragma once
#include <cstdint>

namespace nvpt {

typedef long long ll;

// lindi/lindj/lindk of src/indices_norm.F90:42-45, closed form.
__host__ __device__ __forceinline__ int lindice4(int i, int j, int k, int l) {
    return (i - 1) * i * (i + 1) * (i + 2) / 24 + (j - 1) * j * (j + 1) / 6 + (k - 1) * k / 2 + l;
}

// norm(): value of lindice for the descending-sorted quadruple.
__host__ __device__ __forceinline__ int normind4(int a, int b, int c, int d) {
    int v0 = a, v1 = b, v2 = c, v3 = d, t;
#define NV_SWAP_DESC(x, y) if (x < y) { t = x; x = y; y = t; }
    NV_SWAP_DESC(v0, v1) NV_SWAP_DESC(v2, v3) NV_SWAP_DESC(v0, v2) NV_SWAP_DESC(v1, v3) NV_SWAP_DESC(v1, v2)
#undef NV_SWAP_DESC
    return lindice4(v0, v1, v2, v3);
}

// ord8 of src/ord_utils.F90:71-129: returns the packed key index
// lindice(i1..i4) and the permuted partner (i5..i8).  The key group is the
// one with the larger normind (the first on ties); the key is selection-sorted
// descending with the first maximum chosen, and every swap is mirrored on the
// partner, so tie handling matches the reference bit for bit.
__host__ __device__ __forceinline__ int ord8_key(int a1, int c1, int e1, int g1, int a2, int c2, int e2, int g2,
                                                 int &p0, int &p1, int &p2, int &p3) {
    int k[4], p[4];
    if (normind4(a1, c1, e1, g1) >= normind4(a2, c2, e2, g2)) {
        k[0] = a1; k[1] = c1; k[2] = e1; k[3] = g1;
        p[0] = a2; p[1] = c2; p[2] = e2; p[3] = g2;
    } else {
        k[0] = a2; k[1] = c2; k[2] = e2; k[3] = g2;
        p[0] = a1; p[1] = c1; p[2] = e1; p[3] = g1;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int imax = k[i], jmax = i;
#pragma unroll
        for (int j = i + 1; j < 4; ++j)
            if (k[j] > imax) { imax = k[j]; jmax = j; }
        if (jmax != i) {
            int t = k[i]; k[i] = k[jmax]; k[jmax] = t;
            t = p[i]; p[i] = p[jmax]; p[jmax] = t;
        }
    }
    p0 = p[0]; p1 = p[1]; p2 = p[2]; p3 = p[3];
    return lindice4(k[0], k[1], k[2], k[3]);
}

// ord9 of src/ord_utils.F90:16-68: the same key choice as ord8, but the key
// is exchange-sorted (every larger later element is swapped into place at
// once, and the partner swapped with it), which differs from ord8 on ties.
// Returns lindice of the sorted key; k0..k3 the key, p0..p3 the partner.
__host__ __device__ __forceinline__ int ord9_key(int a1, int c1, int e1, int g1, int a2, int c2, int e2, int g2,
                                                 int &k0, int &k1, int &k2, int &k3, int &p0, int &p1, int &p2,
                                                 int &p3) {
    int k[4], p[4];
    if (normind4(a1, c1, e1, g1) >= normind4(a2, c2, e2, g2)) {
        k[0] = a1; k[1] = c1; k[2] = e1; k[3] = g1;
        p[0] = a2; p[1] = c2; p[2] = e2; p[3] = g2;
    } else {
        k[0] = a2; k[1] = c2; k[2] = e2; k[3] = g2;
        p[0] = a1; p[1] = c1; p[2] = e1; p[3] = g1;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i + 1; j < 4; ++j)
            if (k[j] > k[i]) {
                int t = k[i]; k[i] = k[j]; k[j] = t;
                t = p[i]; p[i] = p[j]; p[j] = t;
            }
    k0 = k[0]; k1 = k[1]; k2 = k[2]; k3 = k[3];
    p0 = p[0]; p1 = p[1]; p2 = p[2]; p3 = p[3];
    return lindice4(k[0], k[1], k[2], k[3]);
}

// Views of the spin-free RDMs of one problem, reference layouts.
struct Rdm {
    int n, M;
    ll W;
    const double *d1, *d2, *d3, *ro4;

    __device__ __forceinline__ double D1(int s, int a, int b) const {
        return d1[(s - 1) + (ll)M * ((a - 1) + (ll)n * (b - 1))];
    }
    __device__ __forceinline__ double D2(int s, int a, int b, int c, int d) const {
        return d2[(s - 1) + (ll)M * ((a - 1) + (ll)n * ((b - 1) + (ll)n * ((c - 1) + (ll)n * (d - 1))))];
    }
    __device__ __forceinline__ double D3(int s, int a, int b, int c, int d, int e, int f) const {
        return d3[(s - 1) +
                  (ll)M * ((a - 1) + (ll)n * ((b - 1) + (ll)n * ((c - 1) + (ll)n * ((d - 1) + (ll)n * ((e - 1) + (ll)n * (f - 1))))))];
    }
    __device__ __forceinline__ double R4(int ind, int i5, int i6, int i7, int i8, int s) const {
        return ro4[(ind - 1) + W * ((i5 - 1) + (ll)n * ((i6 - 1) + (ll)n * ((i7 - 1) + (ll)n * ((i8 - 1) + (ll)n * (s - 1)))))];
    }

    // eexx_functions.F90:125-135
    __device__ __forceinline__ double ee2(int a, int b, int c, int d, int s) const {
        double r = D2(s, a, c, b, d);
        if (b == c) r += D1(s, a, d);
        return r;
    }
    // eexx_functions.F90:138-148
    __device__ __forceinline__ double ee2t(int a, int b, int c, int d, int s) const {
        double r = -ee2(b, a, c, d, s);
        if (a == b) r += 2.0 * D1(s, c, d);
        return r;
    }
    // eexx_functions.F90:151-161
    __device__ __forceinline__ double ee2tr(int a, int b, int c, int d, int s) const {
        double r = -ee2(a, b, d, c, s);
        if (c == d) r += 2.0 * D1(s, a, b);
        return r;
    }
    // eexx_functions.F90:79-94
    __device__ __forceinline__ double eee2(int a, int b, int c, int d, int e, int f, int s) const {
        double r = D3(s, a, c, e, b, d, f);
        if (e == d) r += D2(s, a, c, b, f);
        if (e == b) r += D2(s, a, c, f, d);
        if (b == c) r += D2(s, a, e, d, f);
        if (b == c && e == d) r += D1(s, a, f);
        return r;
    }
    // eexx_functions.F90:97-108
    __device__ __forceinline__ double eee2t(int a, int b, int c, int d, int e, int f, int s) const {
        double r = -eee2(a, b, d, c, e, f, s);
        if (c == d) r += 2.0 * ee2(a, b, e, f, s);
        return r;
    }
    // eexx_functions.F90:111-122
    __device__ __forceinline__ double eee2tl(int a, int b, int c, int d, int e, int f, int s) const {
        double r = -eee2(b, a, c, d, e, f, s);
        if (a == b) r += 2.0 * ee2(c, d, e, f, s);
        return r;
    }
    // eexx_functions.F90:25-61
    __device__ __forceinline__ double eeee(int a, int b, int c, int d, int e, int f, int g, int h, int s) const {
        int q0, q1, q2, q3;
        int ind = ord8_key(a, c, e, g, b, d, f, h, q0, q1, q2, q3);
        double r = R4(ind, q0, q1, q2, q3, s);
        if (b == c) r += D3(s, a, e, g, d, f, h);
        if (b == e) r += D3(s, a, c, g, f, d, h);
        if (b == g) r += D3(s, a, c, e, h, d, f);
        if (d == e) r += D3(s, a, g, c, b, h, f);
        if (d == g) r += D3(s, a, c, e, b, h, f);
        if (f == g) r += D3(s, a, e, c, b, h, d);
        if (b == c) {
            if (d == e) r += D2(s, a, g, f, h);
            if (d == g) r += D2(s, a, e, h, f);
            if (f == g) r += D2(s, a, e, d, h);
        }
        if (b == e && d == g) r += D2(s, a, c, f, h);
        if (b == e && f == g) r += D2(s, a, c, h, d);
        if (b == g && d == e) r += D2(s, a, c, h, f);
        if (d == e && f == g) r += D2(s, a, c, b, h);
        if (b == c && d == e && f == g) r += D1(s, a, h);
        return r;
    }
    // eexx_functions.F90:64-75
    __device__ __forceinline__ double eeeet(int a, int b, int c, int d, int e, int f, int g, int h, int s) const {
        double r = -eeee(a, b, d, c, e, f, g, h, s);
        if (c == d) r += 2.0 * eee2(a, b, e, f, g, h, s);
        return r;
    }
    // eexx_functions.F90:210-225
    __device__ __forceinline__ double ro2t(int ap, int bp, int a, int b, int s) const {
        double r = D2(s, a, b, ap, bp);
        if (ap == a) r -= 2.0 * D1(s, b, bp);
        if (bp == b) r -= 2.0 * D1(s, a, ap);
        if (ap == b) r += D1(s, a, bp);
        if (bp == a) r += D1(s, b, ap);
        if (ap == a && bp == b) r += 4.0;
        if (ap == b && bp == a) r -= 2.0;
        return r;
    }
    // eexx_functions.F90:164-207
    __device__ double ro3t(int a, int b, int c, int ap, int bp, int cp, int s) const {
        double r = -D3(s, ap, bp, cp, a, b, c);
        if (ap == a) r += 2.0 * D2(s, bp, cp, b, c);
        if (bp == b) r += 2.0 * D2(s, ap, cp, a, c);
        if (cp == c) r += 2.0 * D2(s, ap, bp, a, b);
        if (bp == c) r -= D2(s, ap, cp, a, b);
        if (ap == c) r -= D2(s, cp, bp, a, b);
        if (cp == b) r -= D2(s, bp, ap, c, a);
        if (ap == b) r -= D2(s, bp, cp, a, c);
        if (cp == a) r -= D2(s, ap, bp, c, b);
        if (bp == a) r -= D2(s, ap, cp, b, c);
        if (cp == c && bp == b) r -= 4.0 * D1(s, ap, a);
        if (cp == b && bp == c) r += 2.0 * D1(s, ap, a);
        if (cp == c && ap == a) r -= 4.0 * D1(s, bp, b);
        if (cp == a && ap == c) r += 2.0 * D1(s, bp, b);
        if (ap == a && bp == b) r -= 4.0 * D1(s, cp, c);
        if (ap == b && bp == a) r += 2.0 * D1(s, cp, c);
        if (cp == c && ap == b) r += 2.0 * D1(s, bp, a);
        if (cp == b && ap == c) r -= D1(s, bp, a);
        if (cp == c && bp == a) r += 2.0 * D1(s, ap, b);
        if (cp == a && bp == c) r -= D1(s, ap, b);
        if (bp == b && ap == c) r += 2.0 * D1(s, cp, a);
        if (bp == c && ap == b) r -= D1(s, cp, a);
        if (bp == b && cp == a) r += 2.0 * D1(s, ap, c);
        if (bp == a && cp == b) r -= D1(s, ap, c);
        if (ap == a && cp == b) r += 2.0 * D1(s, bp, c);
        if (ap == b && cp == a) r -= D1(s, bp, c);
        if (ap == a && bp == c) r += 2.0 * D1(s, cp, b);
        if (ap == c && bp == a) r -= D1(s, cp, b);
        if (ap == a && bp == b && cp == c) r += 8.0;
        if (ap == b && bp == a && cp == c) r -= 4.0;
        if (ap == a && bp == c && cp == b) r -= 4.0;
        if (ap == c && bp == b && cp == a) r -= 4.0;
        if (ap == b && bp == c && cp == a) r += 2.0;
        if (ap == c && bp == a && cp == b) r += 2.0;
        return r;
    }
};

// Lower-triangle packed one-electron operator: indice(i,j) of
// src/koop_matrices.F90:186 over the full orbital range (1-based).
__host__ __device__ __forceinline__ ll tri_index(int i, int j) {
    int mx = i > j ? i : j, mn = i > j ? j : i;
    return (ll)mx * (mx - 1) / 2 + mn;
}

}  // namespace nvpt
