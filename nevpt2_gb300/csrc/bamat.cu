// A-matrices of the (+-1') perturber classes, src/koopro4QD.F90:3974-4104
// (bamat, C1 branch), FP64.
//
// The reference loops over (a,b,c,ap,bp,cp) and scatters part of the EA
// contribution into the b<->bp transposed element atmat(ap,b,cp,a,bp,c).  Here
// one thread owns one output element O = (ap,bp,cp,a,b,c) of both amat and
// atmat: it evaluates the iteration (a,b,c,ap,bp,cp) for amat and for the
// non-transposed atmat terms, and the mirror iteration (a,bp,c,ap,b,cp) for the
// transposed atmat terms, so there is no atomic and no race.
#include "nvpt2_internal.h"

namespace nvpt {

#define ATWO(i, j, k, l) atwo[((i)-1) + (ll)n * (((j)-1) + (ll)n * (((k)-1) + (ll)n * ((l)-1)))]
#define FF(i, j) f[tri_index((i) + ncore, (j) + ncore) - 1]

__global__ void __launch_bounds__(128) k_bamat_direct(Rdm r, const double *atwo, const double *f, int ncore,
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
                // direct iteration (b, bp)
                double dum1 = r.eee2(cp, ap, bp, b, d, ie, s);
                double dum2 = r.eee2(cp, ap, bp, b, d, c, s);
                double dum3 = r.eee2(cp, ap, bp, b, a, ie, s);
                double dum4 = r.eee2(cp, ap, bp, ie, a, c, s);
                A += dum1 * dint1 - 0.5 * (dum2 * dint2 + dum3 * dint3 - dum4 * dint4);
                At += 0.5 * r.eee2t(cp, ap, bp, ie, a, c, s) * dint4;
                // mirror iteration: loop b = bp(O), loop bp = b(O)
                double m1 = -r.eee2(cp, ap, b, bp, d, ie, s);
                double m2 = -r.eee2(cp, ap, b, bp, d, c, s);
                double m3 = -r.eee2(cp, ap, b, bp, a, ie, s);
                if (b == bp) {
                    m1 += 2.0 * r.ee2(cp, ap, d, ie, s);
                    m2 += 2.0 * r.ee2(cp, ap, d, c, s);
                    m3 += 2.0 * r.ee2(cp, ap, a, ie, s);
                }
                At += m1 * dint1 - 0.5 * (m2 * dint2 + m3 * dint3);
                for (int ief = 1; ief <= n; ++ief) {
                    double di1 = ATWO(d, ief, ie, a), di2 = ATWO(d, ief, c, ie), di3 = ATWO(d, ief, b, ie);
                    A += r.eeee(cp, ap, bp, b, d, ief, ie, c, s) * di1 - r.eeee(cp, ap, bp, b, d, ief, a, ie, s) * di2 -
                         r.eeee(cp, ap, bp, ie, d, ief, a, c, s) * di3;
                    At += r.eeeet(cp, ap, bp, ie, d, ief, a, c, s) * di3;
                    double e1t = -r.eeee(cp, ap, b, bp, d, ief, ie, c, s);
                    double e2t = -r.eeee(cp, ap, b, bp, d, ief, a, ie, s);
                    if (b == bp) {
                        e1t += 2.0 * r.eee2(cp, ap, d, ief, ie, c, s);
                        e2t += 2.0 * r.eee2(cp, ap, d, ief, a, ie, s);
                    }
                    At += e1t * di1 - e2t * di2;
                }
            }
        }
        ll o = (s - 1) + (ll)M * t;
        amat[o] = A;
        atmat[o] = At;
    }
}

void launch_bamat_direct(const Rdm &r, const double *atwo, const double *f, int ncore, double *amat, double *atmat,
                         cudaStream_t st) {
    ll n6 = (ll)r.n * r.n * r.n * r.n * r.n * r.n;
    k_bamat_direct<<<(unsigned)((n6 + 127) / 128), 128, 0, st>>>(r, atwo, f, ncore, amat, atmat);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

}  // namespace nvpt
