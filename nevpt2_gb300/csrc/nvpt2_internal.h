// Internal declarations shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <string>
#include "eexx.cuh"

namespace nvpt {

// Kernels launched by this library since load (all contexts).
extern std::atomic<long long> g_launches;

void launch_build_f(double *f, const double *aj, const double *atwo, int n, int ncore, int mode, cudaStream_t st);
// 0 on success, 2 if its scratch could not be allocated
int launch_bro3(const Rdm &r, double *daaa, int nele, cudaStream_t st);
void launch_bro2(const Rdm &r, double *taa, int nele, cudaStream_t st);
void launch_bro1(const Rdm &r, double *dal, int nele, cudaStream_t st);
void launch_aj_atwo(const double *oneint, const double *L, int Q, int n, int ncore, int norb, double *atwo,
                    double *aj, cudaStream_t st);
void launch_koopE(const Rdm &r, const double *atwo, const double *f, int ncore, double *ip, double *ea,
                  cudaStream_t st);
void launch_hrdm(const Rdm &r, double *hrdm, cudaStream_t st);
void launch_koop2E(const Rdm &r, const double *atwo, const double *f, int ncore, double *ip2, double *ea2,
                   cudaStream_t st);
void launch_koop0p(const Rdm &r, const double *atwo, const double *f, int ncore, double *gk0pa, double *gk0pd,
                   double *gk0pf, cudaStream_t st);
void launch_bbmat(const Rdm &r, const double *atwo, const double *f, const double *aj, int ncore, double *b,
                  double *bt, cudaStream_t st);
void launch_bcmat(const Rdm &r, const double *atwo, const double *f, int ncore, double *c, double *ct,
                  cudaStream_t st);
void launch_bdmat(const Rdm &r, const double *atwo, const double *f, const double *aj, int ncore, double *d,
                  double *dt, cudaStream_t st);
void launch_bamat_direct(const Rdm &r, const double *atwo, const double *f, int ncore, double *amat, double *atmat,
                         cudaStream_t st);
// Dense-contraction A-matrix builder (bamat_gemm.cu); 0 on success, 2 on a
// failed allocation, 5 if a split-precision product timed out, else a
// cuBLAS / launch failure.  split: the n^9 slab products run as Ozaki digit
// products on the tensor cores (ozaki.cu) instead of FP64 DGEMMs.
int launch_bamat_gemm(const Rdm &r, const double *atwo, const double *f, int ncore, double *amat, double *atmat,
                      cudaStream_t st, int slabs_per_batch, bool split = false);
// No-allocation A-matrix builder (bamat_gemm.cu): scratch in a static device
// array sized for kBamatStaticNactMax active orbitals; 0 on success, 1 if
// nact exceeds the limit.
constexpr int kBamatStaticNactMax = 8;
constexpr long long kBamatStaticDoubles = 4LL * 262144 + 7LL * 4096 + 64;  // 4n^6 + 7n^4 + n^2 at n = 8
double *bamat_static_scratch(int device);
int launch_bamat_static(const Rdm &r, const double *atwo, const double *f, int ncore, double *amat, double *atmat,
                        cudaStream_t st, double *scratch);
// Symmetry-packed two-electron integrals (ijkl_sym.cu): device views of the
// addressing tables of src/ijkl_utils.F90 (1-based values) and of twoint.
struct IjklTables {
    const long long *num, *indic, *jndic, *ndeb, *nad, *kt;
    const double *twoint;
};
int launch_ijkl_tables(int nsym, const long long *nish, const long long *nash, const long long *nssh, int norb,
                       long long *its, long long *itsym, long long *num, long long *indic, long long *jndic,
                       long long *ndeb, long long *nad, long long *kt, long long *ni4, int *bad, cudaStream_t st);
void launch_ai_twoint(const IjklTables &T, long long count, const int64_t *ijkl, double *out, cudaStream_t st);
void launch_sym_screen(double *x, double *y, int M, int n, int k, const long long *irr, cudaStream_t st);
void launch_aj_atwo_twoint(const IjklTables &T, const double *oneint, int n, int ncore, int norb, double *atwo,
                           double *aj, cudaStream_t st);
// Spin-free RDMs of a determinant expansion (rdm_build.cu): dense k <= 3 for
// (bra s, ket t) accumulated at out[slot + ldo (P + n^k Q)]; packed 4-RDM of
// root s.  0 on success, 2 on an allocation failure.
int launch_rdm_dense(int n, int k, long long ndet, const unsigned *amask, const unsigned *bmask, const double *coef,
                     int s, int t, double *out, long long ldo, long long slot, cudaStream_t st);
int launch_rofour(int n, long long ndet, const unsigned *amask, const unsigned *bmask, const double *coef, int s,
                  double *ro4_s, cudaStream_t st);
// Kernel spans for live measurement (nvpt_set_profiling): when enabled, a
// tagged launch is bracketed by CUDA events on its stream together with its
// algorithmic byte count; nvpt_profile_read sums the spans of one tag.
bool prof_enabled();
struct ProfSpan {
    cudaEvent_t a = nullptr, b = nullptr;
    const char *tag = nullptr;
    cudaStream_t st = nullptr;
    long long bytes = 0;
    void begin(const char *t, cudaStream_t s, long long nbytes);
    void end();
};
// QCMaquis label/value unfolding (rdm_unfold.cu); owner: one word per
// destination element; *bad set if a label is out of range.  0 on success.
int launch_unfold4(const int32_t *labels, const double *values, long long nentries, int n, double *ro4,
                   unsigned long long *owner, int *bad, cudaStream_t st);
int launch_unfold3(const int32_t *labels, const double *values, long long nentries, int n, double *rdm3,
                   long long ld, bool trans, unsigned long long *owner, int *bad, cudaStream_t st);
void launch_ord8(const int64_t *in8, int64_t *out8, int64_t *lindex, long long count, cudaStream_t st);

}  // namespace nvpt
