/*
 * nvpt2.h - C ABI of the GB300 (sm_103a) Koopmans-matrix and SC/PC-NEVPT2 library.
 *
 * Drop-in boundary for the compute subroutines of qcscine/nevpt2's two
 * Fortran stages.  Each host-pointer entry point below mirrors one Fortran
 * subroutine: same argument meaning, same array layouts (Fortran
 * column-major, 1-based index semantics inside the tables, the state index
 * first/fastest, except ro4(W,n,n,n,n,M) whose state index is last), and the
 * same in/out behaviour (the one-electron scratch f(*) is overwritten with the
 * builder's own operator on the active upper triangle, exactly as the
 * reference does).  Integer arguments are int64_t because the reference is
 * built with -fdefault-integer-8 (CMakeLists.txt:18, cmake/FortranFlags.cmake:16-20).
 *
 * The Fortran drivers keep allocating every array; the library copies the
 * inputs to the GPU, computes there, and copies the outputs back.  Every call
 * returns an int status (NVPT_OK == 0); where the reference would `stop`, the
 * library returns a nonzero status and nvpt_last_error() describes it.  The
 * `_d` variants take device pointers and a CUDA stream (NULL = the context's
 * stream) for callers that keep the tensors resident on the GPU; they enqueue
 * work and return without synchronising.
 *
 * One context per host thread at a time; contexts are independent.
 */
#ifndef NVPT2_H
#define NVPT2_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NVPT_OK 0
#define NVPT_EINVAL 1    /* bad size or argument (reference: stop)        */
#define NVPT_ECUDA 2     /* CUDA runtime / launch error                    */
#define NVPT_ENOMEM 3    /* device allocation failed                       */
#define NVPT_ENOTSUP 4   /* configuration outside the supported path       */
#define NVPT_ETIMEDOUT 5 /* a bounded device-side wait gave up             */
#define NVPT_EIO 6       /* file missing, unreadable or not a container    */

typedef struct nvpt_context nvpt_context;

/* Context life cycle.  `device` is the CUDA ordinal.  The library's scratch
 * is stream-ordered (cudaMallocAsync on the device's default memory pool);
 * nvpt_create sets that pool's release threshold so that freed scratch stays
 * in the pool between calls instead of returning to the driver at every
 * synchronisation (cudaMemPoolTrimTo gives it back). */
int nvpt_create(nvpt_context **ctx, int device);
int nvpt_destroy(nvpt_context *ctx);
int nvpt_synchronize(nvpt_context *ctx);
const char *nvpt_last_error(const nvpt_context *ctx);
const char *nvpt_status_string(int status);
/* Number of kernels this context has launched since creation. */
int64_t nvpt_launch_count(const nvpt_context *ctx);

/* ------------------------------------------------------------------ */
/* Packed-index maps (integer, bit-exact).                             */
/* ------------------------------------------------------------------ */

/* src/indices_norm.F90:53 nwords = n(n+1)(n+2)(n+3)/24 */
int64_t nvpt_nwords(int64_t nact);

/* src/ord_utils.F90:71 ord8, applied on the device to `count` 8-tuples
 * (1-based, row of 8 per tuple); out8 receives (i1..i8) per tuple and
 * lindex receives lindice(i1,i2,i3,i4) (src/indices_norm.F90:64). */
int nvpt_ord8(nvpt_context *ctx, int64_t nact, int64_t count, const int64_t *in8, int64_t *out8, int64_t *lindex);
/* src/ord_utils.F90:16 ord9 (same arguments as nvpt_ord8): exchange-sort
 * variant, not called on the Koopmans/NEVPT2 path, kept bit-exact. */
int nvpt_ord9(nvpt_context *ctx, int64_t nact, int64_t count, const int64_t *in8, int64_t *out8, int64_t *lindex);

/* ------------------------------------------------------------------ */
/* Stage 1 (koopro4QD.x): RDM partial traces, integrals, Koopmans.     */
/* ------------------------------------------------------------------ */

/* src/koopro4QD.F90:4881 bro3(ro4,daaa,nact,nele,metat):
 * daaa(s,i,j,k,ii,jj,kk) = sum_l ro4[ord8(i,j,k,l;ii,jj,kk,l)] / (nele-3).
 * daaa is overwritten (the reference driver zeroes it before the call). */
int nvpt_bro3(nvpt_context *ctx, const double *ro4, double *daaa, int64_t nact, int64_t nele, int64_t metat);
/* src/koopro4QD.F90:4961 bro2(daaa,taa,nact,nele,metat) */
int nvpt_bro2(nvpt_context *ctx, const double *daaa, double *taa, int64_t nact, int64_t nele, int64_t metat);
/* src/koopro4QD.F90:5002 bro1(taa,dal,nact,nele,metat) */
int nvpt_bro1(nvpt_context *ctx, const double *taa, double *dal, int64_t nact, int64_t nele, int64_t metat);

/* src/koopro4QD.F90:3900 get_aj_atwo(atwo,nact,ncore,norb,aj) on the
 * Cholesky/DF integral path (src/ijkl_utils.F90:637 ai_cholesky).  The
 * reference reads the integrals from module state; here they are passed:
 * oneint(norb(norb+1)/2) and cholesky_array(nchovec, norb(norb+1)/2). */
int nvpt_get_aj_atwo(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                     const double *oneint, const double *cholesky_array, int64_t nchovec);

/* Symmetry-packed two-electron integrals (the non-Cholesky integral path of
 * readint, src/ijkl_utils.F90:209-262, which supports point-group symmetry).
 *
 * nvpt_ijkl_init: src/infsym.F90:16 initialize_infsym (its = D2h product
 * table, itsym = irrep of every orbital, inactive then active then secondary,
 * irrep by irrep), src/ijkl_utils.F90:111 determine_n2int (ndeb, nad, kt,
 * ni4) and :173 reijkl (num, indic, jndic), built on the device and kept in
 * ctx.  nish/nash/nssh (nsym) are the inactive/active/secondary counts per
 * irrep (inforb), nsym in {1,2,4,8}, norb = their sum <= 4096; *ni4
 * receives the number of stored integrals (the length of twoint).
 * nvpt_ijkl_tables: host copies of the tables (1-based values as in the
 * reference): its (nsym,nsym), itsym (norb), num/indic/jndic
 * (norb(norb+1)/2), ndeb (nsym), nad/kt (nsym(nsym+1)/2); NULL skips one.
 * nvpt_ijkl_set_twoint: the integral list twoint(ni4) that ext2int2nev2int
 * leaves in module state (src/ijkl_utils.F90:232-241), copied to the device.
 * nvpt_ai_twoint: src/ijkl_utils.F90:690 ai_twoint for count quadruples
 * (1-based, 4 per row); symmetry-forbidden integrals are 0.
 * nvpt_get_aj_atwo_twoint: src/koopro4QD.F90:3900 get_aj_atwo with ai ->
 * ai_twoint (src/ijkl_utils.F90:627); norb must be the one of init. */
int nvpt_ijkl_init(nvpt_context *ctx, int64_t nsym, const int64_t *nish, const int64_t *nash, const int64_t *nssh,
                   int64_t *ni4);
int nvpt_ijkl_tables(nvpt_context *ctx, int64_t *its, int64_t *itsym, int64_t *num, int64_t *indic, int64_t *jndic,
                     int64_t *ndeb, int64_t *nad, int64_t *kt);
int nvpt_ijkl_set_twoint(nvpt_context *ctx, const double *twoint);
int nvpt_ai_twoint(nvpt_context *ctx, int64_t count, const int64_t *ijkl, double *out);
int nvpt_get_aj_atwo_twoint(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                            const double *oneint);
int nvpt_get_aj_atwo_twoint_d(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                              const double *oneint, void *stream);

/* src/koop_matrices.F90:16 koop_matrices_ctl(metat,nact,ncore,atwo,daaa,taa,dal,f,aj).
 * The reference writes its results to nevpt.h5; they are returned here in
 * the dataset shapes: ipko1/eako1 (metat,n,n) "1-IPKO"/"1-EAKO";
 * hrdm2 (metat,n^4) "2-HRDM"; ipko2/eako2 (metat,n^4) "2-IPKO"/"2-EAKO";
 * gk0pa/gk0pd (metat,n^4); gk0pf (metat,n,n).  f is in/out scratch of at
 * least (ncore+nact)(ncore+nact+1)/2 elements. */
int nvpt_koop_matrices_ctl(nvpt_context *ctx, int64_t metat, int64_t nact, int64_t ncore, const double *atwo,
                           const double *daaa, const double *taa, const double *dal, double *f, const double *aj,
                           double *ipko1, double *eako1, double *hrdm2, double *ipko2, double *eako2, double *gk0pa,
                           double *gk0pd, double *gk0pf);

/* src/koopro4QD.F90:3974 bamat(amat,atmat,atwo,ro4,daaa,taa,dal,nact,ncore,f,aj,norb,metat,nsym):
 * amat "amatIP", atmat "amatEA", both (metat,n^6).  nsym = 1 is the C1
 * branch (:4008-4104).  nsym > 1 is the symmetry-screened branch
 * (:4105-4228): it needs nvpt_ijkl_init on ctx with the same nsym and norb
 * (the orbital irreps), computes the same dense contractions -- the terms the
 * reference skips carry integrals that vanish by symmetry -- and zeroes the
 * elements the reference never assigns (irreps of ap,bp,cp,a,b,c not
 * multiplying to the totally symmetric one).  With symmetry tables on ctx,
 * nvpt_koop_matrices_ctl likewise applies koop2E's screen
 * (src/koop_matrices.F90:289-351) to the 2-IP/2-EA matrices. */
int nvpt_bamat(nvpt_context *ctx, double *amat, double *atmat, const double *atwo, const double *ro4,
               const double *daaa, const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f,
               const double *aj, int64_t norb, int64_t metat, int64_t nsym);

/* src/koopro4QD.F90:4231 bbmat(atwo,bmat,btmat,daaa,taa,dal,nact,ncore,f,aj,metat) */
int nvpt_bbmat(nvpt_context *ctx, const double *atwo, double *bmat, double *btmat, const double *daaa,
               const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
               int64_t metat);
/* src/koopro4QD.F90:4301 bcmat(atwo,cmat,ctmat,daaa,taa,dal,nact,ncore,f,aj,metat) */
int nvpt_bcmat(nvpt_context *ctx, const double *atwo, double *cmat, double *ctmat, const double *daaa,
               const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
               int64_t metat);
/* src/koopro4QD.F90:4399 bdmat(atwo,dmat,dtmat,taa,dal,nact,ncore,f,aj,metat) */
int nvpt_bdmat(nvpt_context *ctx, const double *atwo, double *dmat, double *dtmat, const double *taa,
               const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj, int64_t metat);

/* ------------------------------------------------------------------ */
/* Device-pointer variants (resident tensors, asynchronous).           */
/* ------------------------------------------------------------------ */
int nvpt_bro3_d(nvpt_context *ctx, const double *ro4, double *daaa, int64_t nact, int64_t nele, int64_t metat,
                void *stream);
int nvpt_bro2_d(nvpt_context *ctx, const double *daaa, double *taa, int64_t nact, int64_t nele, int64_t metat,
                void *stream);
int nvpt_bro1_d(nvpt_context *ctx, const double *taa, double *dal, int64_t nact, int64_t nele, int64_t metat,
                void *stream);
int nvpt_get_aj_atwo_d(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                       const double *oneint, const double *cholesky_array, int64_t nchovec, void *stream);
int nvpt_koop_matrices_ctl_d(nvpt_context *ctx, int64_t metat, int64_t nact, int64_t ncore, const double *atwo,
                             const double *daaa, const double *taa, const double *dal, double *f, const double *aj,
                             double *ipko1, double *eako1, double *hrdm2, double *ipko2, double *eako2,
                             double *gk0pa, double *gk0pd, double *gk0pf, void *stream);
int nvpt_bamat_d(nvpt_context *ctx, double *amat, double *atmat, const double *atwo, const double *ro4,
                 const double *daaa, const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f,
                 const double *aj, int64_t norb, int64_t metat, int64_t nsym, void *stream);
int nvpt_bbmat_d(nvpt_context *ctx, const double *atwo, double *bmat, double *btmat, const double *daaa,
                 const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
                 int64_t metat, void *stream);
int nvpt_bcmat_d(nvpt_context *ctx, const double *atwo, double *cmat, double *ctmat, const double *daaa,
                 const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
                 int64_t metat, void *stream);
int nvpt_bdmat_d(nvpt_context *ctx, const double *atwo, double *dmat, double *dtmat, const double *taa,
                 const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj, int64_t metat,
                 void *stream);

/* src/rdm_utils.F90:236 permute_4rdm / :470 permute_3rdm as applied by
 * hdf5_read_rdm_from_resfile (:193-226) to a QCMaquis label/value list:
 * labels are the file's 0-based int32 indices, label-major (8 per entry for
 * the 4-RDM, 6 for the 3-RDM), values the entries in file order.  Every
 * entry writes its images (assignments; a later entry overwrites an earlier
 * one) into ro4(W,n,n,n,n) of one state, or into the 3-RDM element
 * (i,j,k,l,m,n) at rdm3[ld*((i-1)+n((j-1)+...))] (ld = metat for daaa(s,...)
 * with rdm3 pointing at the state's first element).  trans != 0: transition
 * 3-RDM (6 images, value not negated).  Elements no entry writes keep their
 * values.  A label outside [0,nact) returns NVPT_EINVAL. */
int nvpt_permute_4rdm(nvpt_context *ctx, double *ro4, int64_t nact, const int32_t *labels, const double *values,
                      int64_t nentries);
int nvpt_permute_3rdm(nvpt_context *ctx, double *rdm3, int64_t ld, int64_t nact, const int32_t *labels,
                      const double *values, int64_t nentries, int trans);
int nvpt_permute_4rdm_d(nvpt_context *ctx, double *ro4, int64_t nact, const int32_t *labels, const double *values,
                        int64_t nentries, void *stream);
int nvpt_permute_3rdm_d(nvpt_context *ctx, double *rdm3, int64_t ld, int64_t nact, const int32_t *labels,
                        const double *values, int64_t nentries, int trans, void *stream);

/* Dataset container for the path's files (no counterpart in the reference's
 * code; it stands in for HDF5 where libhdf5 is absent).  Datasets keep the
 * HDF5 names of the reference -- nevpt.h5 ("amatIP", "1-IPKO", "3-RDM", ...,
 * src/koopro4QD.F90:305,369-418,473-477, src/qdnevpt.F:792-853) and the
 * QCMaquis result datasets "/spectrum/results/fourptdm/labels_num" (int32,
 * (8, nentries)) and ".../mean/value" (float64, (nentries)) -- with their
 * element type (1 int32, 2 int64, 3 float64) and Fortran-order dims.
 * nvpt_h5c_write creates the file (append = 0) or adds a dataset to it
 * (append != 0; a later dataset of the same name replaces an earlier one);
 * nvpt_h5c_info gives type, rank (<= 8) and dims; nvpt_h5c_read copies the
 * payload (nbytes must match).  NVPT_EINVAL if the dataset is absent,
 * NVPT_EIO if the file is missing or not a container. */
int nvpt_h5c_write(const char *path, const char *name, int type, int rank, const int64_t *dims, const void *data,
                   int append);
int nvpt_h5c_info(const char *path, const char *name, int *type, int *rank, int64_t *dims);
int nvpt_h5c_read(const char *path, const char *name, void *data, int64_t nbytes);
/* Sorted names in a directory, newline-separated, into buf (len bytes);
 * returns the length the full list needs, or -1 if dir cannot be opened. */
int nvpt_h5c_list_dir(const char *path, char *buf, int64_t len);

/* src/rdm_utils.F90:69 hdf5_read_rdm_from_resfile on a container file: the
 * label/value lists of the 4-RDM (which = 4, into ro4(W,n,n,n,n) of one
 * state, as nvpt_permute_4rdm) or the (transition, trans != 0) 3-RDM
 * (which = 3, element stride ld, as nvpt_permute_3rdm); the reference's
 * checks (8 or 6 labels per entry, label/value count match) give
 * NVPT_EINVAL with its message.  *read_num_elements receives nentries. */
int nvpt_read_rdm_from_resfile(nvpt_context *ctx, const char *path, int which, int trans, double *rdm, int64_t ld,
                               int64_t nact, int64_t *read_num_elements);
/* src/rdm_utils.F90:522 read_distributed_rdm: reads result_name from every
 * subdirectory of dir that holds it, in sorted order, until total_elements
 * entries have been read; fewer gives NVPT_EINVAL. */
int nvpt_read_distributed_rdm(nvpt_context *ctx, const char *dir, const char *result_name, int which, int trans,
                              double *rdm, int64_t ld, int64_t nact, int64_t total_elements);

/* Spin-free RDMs of a determinant-expanded CI vector, on the device (the
 * role of src/koopro4QD.F90:921 rofour, :1571 ro3, :2412 ro2, :2861 ro1 and
 * the transition variants ro3off :1978, ro2off :2620, ro1off :2936, for CI
 * vectors given as determinant lists).  Determinant I is the bitmask pair
 * amask[I], bmask[I] (bit p = active orbital p occupied), creators in
 * ascending spin-orbital order with all alpha before all beta; coef is
 * (ndet, nroot) column-major; all pointers are device pointers.
 * nvpt_rdm_dense_d adds the k-RDM (k = 1, 2, 3) of bra root s and ket root t
 * to out[slot + ldo (P1 + n P2 + ... + n^(2k-1) Q_k)] -- the reference's
 * dal/taa/daaa(s,...) layouts with ldo = metat, slot = the state (or the
 * pair index for transition matrices): dal(i,j) = <E_ij>, taa(i,j,k,l) =
 * sum <a+_i a+_j a_l a_k>, daaa(i,j,k,l,m,n) = sum <a+_i a+_j a+_k a_n a_m a_l>.
 * nvpt_rofour_d adds the packed 4-RDM of root s to ro4_s (W x n^4, the
 * state's slice of ro4), every slot (ind(K), L) with normind(L) <=
 * normind(K); other slots are not touched.  Both read out/ro4_s, so the
 * caller zeroes them first. */
int nvpt_rdm_dense_d(nvpt_context *ctx, int64_t nact, int64_t k, int64_t ndet, const uint32_t *amask,
                     const uint32_t *bmask, const double *coef, int64_t nroot, int64_t s, int64_t t, double *out,
                     int64_t ldo, int64_t slot, void *stream);
int nvpt_rofour_d(nvpt_context *ctx, int64_t nact, int64_t ndet, const uint32_t *amask, const uint32_t *bmask,
                  const double *coef, int64_t nroot, int64_t s, double *ro4_s, void *stream);

/* Precision of the dense contractions of later calls on ctx (no counterpart
 * in the reference).  NVPT_PRECISION_FP64 (the default) is the drop-in.
 * NVPT_PRECISION_SPLIT runs the n^9 slab products of bamat, and in
 * nvpt_qdnevpt the large products (DF integral blocks, metric and Koopmans
 * builds, numerators), as Ozaki digit products on the tensor cores: each
 * FP64 operand row/column is scaled by a power of two, rounded to 60 bits and
 * cut into ten 6-bit digits held exactly in BF16, every digit pair with
 * weight >= 2^-72 is summed exactly in FP32, and the partial products are
 * recombined in integer and FP64 arithmetic (error about 2^-59..2^-61 of the
 * row/column maximum per product).  Eigensolves, pseudo-inverses,
 * triangular solves, denominators and energy sums always run in FP64. */
#define NVPT_PRECISION_FP64 0
#define NVPT_PRECISION_SPLIT 1
int nvpt_set_precision(nvpt_context *ctx, int precision);
int nvpt_get_precision(nvpt_context *ctx);

/* Live kernel timing (no counterpart in the reference).  While enabled
 * (process-wide), tagged launches are bracketed by CUDA events on their
 * stream; nvpt_profile_read waits for and sums the spans of one tag (total
 * ms, launch count, algorithmic bytes) and forgets them.  Tags: "oz_gemm"
 * (the skinny split-precision product kernel), "oz_wide" (the general one;
 * its bytes field holds the product's FP64 flops 2 m n k), "s2_prepare" (stage-2 orbitals and
 * transformed integrals of one state), "s2_class_0", "s2_class_+1",
 * "s2_class_-1", "s2_class_+2", "s2_class_-2", "s2_class_0p",
 * "s2_class_+1p", "s2_class_-1p" (one class of one state, on its stream);
 * "pencil_potrf", "pencil_reduce", "pencil_sytrd", "pencil_rhs",
 * "pencil_solve" (the steps of one order-n^3 PC pencil: metric Cholesky,
 * reduction to standard form, tridiagonalisation, right-hand sides and the
 * per-label tridiagonal solves). */
int nvpt_set_profiling(nvpt_context *ctx, int on);
int nvpt_profile_read(nvpt_context *ctx, const char *tag, double *ms, int64_t *launches, int64_t *bytes);

/* Polls a device-side wait (the grid barriers of the order-n^3 pencil
 * tridiagonalisation, in nvpt_sytrd_d and nvpt_qdnevpt) makes before it
 * gives up on ctx; 0 (the default) restores the built-in limit of 2^22
 * polls with back-off (about 0.4 s).  A wait that gives up makes the kernel
 * return, and the call returns NVPT_ETIMEDOUT with the context still usable.
 * No counterpart in the reference; for callers that want a tighter bound. */
int nvpt_set_wait_limit(nvpt_context *ctx, int64_t polls);

/* Route of the PC classes in nvpt_qdnevpt (no counterpart in the reference,
 * which always diagonalises).  mode 0 (default): the order-n^3 metrics of
 * the (+-1') classes (order >= 512) are evaluated as resolvents of the pencil
 * K v = w S v when every metric eigenvalue is kept; the other classes follow
 * the reference's eigenpair sequence.  mode 1: every PC class whose metric
 * keeps all eigenvalues (the (+-2), (0') and (+-1') metrics of any order)
 * takes the resolvent route -- closer to the exact sums on near-singular
 * denominators, and slower: the small pencils add FP64 triangular solves on
 * every label and grid-synchronised tridiagonalisations that compete with
 * the large ones. */
int nvpt_set_pc_route(nvpt_context *ctx, int mode);

/* Autotuning of launch parameters (no counterpart in the reference).  With
 * on = 1, the first call that meets a new shape of a tuned kernel times
 * every candidate of its parameter with CUDA events on the call's stream
 * (synchronising that stream once) and keeps the fastest; later launches of
 * that shape use the kept choice whether tuning is on or not (on = 0 stops
 * tuning new shapes, on = 2 forgets every choice).  Tuned today: the tile
 * height of the FP64 bamat slab products (64 or 128 rows) and the raster
 * group of the general split-precision product (4 .. 32 row tiles sharing a
 * column tile).  Candidates only reorder independent output tiles, so the
 * results do not depend on the choice.  Choices are per device and shared by
 * the contexts of a process.  nvpt_autotune_report writes them as JSON
 * (choice and the timed milliseconds per candidate) into buf (len bytes,
 * NUL-terminated) and returns the length the full text needs. */
int nvpt_set_autotune(nvpt_context *ctx, int on);
int64_t nvpt_autotune_report(nvpt_context *ctx, char *buf, int64_t len);

/* The split-precision product as a building block (no counterpart in the
 * reference): row-major C[m,n] = A[m,k] B[k,n] on device pointers, with
 * n <= 16 and k <= 4096 (the exactness limit of the FP32 digit sums). */
int nvpt_dgemm_split_d(nvpt_context *ctx, int64_t m, int64_t n, int64_t k, const double *A, const double *B,
                       double *C, void *stream);

/* The general split-precision product (no counterpart in the reference):
 * row-major C[m,n] = alpha op(A) op(B) + beta C on device pointers, op(A) =
 * A[m,k] (ld lda) or, with transa, A^T for A[k,m]; op(B) = B[k,n] (ld ldb)
 * or, with transb, B^T for B[n,k].  Any m, n >= 1 and 1 <= k <= 2^19;
 * alpha must be +-2^e (it is folded into the digit exponents).  Each term
 * carries at most 2^-59 max|row of op(A)| max|column of op(B)| of error,
 * at or below an FP64 dot product's rounding.  NVPT_ETIMEDOUT if the
 * product's pipeline timed out. */
int nvpt_dgemm_split_ex_d(nvpt_context *ctx, int transa, int transb, int64_t m, int64_t n, int64_t k, double alpha,
                          const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                          int64_t ldc, void *stream);

/* Householder tridiagonalisation on the device (no counterpart in the reference;
 * the building block of the order-n^3 PC pencils of stage 2): A (n x n,
 * column-major, symmetric, both triangles) -> d[n], e[n-1], tau[n-1] and the
 * reflectors below the subdiagonal of A, in the output form of LAPACK
 * dsytrd('L'): the diagonal and subdiagonal of A hold T (so that a
 * dormtr('L') applies Q).  FP64 throughout.  NVPT_ETIMEDOUT if a grid
 * barrier timed out. */
int nvpt_sytrd_d(nvpt_context *ctx, int64_t n, double *A, double *d, double *e, double *tau, void *stream);

/* No-allocation variant of nvpt_bamat_d -- no counterpart in the reference.
 * Same arguments and results (to rounding: its contractions sum in another
 * order), for callers that must not allocate device memory during a run:
 * a driver whose device memory is budgeted up front by another owner of the
 * pool, or one for which an allocation failure in the middle of a Koopmans
 * pass is not acceptable.  All scratch is one file-scope device array sized
 * for nact <= 8 (4n^6 + 7n^4 + n^2 doubles at n = 8, 8.6 MB); larger nact
 * returns NVPT_EINVAL.  It calls no cudaMalloc/cudaFree and no allocating
 * library routine.  Every call must be made with the context's device
 * current (otherwise NVPT_EINVAL): the array has one address per device.
 * That address is looked up on the first call on a device, which should
 * precede any stream capture.  No scratch word has to start at zero.  Calls
 * that overlap in time share the array and race: serialise them (one stream,
 * or events). */
int nvpt_bamat_static_d(nvpt_context *ctx, double *amat, double *atmat, const double *atwo, const double *ro4,
                        const double *daaa, const double *taa, const double *dal, int64_t nact, int64_t ncore,
                        double *f, const double *aj, int64_t norb, int64_t metat, int64_t nsym, void *stream);


/* ------------------------------------------------------------------ */
/* Stage 2 (QDnevpt2.x): SC/PC-NEVPT2 energies of every state.          */
/* ------------------------------------------------------------------ */

/* Inputs of src/qdnevpt.F:15 qdnevpt for the Cholesky integral path with C1
 * symmetry: the integrals (what readint leaves in module state) and the
 * nevpt.h5 datasets stage 1 wrote, in their reference shapes and Fortran
 * layouts (state index first).  class_mask selects perturber classes
 * (bit 0 (0), 1 (+1), 2 (-1), 3 (+2), 4 (-2), 5 (+1)', 6 (-1)', 7 (0)');
 * 0xFF runs all of them, the reference's order.  frozen (optional, NULL =
 * none) marks frozen core orbitals (.FROZEN, zgel) with a nonzero byte per
 * orbital.  trdm1..3 ("1-TRDM".."3-TRDM", (P,n^k), P = metat(metat-1)/2)
 * are required when metat > 1. */
typedef struct {
    int64_t ncore, nact, nvirt, metat, nchovec;
    double thr_lindep;                 /* .LINDEP (default 1e-6)         */
    int64_t no_pc;                     /* .NO PC                          */
    int64_t class_mask;
    const unsigned char *frozen;
    const double *oneint;              /* norb(norb+1)/2                  */
    const double *cholesky_array;      /* (nchovec, norb(norb+1)/2)       */
    const double *rdm1, *rdm2, *rdm3, *hrdm2;
    const double *ipko1, *eako1, *ipko2, *eako2;
    const double *gk0pa, *gk0pd, *gk0pf;
    const double *amat_ip, *amat_ea, *bmat_ip, *bmat_ea, *cmat_ip, *cmat_ea, *dmat_ip, *dmat_ea;
    const double *trdm1, *trdm2, *trdm3;
} nvpt_qdnevpt_in;

/* Outputs, host arrays the caller owns (any may be NULL): the COMMON
 * /PERTURBER/ per-class energies and norms e2mpp/psimpp (SC) and
 * e2enp/psienep (PC), (8, metat) column-major; the second-order effective
 * Hamiltonians e2mp (SC) and e2en (PC), (metat, metat), before the reference
 * energies are added to the diagonal (src/qdnevpt.F:1050); the norms
 * psimp/psien (metat); epsnew (norb, metat), the canonical core and virtual
 * orbital energies; nnew (10, metat), the PC metric ranks of classes
 * (+1), (-1), (+2)a, (+2)b, (-2)a, (-2)b, (+1)', (-1)', (0)' (-1 if not run). */
typedef struct {
    double *e2mpp, *psimpp, *e2enp, *psienep;
    double *e2mp, *e2en, *psimp, *psien, *epsnew;
    int64_t *nnew;
    /* .NATORB (compute_rho1st): the first-order density blocks of the PC
     * classes in the canonical orbitals, Fortran order with the state last:
     * rhoir (ncore, nvirt, metat) from (0') (src/qdnevpt.F:4971), rhoid
     * (ncore, nact, metat) from (+1') (:5187), rhodr (nact, nvirt, metat)
     * from (-1') (:5407).  Any non-NULL pointer makes the call form all three;
     * the reference writes them to its RHOFILE and assembles the density at
     * :1240-1300.  The canonical orbitals' signs are the device eigensolver's
     * choice: a block's row or column may differ in sign from another
     * eigensolver's result, the density's eigenvalues do not. */
    double *rhoir, *rhoid, *rhodr;
} nvpt_qdnevpt_out;

/* src/qdnevpt.F:858-993, the per-state loop of qdnevpt (integral transforms,
 * core/virtual Fock eigensolves and the eight classes), for every state.
 * The QD effective-Hamiltonian diagonalisation (:1010-1230, metat x metat)
 * stays with the caller. */
int nvpt_qdnevpt(nvpt_context *ctx, const nvpt_qdnevpt_in *in, nvpt_qdnevpt_out *out);
/* Same with device pointers in `in` (outputs still on the host). */
int nvpt_qdnevpt_d(nvpt_context *ctx, const nvpt_qdnevpt_in *in, nvpt_qdnevpt_out *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NVPT2_H */
