// C ABI of the library (include/nvpt2.h): context handling, argument checks,
// host<->device staging for the drop-in host-pointer entry points, and the
// device-pointer (_d) entry points that enqueue the kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/nvpt2.h"
#include "nvpt2_internal.h"
#include "ozaki.cuh"
#include "tuner.h"

namespace nvpt {
std::atomic<long long> g_launches{0};

namespace {
std::atomic<bool> g_prof{false};
struct ProfRecord {
    std::string tag;
    cudaEvent_t a, b;
    long long bytes;
};
std::mutex g_prof_mu;
std::vector<ProfRecord> g_prof_rec;
}  // namespace

bool prof_enabled() { return g_prof.load(std::memory_order_relaxed); }

void ProfSpan::begin(const char *t, cudaStream_t s, long long nbytes) {
    if (!prof_enabled()) return;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        a = b = nullptr;
        return;
    }
    tag = t;
    st = s;
    bytes = nbytes;
    cudaEventRecord(a, s);
}

void ProfSpan::end() {
    if (!a) return;
    cudaEventRecord(b, st);
    std::lock_guard<std::mutex> g(g_prof_mu);
    g_prof_rec.push_back(ProfRecord{tag, a, b, bytes});
    a = b = nullptr;
}

// src/ord_utils.F90:71 ord8 over a batch of tuples (bit-exactness tests).
__global__ void k_ord8(const int64_t *in8, int64_t *out8, int64_t *lindex, long long count) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t *x = in8 + 8 * t;
    int q0, q1, q2, q3;
    int a1 = (int)x[0], c1 = (int)x[1], e1 = (int)x[2], g1 = (int)x[3];
    int a2 = (int)x[4], c2 = (int)x[5], e2 = (int)x[6], g2 = (int)x[7];
    int ind = ord8_key(a1, c1, e1, g1, a2, c2, e2, g2, q0, q1, q2, q3);
    // recover the sorted key from the packed index: the key group is the one
    // with the larger normind (first on ties), sorted descending
    int k[4];
    if (normind4(a1, c1, e1, g1) >= normind4(a2, c2, e2, g2)) { k[0] = a1; k[1] = c1; k[2] = e1; k[3] = g1; }
    else { k[0] = a2; k[1] = c2; k[2] = e2; k[3] = g2; }
    for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j)
            if (k[j] > k[i]) { int tt = k[i]; k[i] = k[j]; k[j] = tt; }
    out8[8 * t + 0] = k[0]; out8[8 * t + 1] = k[1]; out8[8 * t + 2] = k[2]; out8[8 * t + 3] = k[3];
    out8[8 * t + 4] = q0; out8[8 * t + 5] = q1; out8[8 * t + 6] = q2; out8[8 * t + 7] = q3;
    lindex[t] = ind;
}

// src/ord_utils.F90:16 ord9 over a batch of tuples.
__global__ void k_ord9(const int64_t *in8, int64_t *out8, int64_t *lindex, long long count) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int64_t *x = in8 + 8 * t;
    int o[8];
    int ind = ord9_key((int)x[0], (int)x[1], (int)x[2], (int)x[3], (int)x[4], (int)x[5], (int)x[6], (int)x[7], o[0],
                       o[1], o[2], o[3], o[4], o[5], o[6], o[7]);
    for (int i = 0; i < 8; ++i) out8[8 * t + i] = o[i];
    lindex[t] = ind;
}

void launch_ord8(const int64_t *in8, int64_t *out8, int64_t *lindex, long long count, cudaStream_t st) {
    k_ord8<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(in8, out8, lindex, count);
    g_launches.fetch_add(1, std::memory_order_relaxed);
}
}  // namespace nvpt

using namespace nvpt;

// Device tables of the symmetry-packed integral path (nvpt_ijkl_init) and
// the integral list (nvpt_ijkl_set_twoint), owned by the context.
struct IjklState {
    int nsym = 0, norb = 0;
    long long ni4 = -1;
    long long *tab = nullptr;  // its | itsym | num | indic | jndic | ndeb | nad | kt
    double *twoint = nullptr;
    long long npair() const { return (long long)norb * (norb + 1) / 2; }
    long long *its() const { return tab; }
    long long *itsym() const { return tab + nsym * nsym; }
    long long *num() const { return itsym() + norb; }
    long long *indic() const { return num() + npair(); }
    long long *jndic() const { return indic() + npair(); }
    long long *ndeb() const { return jndic() + npair(); }
    long long *nad() const { return ndeb() + nsym; }
    long long *kt() const { return nad() + nsym * (nsym + 1) / 2; }
    long long total() const { return nsym * nsym + norb + 3 * npair() + nsym + nsym * (nsym + 1) + 2; }
    void release() {
        if (tab) cudaFree(tab);
        if (twoint) cudaFree(twoint);
        tab = nullptr;
        twoint = nullptr;
        ni4 = -1;
    }
};

struct nvpt_context {
    int device = 0;
    int precision = NVPT_PRECISION_FP64;
    cudaStream_t stream = nullptr;
    std::string err;
    long long launches_at_create = 0;
    IjklState ijkl;
    unsigned wait_limit = 0;  // nvpt_set_wait_limit (0 = built-in)
    int pc_route = 0;         // nvpt_set_pc_route
};

namespace {

const int64_t kMaxNact = 16;  // packed-index arithmetic and generator limits

int fail(nvpt_context *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_check(nvpt_context *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return NVPT_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(ctx, e == cudaErrorMemoryAllocation ? NVPT_ENOMEM : NVPT_ECUDA, m);
}

#define NV_TRY(expr)                 \
    do {                             \
        int _st = (expr);            \
        if (_st != NVPT_OK) return _st; \
    } while (0)

cudaStream_t pick(nvpt_context *ctx, void *stream) { return stream ? (cudaStream_t)stream : ctx->stream; }

int check_nact(nvpt_context *ctx, int64_t nact, int64_t metat) {
    if (!ctx) return NVPT_EINVAL;
    if (nact < 1 || nact > kMaxNact) return fail(ctx, NVPT_EINVAL, "nact must be in [1,16]");
    if (metat < 1 || metat > 64) return fail(ctx, NVPT_EINVAL, "metat must be in [1,64]");
    return NVPT_OK;
}

int after_launch(nvpt_context *ctx, const char *what) { return cuda_check(ctx, cudaGetLastError(), what); }

Rdm make_rdm(int64_t n, int64_t M, const double *d1, const double *d2, const double *d3, const double *ro4) {
    Rdm r;
    r.n = (int)n;
    r.M = (int)M;
    r.W = n * (n + 1) * (n + 2) * (n + 3) / 24;
    r.d1 = d1; r.d2 = d2; r.d3 = d3; r.ro4 = ro4;
    return r;
}

int64_t ipow(int64_t b, int e) {
    int64_t r = 1;
    for (int i = 0; i < e; ++i) r *= b;
    return r;
}

int64_t f_len(int64_t nact, int64_t ncore) { return (ncore + nact) * (ncore + nact + 1) / 2; }

// Stream-ordered device staging area for one host-pointer call.
struct Stage {
    nvpt_context *ctx;
    cudaStream_t st;
    std::vector<void *> bufs;
    int status = NVPT_OK;
    Stage(nvpt_context *c) : ctx(c), st(c->stream) {}
    ~Stage() {
        for (void *p : bufs) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
    }
    double *alloc(int64_t count) {
        if (status != NVPT_OK) return nullptr;
        void *p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, sizeof(double) * (size_t)(count > 0 ? count : 1), st);
        if (e != cudaSuccess) { status = cuda_check(ctx, e, "cudaMallocAsync"); return nullptr; }
        bufs.push_back(p);
        return (double *)p;
    }
    double *up(const double *h, int64_t count) {
        double *d = alloc(count);
        if (!d) return nullptr;
        cudaError_t e = cudaMemcpyAsync(d, h, sizeof(double) * (size_t)count, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) { status = cuda_check(ctx, e, "H2D copy"); return nullptr; }
        return d;
    }
    void *up_bytes(const void *h, size_t bytes) {
        if (status != NVPT_OK) return nullptr;
        void *p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, bytes > 0 ? bytes : 1, st);
        if (e != cudaSuccess) { status = cuda_check(ctx, e, "cudaMallocAsync"); return nullptr; }
        bufs.push_back(p);
        e = cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) { status = cuda_check(ctx, e, "H2D copy"); return nullptr; }
        return p;
    }
    int down(double *h, const double *d, int64_t count) {
        if (status != NVPT_OK) return status;
        cudaError_t e = cudaMemcpyAsync(h, d, sizeof(double) * (size_t)count, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) status = cuda_check(ctx, e, "D2H copy");
        return status;
    }
    int finish() {
        if (status != NVPT_OK) return status;
        return cuda_check(ctx, cudaStreamSynchronize(st), "stream synchronize");
    }
};

}  // namespace

extern "C" {

int nvpt_create(nvpt_context **out, int device) {
    if (!out) return NVPT_EINVAL;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return NVPT_ECUDA;
    if (device < 0 || device >= ndev) return NVPT_EINVAL;
    nvpt_context *ctx = new nvpt_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return NVPT_ECUDA;
    }
    // The library's scratch comes from the device's default stream-ordered
    // pool.  Its default release threshold (0) hands every freed byte back to
    // the driver at each synchronisation, so the many allocate / synchronise /
    // free cycles of a call (solver info words, eigenvalue read-backs) remap
    // GBs of device memory again and again.  Keep freed memory in the pool;
    // cudaMemPoolTrimTo returns it when the caller wants it back.
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess && pool) {
        unsigned long long keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    ctx->launches_at_create = g_launches.load();
    *out = ctx;
    return NVPT_OK;
}

int nvpt_destroy(nvpt_context *ctx) {
    if (!ctx) return NVPT_EINVAL;
    cudaStreamSynchronize(ctx->stream);
    ctx->ijkl.release();
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return NVPT_OK;
}

int nvpt_synchronize(nvpt_context *ctx) {
    if (!ctx) return NVPT_EINVAL;
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "stream synchronize");
}

const char *nvpt_last_error(const nvpt_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

const char *nvpt_status_string(int status) {
    switch (status) {
        case NVPT_OK: return "ok";
        case NVPT_EINVAL: return "invalid argument";
        case NVPT_ECUDA: return "CUDA error";
        case NVPT_ENOMEM: return "device allocation failed";
        case NVPT_ENOTSUP: return "unsupported configuration";
        case NVPT_ETIMEDOUT: return "device wait timed out";
        case NVPT_EIO: return "file error";
        default: return "unknown status";
    }
}

const char *nvpt_context_error_set(nvpt_context *ctx, const char *msg) {
    if (!ctx) return "";
    ctx->err = msg ? msg : "";
    return ctx->err.c_str();
}

void *nvpt_context_stream(nvpt_context *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

unsigned nvpt_context_wait_limit(const nvpt_context *ctx) { return ctx ? ctx->wait_limit : 0u; }

int nvpt_set_wait_limit(nvpt_context *ctx, int64_t polls) {
    if (!ctx || polls < 0 || polls > 0xffffffffLL) return NVPT_EINVAL;
    ctx->wait_limit = (unsigned)polls;
    return NVPT_OK;
}

int nvpt_context_pc_route(const nvpt_context *ctx) { return ctx ? ctx->pc_route : 0; }

int nvpt_set_pc_route(nvpt_context *ctx, int mode) {
    if (!ctx || mode < 0 || mode > 1) return NVPT_EINVAL;
    ctx->pc_route = mode;
    return NVPT_OK;
}

int64_t nvpt_launch_count(const nvpt_context *ctx) { return ctx ? g_launches.load() - ctx->launches_at_create : 0; }

int nvpt_set_autotune(nvpt_context *ctx, int on) {
    if (!ctx) return NVPT_EINVAL;
    if (on == 2) {
        tune::clear();
        return NVPT_OK;
    }
    tune::set_enabled(on != 0);
    return NVPT_OK;
}

int64_t nvpt_autotune_report(nvpt_context *ctx, char *buf, int64_t len) {
    if (!ctx) return -1;
    const std::string r = tune::report();
    if (buf && len > 0) {
        const size_t k = std::min((size_t)(len - 1), r.size());
        memcpy(buf, r.data(), k);
        buf[k] = 0;
    }
    return (int64_t)r.size() + 1;
}

int64_t nvpt_nwords(int64_t nact) { return nact * (nact + 1) * (nact + 2) * (nact + 3) / 24; }

int nvpt_ord8(nvpt_context *ctx, int64_t nact, int64_t count, const int64_t *in8, int64_t *out8, int64_t *lindex) {
    NV_TRY(check_nact(ctx, nact, 1));
    if (count < 0 || (count > 0 && (!in8 || !out8 || !lindex))) return fail(ctx, NVPT_EINVAL, "ord8: bad buffers");
    for (int64_t i = 0; i < 8 * count; ++i)
        if (in8[i] < 1 || in8[i] > nact) return fail(ctx, NVPT_EINVAL, "ord8: index outside [1,nact]");
    if (count == 0) return NVPT_OK;
    cudaStream_t st = ctx->stream;
    int64_t *d = nullptr;
    size_t bytes = sizeof(int64_t) * (size_t)count * 17;
    NV_TRY(cuda_check(ctx, cudaMallocAsync((void **)&d, bytes, st), "cudaMallocAsync"));
    cudaMemcpyAsync(d, in8, sizeof(int64_t) * 8 * count, cudaMemcpyHostToDevice, st);
    launch_ord8(d, d + 8 * count, d + 16 * count, count, st);
    int rc = after_launch(ctx, "ord8 launch");
    cudaMemcpyAsync(out8, d + 8 * count, sizeof(int64_t) * 8 * count, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(lindex, d + 16 * count, sizeof(int64_t) * count, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    int rc2 = cuda_check(ctx, cudaStreamSynchronize(st), "ord8 sync");
    return rc != NVPT_OK ? rc : rc2;
}

int nvpt_ord9(nvpt_context *ctx, int64_t nact, int64_t count, const int64_t *in8, int64_t *out8, int64_t *lindex) {
    NV_TRY(check_nact(ctx, nact, 1));
    if (count < 0 || (count > 0 && (!in8 || !out8 || !lindex))) return fail(ctx, NVPT_EINVAL, "ord9: bad buffers");
    for (int64_t i = 0; i < 8 * count; ++i)
        if (in8[i] < 1 || in8[i] > nact) return fail(ctx, NVPT_EINVAL, "ord9: index outside [1,nact]");
    if (count == 0) return NVPT_OK;
    cudaStream_t st = ctx->stream;
    int64_t *d = nullptr;
    size_t bytes = sizeof(int64_t) * (size_t)count * 17;
    NV_TRY(cuda_check(ctx, cudaMallocAsync((void **)&d, bytes, st), "cudaMallocAsync"));
    cudaMemcpyAsync(d, in8, sizeof(int64_t) * 8 * count, cudaMemcpyHostToDevice, st);
    k_ord9<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(d, d + 8 * count, d + 16 * count, count);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    int rc = after_launch(ctx, "ord9 launch");
    cudaMemcpyAsync(out8, d + 8 * count, sizeof(int64_t) * 8 * count, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(lindex, d + 16 * count, sizeof(int64_t) * count, cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    int rc2 = cuda_check(ctx, cudaStreamSynchronize(st), "ord9 sync");
    return rc != NVPT_OK ? rc : rc2;
}

// ----------------------------------------------------------------- _d entries
int nvpt_bro3_d(nvpt_context *ctx, const double *ro4, double *daaa, int64_t nact, int64_t nele, int64_t metat,
                void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    if (nele <= 3) return fail(ctx, NVPT_EINVAL, "bro3 needs nele > 3 (it divides by nele-3)");
    Rdm r = make_rdm(nact, metat, nullptr, nullptr, nullptr, ro4);
    if (launch_bro3(r, daaa, (int)nele, pick(ctx, stream)) != 0)
        return fail(ctx, NVPT_ENOMEM, "bro3: device allocation failed");
    return after_launch(ctx, "bro3");
}

int nvpt_bro2_d(nvpt_context *ctx, const double *daaa, double *taa, int64_t nact, int64_t nele, int64_t metat,
                void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    if (nele <= 2) return fail(ctx, NVPT_EINVAL, "bro2 needs nele > 2");
    Rdm r = make_rdm(nact, metat, nullptr, nullptr, daaa, nullptr);
    launch_bro2(r, taa, (int)nele, pick(ctx, stream));
    return after_launch(ctx, "bro2");
}

int nvpt_bro1_d(nvpt_context *ctx, const double *taa, double *dal, int64_t nact, int64_t nele, int64_t metat,
                void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    if (nele <= 1) return fail(ctx, NVPT_EINVAL, "bro1 needs nele > 1");
    Rdm r = make_rdm(nact, metat, nullptr, taa, nullptr, nullptr);
    launch_bro1(r, dal, (int)nele, pick(ctx, stream));
    return after_launch(ctx, "bro1");
}

int nvpt_get_aj_atwo_d(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                       const double *oneint, const double *chol, int64_t nchovec, void *stream) {
    NV_TRY(check_nact(ctx, nact, 1));
    if (ncore < 0 || norb < ncore + nact || nchovec < 1) return fail(ctx, NVPT_EINVAL, "get_aj_atwo: bad sizes");
    launch_aj_atwo(oneint, chol, (int)nchovec, (int)nact, (int)ncore, (int)norb, atwo, aj, pick(ctx, stream));
    return after_launch(ctx, "get_aj_atwo");
}

// ------------------------------------------------ RDMs of a CI expansion
static int rdm_args(nvpt_context *ctx, int64_t nact, int64_t ndet, int64_t nroot, int64_t s, int64_t t) {
    if (!ctx) return NVPT_EINVAL;
    if (nact < 1 || nact > 16) return fail(ctx, NVPT_EINVAL, "rdm: nact must be in [1,16]");
    if (ndet < 1 || ndet >= (1LL << 31)) return fail(ctx, NVPT_EINVAL, "rdm: ndet must be in [1, 2^31)");
    if (nroot < 1 || s < 0 || s >= nroot || t < 0 || t >= nroot) return fail(ctx, NVPT_EINVAL, "rdm: bad root");
    return NVPT_OK;
}

int nvpt_rdm_dense_d(nvpt_context *ctx, int64_t nact, int64_t k, int64_t ndet, const uint32_t *amask,
                     const uint32_t *bmask, const double *coef, int64_t nroot, int64_t s, int64_t t, double *out,
                     int64_t ldo, int64_t slot, void *stream) {
    NV_TRY(rdm_args(ctx, nact, ndet, nroot, s, t));
    if (k < 1 || k > 3) return fail(ctx, NVPT_EINVAL, "rdm_dense: k must be 1, 2 or 3");
    if (ldo < 1 || slot < 0 || slot >= ldo) return fail(ctx, NVPT_EINVAL, "rdm_dense: bad ldo/slot");
    const int rc = launch_rdm_dense((int)nact, (int)k, ndet, amask, bmask, coef, (int)s, (int)t, out, ldo, slot,
                                    pick(ctx, stream));
    if (rc == 2) return fail(ctx, NVPT_ENOMEM, "rdm_dense: device allocation failed");
    return after_launch(ctx, "rdm_dense");
}

int nvpt_rofour_d(nvpt_context *ctx, int64_t nact, int64_t ndet, const uint32_t *amask, const uint32_t *bmask,
                  const double *coef, int64_t nroot, int64_t s, double *ro4_s, void *stream) {
    NV_TRY(rdm_args(ctx, nact, ndet, nroot, s, s));
    const int rc = launch_rofour((int)nact, ndet, amask, bmask, coef, (int)s, ro4_s, pick(ctx, stream));
    if (rc == 2) return fail(ctx, NVPT_ENOMEM, "rofour: device allocation failed");
    return after_launch(ctx, "rofour");
}

// ------------------------------------------------ symmetry-packed integrals
int nvpt_ijkl_init(nvpt_context *ctx, int64_t nsym, const int64_t *nish, const int64_t *nash, const int64_t *nssh,
                   int64_t *ni4) {
    if (!ctx) return NVPT_EINVAL;
    if (!(nsym == 1 || nsym == 2 || nsym == 4 || nsym == 8))
        return fail(ctx, NVPT_EINVAL, "ijkl_init: nsym must be 1, 2, 4 or 8 (a D2h subgroup)");
    if (!nish || !nash || !nssh) return fail(ctx, NVPT_EINVAL, "ijkl_init: null orbital counts");
    int64_t norb = 0;
    for (int64_t r = 0; r < nsym; ++r) {
        if (nish[r] < 0 || nash[r] < 0 || nssh[r] < 0) return fail(ctx, NVPT_EINVAL, "ijkl_init: negative count");
        norb += nish[r] + nash[r] + nssh[r];
    }
    if (norb < 1 || norb > 4096) return fail(ctx, NVPT_EINVAL, "ijkl_init: norb must be in [1,4096]");
    if (norb * (norb + 1) / 2 < nsym)
        return fail(ctx, NVPT_EINVAL, "ijkl_init: norb(norb+1)/2 must be at least nsym (num is indexed by irrep)");
    cudaStream_t st = ctx->stream;
    ctx->ijkl.release();
    IjklState &S = ctx->ijkl;
    S.nsym = (int)nsym;
    S.norb = (int)norb;
    // tables + three count vectors + ni4 + the error flag
    const size_t words = (size_t)S.total() + 3 * 8 + 2;
    NV_TRY(cuda_check(ctx, cudaMalloc((void **)&S.tab, sizeof(long long) * words), "cudaMalloc (ijkl tables)"));
    long long *cnt = S.tab + S.total(), *d_ni4 = cnt + 24;
    int *bad = (int *)(d_ni4 + 1);
    long long h[24] = {0};
    for (int64_t r = 0; r < nsym; ++r) {
        h[r] = nish[r];
        h[8 + r] = nash[r];
        h[16 + r] = nssh[r];
    }
    NV_TRY(cuda_check(ctx, cudaMemcpyAsync(cnt, h, sizeof(h), cudaMemcpyHostToDevice, st), "H2D copy"));
    if (launch_ijkl_tables(S.nsym, cnt, cnt + 8, cnt + 16, S.norb, S.its(), S.itsym(), S.num(), S.indic(), S.jndic(),
                           S.ndeb(), S.nad(), S.kt(), d_ni4, bad, st))
        return after_launch(ctx, "ijkl_tables launch");
    long long out[2] = {0, 0};
    NV_TRY(cuda_check(ctx, cudaMemcpyAsync(out, d_ni4, sizeof(out), cudaMemcpyDeviceToHost, st), "D2H copy"));
    NV_TRY(cuda_check(ctx, cudaStreamSynchronize(st), "ijkl_tables"));
    if ((int)out[1] != 0) return fail(ctx, NVPT_EINVAL, "ijkl_init: orbital counts do not add up to norb");
    S.ni4 = out[0];
    if (ni4) *ni4 = S.ni4;
    return NVPT_OK;
}

int nvpt_ijkl_tables(nvpt_context *ctx, int64_t *its, int64_t *itsym, int64_t *num, int64_t *indic, int64_t *jndic,
                     int64_t *ndeb, int64_t *nad, int64_t *kt) {
    if (!ctx) return NVPT_EINVAL;
    const IjklState &S = ctx->ijkl;
    if (S.ni4 < 0) return fail(ctx, NVPT_EINVAL, "ijkl_tables: call nvpt_ijkl_init first");
    const long long np = S.npair(), nj = (long long)S.nsym * (S.nsym + 1) / 2;
    struct { int64_t *h; const long long *d; long long n; } c[] = {
        {its, S.its(), (long long)S.nsym * S.nsym}, {itsym, S.itsym(), S.norb}, {num, S.num(), np},
        {indic, S.indic(), np}, {jndic, S.jndic(), np}, {ndeb, S.ndeb(), S.nsym}, {nad, S.nad(), nj},
        {kt, S.kt(), nj}};
    for (auto &x : c)
        if (x.h)
            NV_TRY(cuda_check(ctx, cudaMemcpyAsync(x.h, x.d, sizeof(int64_t) * x.n, cudaMemcpyDeviceToHost, ctx->stream),
                              "D2H copy"));
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ijkl_tables");
}

int nvpt_ijkl_set_twoint(nvpt_context *ctx, const double *twoint) {
    if (!ctx) return NVPT_EINVAL;
    IjklState &S = ctx->ijkl;
    if (S.ni4 < 0) return fail(ctx, NVPT_EINVAL, "ijkl_set_twoint: call nvpt_ijkl_init first");
    if (!twoint) return fail(ctx, NVPT_EINVAL, "ijkl_set_twoint: null twoint");
    if (!S.twoint)
        NV_TRY(cuda_check(ctx, cudaMalloc((void **)&S.twoint, sizeof(double) * (size_t)(S.ni4 > 0 ? S.ni4 : 1)),
                          "cudaMalloc (twoint)"));
    NV_TRY(cuda_check(ctx, cudaMemcpyAsync(S.twoint, twoint, sizeof(double) * (size_t)S.ni4, cudaMemcpyHostToDevice,
                                           ctx->stream), "H2D copy"));
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "ijkl_set_twoint");
}

static int ijkl_ready(nvpt_context *ctx, const char *what, IjklTables *T) {
    const IjklState &S = ctx->ijkl;
    if (S.ni4 < 0 || !S.twoint)
        return fail(ctx, NVPT_EINVAL, std::string(what) + ": call nvpt_ijkl_init and nvpt_ijkl_set_twoint first");
    *T = IjklTables{S.num(), S.indic(), S.jndic(), S.ndeb(), S.nad(), S.kt(), S.twoint};
    return NVPT_OK;
}

int nvpt_ai_twoint(nvpt_context *ctx, int64_t count, const int64_t *ijkl, double *out) {
    if (!ctx) return NVPT_EINVAL;
    IjklTables T;
    NV_TRY(ijkl_ready(ctx, "ai_twoint", &T));
    if (count < 0 || (count > 0 && (!ijkl || !out))) return fail(ctx, NVPT_EINVAL, "ai_twoint: bad buffers");
    for (int64_t i = 0; i < 4 * count; ++i)
        if (ijkl[i] < 1 || ijkl[i] > ctx->ijkl.norb) return fail(ctx, NVPT_EINVAL, "ai_twoint: index outside [1,norb]");
    if (count == 0) return NVPT_OK;
    Stage sg(ctx);
    const int64_t *d_q = (const int64_t *)sg.up_bytes(ijkl, sizeof(int64_t) * 4 * (size_t)count);
    double *d_o = sg.alloc(count);
    NV_TRY(sg.status);
    launch_ai_twoint(T, count, d_q, d_o, sg.st);
    NV_TRY(after_launch(ctx, "ai_twoint"));
    sg.down(out, d_o, count);
    return sg.finish();
}

int nvpt_get_aj_atwo_twoint_d(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                              const double *oneint, void *stream) {
    NV_TRY(check_nact(ctx, nact, 1));
    IjklTables T;
    NV_TRY(ijkl_ready(ctx, "get_aj_atwo_twoint", &T));
    if (ncore < 0 || norb != ctx->ijkl.norb || norb < ncore + nact)
        return fail(ctx, NVPT_EINVAL, "get_aj_atwo_twoint: norb must be the one of nvpt_ijkl_init and >= ncore+nact");
    launch_aj_atwo_twoint(T, oneint, (int)nact, (int)ncore, (int)norb, atwo, aj, pick(ctx, stream));
    return after_launch(ctx, "get_aj_atwo_twoint");
}

int nvpt_get_aj_atwo_twoint(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                            const double *oneint) {
    NV_TRY(check_nact(ctx, nact, 1));
    if (ncore < 0 || norb < ncore + nact) return fail(ctx, NVPT_EINVAL, "get_aj_atwo_twoint: bad sizes");
    const int64_t npair = norb * (norb + 1) / 2;
    Stage sg(ctx);
    double *d_one = sg.up(oneint, npair), *d_aj = sg.alloc(npair), *d_atwo = sg.alloc(ipow(nact, 4));
    NV_TRY(sg.status);
    NV_TRY(nvpt_get_aj_atwo_twoint_d(ctx, d_atwo, nact, ncore, norb, d_aj, d_one, sg.st));
    sg.down(atwo, d_atwo, ipow(nact, 4));
    sg.down(aj, d_aj, npair);
    return sg.finish();
}

int nvpt_koop_matrices_ctl_d(nvpt_context *ctx, int64_t metat, int64_t nact, int64_t ncore, const double *atwo,
                             const double *daaa, const double *taa, const double *dal, double *f, const double *aj,
                             double *ipko1, double *eako1, double *hrdm2, double *ipko2, double *eako2,
                             double *gk0pa, double *gk0pd, double *gk0pf, void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    if (ncore < 0) return fail(ctx, NVPT_EINVAL, "koop_matrices_ctl: ncore < 0");
    cudaStream_t st = pick(ctx, stream);
    Rdm r = make_rdm(nact, metat, dal, taa, daaa, nullptr);
    int n = (int)nact, nc = (int)ncore;
    launch_build_f(f, aj, atwo, n, nc, 0, st);
    launch_koopE(r, atwo, f, nc, ipko1, eako1, st);
    launch_hrdm(r, hrdm2, st);
    launch_build_f(f, aj, atwo, n, nc, 1, st);
    launch_koop2E(r, atwo, f, nc, ipko2, eako2, st);
    // koop2E's its() screen with the context's symmetry tables (none: C1)
    if (ctx->ijkl.ni4 >= 0 && ctx->ijkl.nsym > 1 && ctx->ijkl.norb >= ncore + nact)
        launch_sym_screen(ipko2, eako2, (int)metat, n, 4, ctx->ijkl.itsym() + ncore, st);
    launch_koop0p(r, atwo, f, nc, gk0pa, gk0pd, gk0pf, st);
    return after_launch(ctx, "koop_matrices_ctl");
}

int nvpt_bamat_d(nvpt_context *ctx, double *amat, double *atmat, const double *atwo, const double *ro4,
                 const double *daaa, const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f,
                 const double *aj, int64_t norb, int64_t metat, int64_t nsym, void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    if (norb < ncore + nact) return fail(ctx, NVPT_EINVAL, "bamat: norb < ncore+nact");
    const long long *irr = nullptr;
    if (nsym != 1) {
        // the symmetry-screened branch: the irreps come from the context's
        // integral tables (nvpt_ijkl_init), the reference's module state
        const IjklState &S = ctx->ijkl;
        if (S.ni4 < 0 || S.nsym != nsym || S.norb != norb)
            return fail(ctx, NVPT_ENOTSUP, "bamat: nsym > 1 needs nvpt_ijkl_init with the same nsym and norb");
        irr = S.itsym() + ncore;
    }
    cudaStream_t st = pick(ctx, stream);
    Rdm r = make_rdm(nact, metat, dal, taa, daaa, ro4);
    launch_build_f(f, aj, atwo, (int)nact, (int)ncore, 1, st);
    // Tiny active spaces: one thread per element evaluates the reference's
    // loop directly.  Otherwise the n^9 part runs as dense GEMMs over
    // materialised four-operator slabs (bamat_gemm.cu).  With symmetry the
    // dense contractions are the same (the integrals the reference's branch
    // skips vanish by symmetry) and its output screen follows.
    if (nact <= 5) {
        launch_bamat_direct(r, atwo, f, (int)ncore, amat, atmat, st);
        if (irr) launch_sym_screen(amat, atmat, (int)metat, (int)nact, 6, irr, st);
        return after_launch(ctx, "bamat");
    }
    const bool split = ctx->precision == NVPT_PRECISION_SPLIT;
    const int slabs = 16;
    int rc = launch_bamat_gemm(r, atwo, f, (int)ncore, amat, atmat, st, slabs, split);
    if (rc == 2) return fail(ctx, NVPT_ENOMEM, "bamat: device allocation failed");
    if (rc == 5) return fail(ctx, NVPT_ETIMEDOUT, "bamat: a split-precision product timed out waiting on its pipeline");
    if (rc) return fail(ctx, NVPT_ECUDA, split ? "bamat: split-precision product failed" : "bamat: GEMM failed");
    if (irr) launch_sym_screen(amat, atmat, (int)metat, (int)nact, 6, irr, st);
    return after_launch(ctx, "bamat");
}

int nvpt_bamat_static_d(nvpt_context *ctx, double *amat, double *atmat, const double *atwo, const double *ro4,
                        const double *daaa, const double *taa, const double *dal, int64_t nact, int64_t ncore,
                        double *f, const double *aj, int64_t norb, int64_t metat, int64_t nsym, void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    if (nact > kBamatStaticNactMax)
        return fail(ctx, NVPT_EINVAL,
                    "bamat_static: nact=" + std::to_string(nact) + " exceeds the static scratch limit of " +
                        std::to_string(kBamatStaticNactMax) + " active orbitals; use nvpt_bamat_d");
    if (nsym != 1) return fail(ctx, NVPT_ENOTSUP, "bamat: only the C1 (nsym=1) path is implemented");
    if (norb < ncore + nact) return fail(ctx, NVPT_EINVAL, "bamat: norb < ncore+nact");
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != ctx->device)
        return fail(ctx, NVPT_EINVAL, "bamat_static: the context's device (" + std::to_string(ctx->device) +
                                          ") must be the current device on every call");
    double *scr = bamat_static_scratch(ctx->device);
    if (!scr) return fail(ctx, NVPT_ECUDA, "bamat_static: scratch address lookup failed");
    cudaStream_t st = pick(ctx, stream);
    Rdm r = make_rdm(nact, metat, dal, taa, daaa, ro4);
    launch_build_f(f, aj, atwo, (int)nact, (int)ncore, 1, st);
    launch_bamat_static(r, atwo, f, (int)ncore, amat, atmat, st, scr);
    return after_launch(ctx, "bamat_static");
}

// Device part of the label/value unfolding: scratch, the two passes, the
// label check.
static int unfold_d(nvpt_context *ctx, int which, double *dst, int64_t ld, int64_t nact, const int32_t *labels,
                    const double *values, int64_t nentries, int trans, cudaStream_t st) {
    NV_TRY(check_nact(ctx, nact, 1));
    if (nentries < 0 || !dst || (nentries > 0 && (!labels || !values)) || ld < 1)
        return fail(ctx, NVPT_EINVAL, "permute_rdm: bad arguments");
    const int64_t n = nact, W = n * (n + 1) * (n + 2) * (n + 3) / 24;
    const int64_t slots = which == 4 ? W * n * n * n * n : n * n * n * n * n * n;
    unsigned long long *owner = nullptr;
    int *bad = nullptr;
    NV_TRY(cuda_check(ctx, cudaMallocAsync((void **)&owner, sizeof(unsigned long long) * slots, st), "permute_rdm"));
    if (cudaMallocAsync((void **)&bad, sizeof(int), st) != cudaSuccess) {
        cudaFreeAsync(owner, st);
        return fail(ctx, NVPT_ENOMEM, "permute_rdm: device allocation failed");
    }
    cudaMemsetAsync(bad, 0, sizeof(int), st);
    int rc = which == 4 ? launch_unfold4(labels, values, nentries, (int)n, dst, owner, bad, st)
                        : launch_unfold3(labels, values, nentries, (int)n, dst, ld, trans != 0, owner, bad, st);
    int hbad = 0;
    if (!rc) {
        cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = 1;
    }
    cudaFreeAsync(bad, st);
    cudaFreeAsync(owner, st);
    if (rc) return cuda_check(ctx, cudaGetLastError(), "permute_rdm");
    if (hbad) return fail(ctx, NVPT_EINVAL, "permute_rdm: a label index is outside [0, nact)");
    return after_launch(ctx, "permute_rdm");
}

int nvpt_permute_4rdm_d(nvpt_context *ctx, double *ro4, int64_t nact, const int32_t *labels, const double *values,
                        int64_t nentries, void *stream) {
    if (!ctx) return NVPT_EINVAL;
    return unfold_d(ctx, 4, ro4, 1, nact, labels, values, nentries, 0, pick(ctx, stream));
}

int nvpt_permute_3rdm_d(nvpt_context *ctx, double *rdm3, int64_t ld, int64_t nact, const int32_t *labels,
                        const double *values, int64_t nentries, int trans, void *stream) {
    if (!ctx) return NVPT_EINVAL;
    return unfold_d(ctx, 3, rdm3, ld, nact, labels, values, nentries, trans, pick(ctx, stream));
}

int nvpt_set_precision(nvpt_context *ctx, int precision) {
    if (!ctx) return NVPT_EINVAL;
    if (precision != NVPT_PRECISION_FP64 && precision != NVPT_PRECISION_SPLIT)
        return fail(ctx, NVPT_EINVAL, "precision must be NVPT_PRECISION_FP64 or NVPT_PRECISION_SPLIT");
    ctx->precision = precision;
    return NVPT_OK;
}

int nvpt_get_precision(nvpt_context *ctx) { return ctx ? ctx->precision : -1; }

int nvpt_set_profiling(nvpt_context *ctx, int on) {
    if (!ctx) return NVPT_EINVAL;
    g_prof.store(on != 0);
    return NVPT_OK;
}

int nvpt_profile_read(nvpt_context *ctx, const char *tag, double *ms, int64_t *launches, int64_t *bytes) {
    if (!ctx || !tag) return NVPT_EINVAL;
    double t = 0.0;
    int64_t n = 0, by = 0;
    std::lock_guard<std::mutex> g(g_prof_mu);
    std::vector<ProfRecord> keep;
    int rc = NVPT_OK;
    for (auto &r : g_prof_rec) {
        if (r.tag != tag) {
            keep.push_back(r);
            continue;
        }
        float e = 0.f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&e, r.a, r.b) != cudaSuccess)
            rc = NVPT_ECUDA;
        t += e;
        ++n;
        by += r.bytes;
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    g_prof_rec.swap(keep);
    if (ms) *ms = t;
    if (launches) *launches = n;
    if (bytes) *bytes = by;
    return rc == NVPT_OK ? NVPT_OK : fail(ctx, rc, "profile_read: event query failed");
}

int nvpt_dgemm_split_d(nvpt_context *ctx, int64_t m, int64_t n, int64_t k, const double *A, const double *B,
                       double *C, void *stream) {
    if (!ctx || !A || !B || !C) return NVPT_EINVAL;
    if (m < 1 || n < 1 || n > 16 || k < 1 || k > 4096)
        return fail(ctx, NVPT_EINVAL, "dgemm_split: need m >= 1, 1 <= n <= 16, 1 <= k <= 4096");
    cudaStream_t st = pick(ctx, stream);
    oz::OzPlan pl(1, m, (int)k, (int)n);
    void *w = nullptr;
    NV_TRY(cuda_check(ctx, cudaMallocAsync(&w, pl.bytes(), st), "dgemm_split workspace"));
    const double *X[1] = {A}, *As[1] = {B};
    double *T[1] = {C};
    int rc = oz::oz_gemm_skinny(pl, X, As, T, (int)n, (int)n, w, st);
    int rc2 = rc ? 0 : oz::oz_check_error(w, st);
    cudaFreeAsync(w, st);
    if (rc) return fail(ctx, NVPT_ECUDA, "dgemm_split: launch failed");
    if (rc2 == 4) return fail(ctx, NVPT_ETIMEDOUT, "dgemm_split: the product timed out waiting on its pipeline");
    if (rc2) return fail(ctx, NVPT_ECUDA, "dgemm_split: error flag read-back failed");
    return after_launch(ctx, "dgemm_split");
}

int nvpt_dgemm_split_ex_d(nvpt_context *ctx, int transa, int transb, int64_t m, int64_t n, int64_t k, double alpha,
                          const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C,
                          int64_t ldc, void *stream) {
    if (!ctx || !A || !B || !C) return NVPT_EINVAL;
    int e2 = 0;
    if (m < 1 || n < 1 || k < 1 || k > oz::kWideMaxK || ldc < n || lda < (transa ? m : k) ||
        ldb < (transb ? k : n) || std::frexp(std::fabs(alpha), &e2) != 0.5)
        return fail(ctx, NVPT_EINVAL,
                    "dgemm_split_ex: need m, n >= 1, 1 <= k <= 2^19, lda/ldb/ldc >= the row lengths, alpha = +-2^e");
    cudaStream_t st = pick(ctx, stream);
    oz::WideGemm g;
    g.K = (int)k;
    g.alpha = alpha; g.beta = beta; g.C = C; g.ldc = ldc;
    if (m >= 64 || n < 128) {
        g.m = m; g.n = n;
        g.A = A; g.a_r = transa ? 1 : lda; g.a_k = transa ? lda : 1;
        g.B = B; g.b_c = transb ? ldb : 1; g.b_k = transb ? 1 : ldb;
    } else {  // few rows, many columns: C^T = op(B)^T op(A)^T fills the 128-row tiles
        g.m = n; g.n = m;
        g.A = B; g.a_r = transb ? ldb : 1; g.a_k = transb ? 1 : ldb;
        g.B = A; g.b_c = transa ? 1 : lda; g.b_k = transa ? lda : 1;
        g.c_trans = true;
    }
    const size_t bytes = oz::oz_wide_bytes(g.m, g.n, (int)k) + 256;
    void *w = nullptr;
    NV_TRY(cuda_check(ctx, cudaMallocAsync(&w, bytes, st), "dgemm_split_ex workspace"));
    int *err = (int *)((uint8_t *)w + bytes - 256);
    cudaMemsetAsync(err, 0, sizeof(int), st);
    int rc = oz::oz_gemm_wide(g, w, err, st);
    int rc2 = rc ? 0 : oz::oz_check_error(err, st);
    cudaFreeAsync(w, st);
    if (rc) return fail(ctx, NVPT_ECUDA, "dgemm_split_ex: launch failed");
    if (rc2 == 4) return fail(ctx, NVPT_ETIMEDOUT, "dgemm_split_ex: the product timed out waiting on its pipeline");
    if (rc2) return fail(ctx, NVPT_ECUDA, "dgemm_split_ex: error flag read-back failed");
    return after_launch(ctx, "dgemm_split_ex");
}

int nvpt_bbmat_d(nvpt_context *ctx, const double *atwo, double *bmat, double *btmat, const double *daaa,
                 const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
                 int64_t metat, void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    cudaStream_t st = pick(ctx, stream);
    Rdm r = make_rdm(nact, metat, dal, taa, daaa, nullptr);
    launch_build_f(f, aj, atwo, (int)nact, (int)ncore, 2, st);
    launch_bbmat(r, atwo, f, aj, (int)ncore, bmat, btmat, st);
    return after_launch(ctx, "bbmat");
}

int nvpt_bcmat_d(nvpt_context *ctx, const double *atwo, double *cmat, double *ctmat, const double *daaa,
                 const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
                 int64_t metat, void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    cudaStream_t st = pick(ctx, stream);
    Rdm r = make_rdm(nact, metat, dal, taa, daaa, nullptr);
    launch_build_f(f, aj, atwo, (int)nact, (int)ncore, 1, st);
    launch_bcmat(r, atwo, f, (int)ncore, cmat, ctmat, st);
    return after_launch(ctx, "bcmat");
}

int nvpt_bdmat_d(nvpt_context *ctx, const double *atwo, double *dmat, double *dtmat, const double *taa,
                 const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj, int64_t metat,
                 void *stream) {
    NV_TRY(check_nact(ctx, nact, metat));
    cudaStream_t st = pick(ctx, stream);
    Rdm r = make_rdm(nact, metat, dal, taa, nullptr, nullptr);
    launch_build_f(f, aj, atwo, (int)nact, (int)ncore, 2, st);
    launch_bdmat(r, atwo, f, aj, (int)ncore, dmat, dtmat, st);
    return after_launch(ctx, "bdmat");
}

// ----------------------------------------------------------- host entries
int nvpt_bro3(nvpt_context *ctx, const double *ro4, double *daaa, int64_t nact, int64_t nele, int64_t metat) {
    NV_TRY(check_nact(ctx, nact, metat));
    int64_t W = nvpt_nwords(nact), n4 = ipow(nact, 4), n6 = ipow(nact, 6);
    Stage S(ctx);
    const double *d_ro4 = S.up(ro4, W * n4 * metat);
    double *d_out = S.alloc(n6 * metat);
    if (S.status) return S.status;
    NV_TRY(nvpt_bro3_d(ctx, d_ro4, d_out, nact, nele, metat, nullptr));
    S.down(daaa, d_out, n6 * metat);
    return S.finish();
}

int nvpt_bro2(nvpt_context *ctx, const double *daaa, double *taa, int64_t nact, int64_t nele, int64_t metat) {
    NV_TRY(check_nact(ctx, nact, metat));
    int64_t n4 = ipow(nact, 4), n6 = ipow(nact, 6);
    Stage S(ctx);
    const double *d_in = S.up(daaa, n6 * metat);
    double *d_out = S.alloc(n4 * metat);
    if (S.status) return S.status;
    NV_TRY(nvpt_bro2_d(ctx, d_in, d_out, nact, nele, metat, nullptr));
    S.down(taa, d_out, n4 * metat);
    return S.finish();
}

int nvpt_bro1(nvpt_context *ctx, const double *taa, double *dal, int64_t nact, int64_t nele, int64_t metat) {
    NV_TRY(check_nact(ctx, nact, metat));
    int64_t n2 = ipow(nact, 2), n4 = ipow(nact, 4);
    Stage S(ctx);
    const double *d_in = S.up(taa, n4 * metat);
    double *d_out = S.alloc(n2 * metat);
    if (S.status) return S.status;
    NV_TRY(nvpt_bro1_d(ctx, d_in, d_out, nact, nele, metat, nullptr));
    S.down(dal, d_out, n2 * metat);
    return S.finish();
}

int nvpt_get_aj_atwo(nvpt_context *ctx, double *atwo, int64_t nact, int64_t ncore, int64_t norb, double *aj,
                     const double *oneint, const double *chol, int64_t nchovec) {
    NV_TRY(check_nact(ctx, nact, 1));
    if (ncore < 0 || norb < ncore + nact || nchovec < 1) return fail(ctx, NVPT_EINVAL, "get_aj_atwo: bad sizes");
    int64_t npair = norb * (norb + 1) / 2;
    Stage S(ctx);
    const double *d_one = S.up(oneint, npair);
    const double *d_L = S.up(chol, npair * nchovec);
    double *d_atwo = S.alloc(ipow(nact, 4));
    double *d_aj = S.alloc(npair);
    if (S.status) return S.status;
    NV_TRY(nvpt_get_aj_atwo_d(ctx, d_atwo, nact, ncore, norb, d_aj, d_one, d_L, nchovec, nullptr));
    S.down(atwo, d_atwo, ipow(nact, 4));
    S.down(aj, d_aj, npair);
    return S.finish();
}

int nvpt_koop_matrices_ctl(nvpt_context *ctx, int64_t metat, int64_t nact, int64_t ncore, const double *atwo,
                           const double *daaa, const double *taa, const double *dal, double *f, const double *aj,
                           double *ipko1, double *eako1, double *hrdm2, double *ipko2, double *eako2, double *gk0pa,
                           double *gk0pd, double *gk0pf) {
    NV_TRY(check_nact(ctx, nact, metat));
    int64_t M = metat, n2 = ipow(nact, 2), n4 = ipow(nact, 4), n6 = ipow(nact, 6), nf = f_len(nact, ncore);
    Stage S(ctx);
    const double *d_atwo = S.up(atwo, n4);
    const double *d3 = S.up(daaa, n6 * M), *d2 = S.up(taa, n4 * M), *d1 = S.up(dal, n2 * M);
    double *d_f = S.up(f, nf);
    const double *d_aj = S.up(aj, nf);
    double *o_ip1 = S.alloc(n2 * M), *o_ea1 = S.alloc(n2 * M), *o_h = S.alloc(n4 * M), *o_ip2 = S.alloc(n4 * M);
    double *o_ea2 = S.alloc(n4 * M), *o_a = S.alloc(n4 * M), *o_d = S.alloc(n4 * M), *o_f = S.alloc(n2 * M);
    if (S.status) return S.status;
    NV_TRY(nvpt_koop_matrices_ctl_d(ctx, metat, nact, ncore, d_atwo, d3, d2, d1, d_f, d_aj, o_ip1, o_ea1, o_h, o_ip2,
                                    o_ea2, o_a, o_d, o_f, nullptr));
    S.down(ipko1, o_ip1, n2 * M); S.down(eako1, o_ea1, n2 * M); S.down(hrdm2, o_h, n4 * M);
    S.down(ipko2, o_ip2, n4 * M); S.down(eako2, o_ea2, n4 * M); S.down(gk0pa, o_a, n4 * M);
    S.down(gk0pd, o_d, n4 * M); S.down(gk0pf, o_f, n2 * M); S.down(f, d_f, nf);
    return S.finish();
}

int nvpt_bamat(nvpt_context *ctx, double *amat, double *atmat, const double *atwo, const double *ro4,
               const double *daaa, const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f,
               const double *aj, int64_t norb, int64_t metat, int64_t nsym) {
    NV_TRY(check_nact(ctx, nact, metat));
    int64_t M = metat, n2 = ipow(nact, 2), n4 = ipow(nact, 4), n6 = ipow(nact, 6), nf = f_len(nact, ncore);
    int64_t W = nvpt_nwords(nact);
    Stage S(ctx);
    const double *d_atwo = S.up(atwo, n4);
    const double *d_ro4 = S.up(ro4, W * n4 * M);
    const double *d3 = S.up(daaa, n6 * M), *d2 = S.up(taa, n4 * M), *d1 = S.up(dal, n2 * M);
    double *d_f = S.up(f, nf);
    const double *d_aj = S.up(aj, nf);
    double *o_a = S.alloc(n6 * M), *o_at = S.alloc(n6 * M);
    if (S.status) return S.status;
    NV_TRY(nvpt_bamat_d(ctx, o_a, o_at, d_atwo, d_ro4, d3, d2, d1, nact, ncore, d_f, d_aj, norb, metat, nsym, nullptr));
    S.down(amat, o_a, n6 * M); S.down(atmat, o_at, n6 * M); S.down(f, d_f, nf);
    return S.finish();
}

static int unfold_host(nvpt_context *ctx, int which, double *dst, int64_t ld, int64_t nact, const int32_t *labels,
                       const double *values, int64_t nentries, int trans) {
    NV_TRY(check_nact(ctx, nact, 1));
    if (nentries < 0 || ld < 1) return fail(ctx, NVPT_EINVAL, "permute_rdm: bad arguments");
    const int64_t n = nact, W = nvpt_nwords(nact);
    const int64_t count = which == 4 ? W * ipow(n, 4) : ld * ipow(n, 6);
    Stage S(ctx);
    double *d = S.up(dst, count);
    const int32_t *l = nentries ? (const int32_t *)S.up_bytes(labels, sizeof(int32_t) * (which == 4 ? 8 : 6) * nentries)
                                : nullptr;
    const double *v = nentries ? S.up(values, nentries) : nullptr;
    if (S.status) return S.status;
    NV_TRY(unfold_d(ctx, which, d, ld, nact, l, v, nentries, trans, ctx->stream));
    S.down(dst, d, count);
    return S.finish();
}

int nvpt_permute_4rdm(nvpt_context *ctx, double *ro4, int64_t nact, const int32_t *labels, const double *values,
                      int64_t nentries) {
    return unfold_host(ctx, 4, ro4, 1, nact, labels, values, nentries, 0);
}

int nvpt_permute_3rdm(nvpt_context *ctx, double *rdm3, int64_t ld, int64_t nact, const int32_t *labels,
                      const double *values, int64_t nentries, int trans) {
    return unfold_host(ctx, 3, rdm3, ld, nact, labels, values, nentries, trans);
}

static int bcd_host(nvpt_context *ctx, int which, const double *atwo, double *x, double *xt, const double *daaa,
                    const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
                    int64_t metat) {
    NV_TRY(check_nact(ctx, nact, metat));
    int64_t M = metat, n2 = ipow(nact, 2), n4 = ipow(nact, 4), n6 = ipow(nact, 6), nf = f_len(nact, ncore);
    int64_t nout = (which == 3 ? n2 : n4) * M;
    Stage S(ctx);
    const double *d_atwo = S.up(atwo, n4);
    const double *d3 = which == 3 ? nullptr : S.up(daaa, n6 * M);
    const double *d2 = S.up(taa, n4 * M), *d1 = S.up(dal, n2 * M);
    double *d_f = S.up(f, nf);
    const double *d_aj = S.up(aj, nf);
    double *o = S.alloc(nout), *ot = S.alloc(nout);
    if (S.status) return S.status;
    int rc;
    if (which == 1) rc = nvpt_bbmat_d(ctx, d_atwo, o, ot, d3, d2, d1, nact, ncore, d_f, d_aj, metat, nullptr);
    else if (which == 2) rc = nvpt_bcmat_d(ctx, d_atwo, o, ot, d3, d2, d1, nact, ncore, d_f, d_aj, metat, nullptr);
    else rc = nvpt_bdmat_d(ctx, d_atwo, o, ot, d2, d1, nact, ncore, d_f, d_aj, metat, nullptr);
    if (rc != NVPT_OK) return rc;
    S.down(x, o, nout); S.down(xt, ot, nout); S.down(f, d_f, nf);
    return S.finish();
}

int nvpt_bbmat(nvpt_context *ctx, const double *atwo, double *bmat, double *btmat, const double *daaa,
               const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
               int64_t metat) {
    return bcd_host(ctx, 1, atwo, bmat, btmat, daaa, taa, dal, nact, ncore, f, aj, metat);
}
int nvpt_bcmat(nvpt_context *ctx, const double *atwo, double *cmat, double *ctmat, const double *daaa,
               const double *taa, const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj,
               int64_t metat) {
    return bcd_host(ctx, 2, atwo, cmat, ctmat, daaa, taa, dal, nact, ncore, f, aj, metat);
}
int nvpt_bdmat(nvpt_context *ctx, const double *atwo, double *dmat, double *dtmat, const double *taa,
               const double *dal, int64_t nact, int64_t ncore, double *f, const double *aj, int64_t metat) {
    return bcd_host(ctx, 3, atwo, dmat, dtmat, nullptr, taa, dal, nact, ncore, f, aj, metat);
}

}  // extern "C"
