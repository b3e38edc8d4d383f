// csim_host.cpp — host side of libcsimgpu.so: the C ABI of include/csim.h.
//
// Contexts, device buffers, argument checks, the estimator drivers
// (singleProjectorSample / sampledProjector / multiSampledProjector /
// exactProjector of libcirc/innerprod.c), decompose (libcirc/probability.c:
// 307-415) and the C library's rand() sequence.  All stabilizer algebra runs
// in the kernels of csim_kernels.cu; the host only prepares inputs, converts
// the kernels' exact Z[w] sums to doubles and does the per-query reductions.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/csim.h"
#include "csim_internal.h"

namespace {

// ---------------------------------------------------------------- libc rand()
// The C library's srand()/rand(): additive lagged-Fibonacci r_i = r_{i-3} +
// r_{i-31} (mod 2^32) seeded by the Park–Miller recurrence (Schrage's method),
// first 310 outputs discarded, outputs r_i >> 1 (P. Selinger, "The GLIBC
// pseudo-random number generator").
struct LibcRand {
    uint32_t ring[34];
    int idx;

    uint32_t step() {
        const uint32_t v = ring[(idx + 31) % 34] + ring[(idx + 3) % 34];
        ring[idx] = v;
        idx = (idx + 1) % 34;
        return v;
    }
    void seed(uint32_t s) {
        int32_t word = (int32_t)(s == 0 ? 1u : s);
        int32_t v[34];
        v[0] = word;
        for (int i = 1; i < 31; i++) {
            const int64_t hi = word / 127773, lo = word % 127773;
            word = (int32_t)(16807 * lo - 2836 * hi);
            if (word < 0) word += 2147483647;
            v[i] = word;
        }
        for (int i = 31; i < 34; i++) v[i] = v[i - 31];
        for (int i = 0; i < 34; i++) ring[i] = (uint32_t)v[i];
        idx = 0;
        for (int i = 34; i < 344; i++) step();
    }
    int32_t next() { return (int32_t)(step() >> 1); }
};

// ---------------------------------------------------------------- helpers
inline int popc(uint64_t x) { return __builtin_popcountll(x); }
inline int par(uint64_t x) { return __builtin_popcountll(x) & 1; }
inline int phase_m(int v) { return 2 * (((v / 2) % 2) & 1) + ((v % 2) & 1); }  // comms.c:23-25, innerprod.c:101-102

// logeta (stabilizer.c:677-687) and the normalized cumulative table of
// randomStabilizerState (stabilizer.c:694-716), same expressions, same libm
double logeta(int d, int n) {
    if (d == 0) return 0.;
    double product = 0;
    for (int a = 1; a <= d; a++) {
        product += log2(1 - pow(2, d - n - a));
        product -= log2(1 - pow(2, -a));
    }
    return (-d * (d + 1) / 2) + product;
}

void cum_table(int n, double* cum) {
    double dist[CSIM_MAX_QUBITS + 1];
    double sum = 0;
    for (int d = 0; d <= n; d++) {
        dist[d] = pow(2, logeta(d, n));
        sum += dist[d];
    }
    for (int d = 0; d <= n; d++) dist[d] /= sum;
    for (int i = 0; i <= n; i++) {
        cum[i] = 0;
        for (int d = 0; d <= i; d++) cum[i] += dist[d];
    }
    for (int i = 0; i <= n; i++) cum[i] /= cum[n];
}

uint64_t codeword(int64_t j, const uint64_t* L, int k) {
    uint64_t x = 0;
    for (int r = 0; r < k; r++)
        if ((j >> (k - 1 - r)) & 1) x ^= L[r];
    return x;
}

// The rand() words randomStabilizerState consumes for one n-qubit state, drawn
// from `lr` in the reference's order.  The lazy shrink loop is simulated on G
// alone to know how many random vectors are drawn (stabilizer.c:736-740).
void draw_state_words(LibcRand& lr, int n, const double* cum, std::vector<uint32_t>& words) {
    double sample;
    do {
        const int32_t w = lr.next();
        words.push_back((uint32_t)w);
        sample = 0. + (w / (2147483647 / 1.0));
    } while (sample == 0.);
    int d = 0;
    for (; d <= n; d++)
        if (sample <= cum[d]) break;
    const int kt = n - d;
    uint64_t G[CSIM_MAX_QUBITS];
    for (int i = 0; i < n; i++) G[i] = 1ull << i;
    int k = n;
    const int bytes = (n + 7) / 8;
    while (k > kt) {
        uint64_t xi = 0;
        for (int b = 0; b < bytes; b++) {
            const int32_t w = lr.next();
            words.push_back((uint32_t)w);
            const int byte = w % 256;
            for (int j = 0; j < 8; j++) {
                const int loc = 8 * b + j;
                if (loc < n && (byte & (0x80 >> j))) xi |= 1ull << loc;
            }
        }
        int last = -1;
        uint64_t S = 0;
        for (int a = 0; a < k; a++)
            if (par(G[a] & xi)) {
                S |= 1ull << a;
                last = a;
            }
        if (last < 0) continue;
        for (int a = 0; a < k; a++)
            if (a != last && ((S >> a) & 1)) G[a] ^= G[last];
        std::swap(G[last], G[k - 1]);
        k--;
    }
    const int64_t rest = 3 * bytes + (int64_t)k * (k - 1) / 2;
    for (int64_t i = 0; i < rest; i++) words.push_back((uint32_t)lr.next());
}

// z0 + z1 w + z2 w^2 + z3 w^3 (w = e^{i pi/4}) times 2^{-P/2}, P even
void zomega_to_complex(const __int128* z, int P, double* re, double* im) {
    const double s = 0.70710678118654752440;
    const double r = (double)z[0] + (double)(z[1] - z[3]) * s;
    const double i = (double)z[2] + (double)(z[1] + z[3]) * s;
    *re = std::ldexp(r, -P / 2);
    *im = std::ldexp(i, -P / 2);
}

// terms per work item of the pair kernel: at most 64 items per theta
int64_t chunk_for(int64_t chi) { return std::max<int64_t>(256, (chi + 63) / 64); }

double sqrt_half_power(int c) {  // projfactor of innerprod.c:104-111: c successive *= 2^{-1/2}
    double pf = 1;
    const double r = pow(2, -0.5);
    for (int i = 0; i < c; i++) pf *= r;
    return pf;
}

}  // namespace

// ---------------------------------------------------------------- context
enum BufId {
    kBufA, kBufB, kBufEps, kBufP, kBufM, kBufXi, kBufZeta, kBufAlpha, kBufCode, kBufWords, kBufOffsets,
    kBufCum, kBufCodewords, kBufAcc, kBufAccDiag, kBufPhis, kBufIdx, kBufConsumed, kBufPm, kBufPz, kBufPx,
    kBufL, kBufParts, kBufPartsDiag, kNumBufs
};

struct csim_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    int* d_err = nullptr;
    int64_t launches = 0;
    std::string last_error;
    void* buf[kNumBufs + 32] = {};
    size_t cap[kNumBufs + 32] = {};
    LibcRand lr;
    uint64_t philox_seed = 0;
    uint64_t philox_next = 0;
    csim_stats stats = {};
    int64_t stats_launch0 = 0;
    int pair_kernel = 0;  // CSIM_OPT_PAIR_KERNEL
    int per_thread = 16;  // CSIM_OPT_PER_THREAD
    cudaEvent_t ev[4] = {};
};

namespace {

int fail(csim_ctx* ctx, int code, const char* fmt, ...) {
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof(msg), fmt, ap);
    va_end(ap);
    if (ctx) ctx->last_error = msg;
    return code;
}

#define CK(call)                                                                                              \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess) return fail(ctx, CSIM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));      \
    } while (0)

#define CKR(expr)            \
    do {                     \
        int r_ = (expr);     \
        if (r_ != 0) return r_; \
    } while (0)

int dbuf(csim_ctx* ctx, int id, size_t bytes, void** out) {
    if (bytes == 0) bytes = 16;
    if (ctx->cap[id] < bytes) {
        if (ctx->buf[id]) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->buf[id]);
            ctx->buf[id] = nullptr;
            ctx->cap[id] = 0;
        }
        size_t c = bytes + bytes / 4;
        if (cudaMalloc(&ctx->buf[id], c) != cudaSuccess) {
            ctx->buf[id] = nullptr;
            return fail(ctx, CSIM_ERR_NOMEM, "cudaMalloc of %zu bytes failed", c);
        }
        ctx->cap[id] = c;
    }
    *out = ctx->buf[id];
    return 0;
}

template <class T>
int dput(csim_ctx* ctx, int id, const T* src, size_t count, T** out) {
    void* p;
    CKR(dbuf(ctx, id, count * sizeof(T), &p));
    if (count) CK(cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    ctx->stats.h2d_bytes += (int64_t)(count * sizeof(T));
    *out = (T*)p;
    return 0;
}

template <class T>
int dget(csim_ctx* ctx, T* dst, const T* src, size_t count) {
    if (count) CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->stats.d2h_bytes += (int64_t)(count * sizeof(T));
    return 0;
}

void stats_begin(csim_ctx* ctx) {
    ctx->stats = csim_stats{};
    ctx->stats_launch0 = ctx->launches;
}

// adds the event-timed spans of one batch: ev0..ev3 = start, pair kernel start, pair kernel end, end
int stats_batch(csim_ctx* ctx) {
    float a = 0, b = 0;
    CK(cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[3]));
    CK(cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]));
    ctx->stats.device_ms += a;
    ctx->stats.pair_kernel_ms += b;
    return 0;
}

void stats_end(csim_ctx* ctx) { ctx->stats.kernels = ctx->launches - ctx->stats_launch0; }

csim::Launch launch_of(csim_ctx* ctx) { return csim::Launch{ctx->stream, ctx->d_err, &ctx->launches, ctx->num_sms}; }

// waits for the stream, then turns device error flags into a status
int finish(csim_ctx* ctx) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaGetLastError());
    if (h) {
        CK(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        return fail(ctx, CSIM_ERR_DEVICE, "kernel flagged error bits 0x%x (1 range, 2 replay, 4 expsum, 8 gamma, 16 arg)",
                    h);
    }
    return 0;
}

int check_states(csim_ctx* ctx, const csim_state* s, int64_t count, int* nr_out, int n_expect = -1) {
    int nmax = 0;
    for (int64_t i = 0; i < count; i++) {
        const int n = s[i].n, k = s[i].k;
        if (n < 1 || n > CSIM_MAX_QUBITS || k < 0 || k > n)
            return fail(ctx, CSIM_ERR_ARG, "state %lld: n=%d k=%d out of range", (long long)i, n, k);
        if (n_expect > 0 && n != n_expect)
            return fail(ctx, CSIM_ERR_ARG, "state %lld: n=%d, expected %d", (long long)i, n, n_expect);
        nmax = std::max(nmax, n);
    }
    *nr_out = nmax > 32 ? 2 : 1;
    return 0;
}

constexpr int64_t kBatch = 1 << 18;  // states per device round trip in the batched primitives

}  // namespace

// ---------------------------------------------------------------- context API
extern "C" void csim_ctx_destroy(csim_ctx* ctx);

extern "C" int csim_ctx_create(int device, csim_ctx** out) {
    if (!out) return CSIM_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return CSIM_ERR_NODEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return CSIM_ERR_NODEVICE;
    if (!(prop.major == 10 && prop.minor == 3)) {
        fprintf(stderr, "csim: device %d is sm_%d%d; libcsimgpu is built for sm_103a only\n", device, prop.major,
                prop.minor);
        return CSIM_ERR_NODEVICE;
    }
    csim_ctx* ctx = new csim_ctx();
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) !=
                                                    cudaSuccess ||
        cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess || cudaMemset(ctx->d_err, 0, sizeof(int)) != cudaSuccess) {
        delete ctx;
        return CSIM_ERR_CUDA;
    }
    for (int i = 0; i < 4; i++)
        if (cudaEventCreate(&ctx->ev[i]) != cudaSuccess) {
            csim_ctx_destroy(ctx);
            return CSIM_ERR_CUDA;
        }
    ctx->lr.seed(1);  // an unseeded rand() behaves as srand(1)
    *out = ctx;
    return CSIM_OK;
}

extern "C" void csim_ctx_destroy(csim_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int i = 0; i < kNumBufs + 32; i++)
        if (ctx->buf[i]) cudaFree(ctx->buf[i]);
    if (ctx->d_err) cudaFree(ctx->d_err);
    for (int i = 0; i < 4; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" int csim_set_option(csim_ctx* ctx, int32_t option, int64_t value) {
    if (!ctx) return CSIM_ERR_ARG;
    switch (option) {
    case CSIM_OPT_PAIR_KERNEL:
        if (value != 0 && value != 1) return fail(ctx, CSIM_ERR_ARG, "pair kernel must be 0 or 1");
        ctx->pair_kernel = (int)value;
        return CSIM_OK;
    case CSIM_OPT_PER_THREAD:
        if (value < 1 || value > 64) return fail(ctx, CSIM_ERR_ARG, "per-thread pairs must be 1..64");
        ctx->per_thread = (int)value;
        return CSIM_OK;
    default:
        return fail(ctx, CSIM_ERR_ARG, "unknown option %d", option);
    }
}

extern "C" int csim_rng_position(csim_ctx* ctx, uint64_t seed, uint64_t first) {
    if (!ctx) return CSIM_ERR_ARG;
    ctx->philox_seed = seed;
    ctx->philox_next = first;
    return CSIM_OK;
}

extern "C" int csim_last_stats(const csim_ctx* ctx, csim_stats* out) {
    if (!ctx || !out) return CSIM_ERR_ARG;
    *out = ctx->stats;
    return CSIM_OK;
}

extern "C" const char* csim_last_error(const csim_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }
extern "C" int64_t csim_launch_count(const csim_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" int64_t csim_libc_rand_size(void) { return (int64_t)sizeof(LibcRand); }
extern "C" void csim_libc_rand_seed(void* state, uint32_t seed) { ((LibcRand*)state)->seed(seed); }
extern "C" int32_t csim_libc_rand_next(void* state) { return ((LibcRand*)state)->next(); }

// ---------------------------------------------------------------- primitives
extern "C" int csim_inner_product_exact(csim_ctx* ctx, int64_t count, const csim_state* a, const csim_state* b,
                                        int32_t* eps, int32_t* p, int32_t* m) {
    if (!ctx || count < 0 || (count && (!a || !b || !eps || !p || !m))) return fail(ctx, CSIM_ERR_ARG, "null argument");
    cudaSetDevice(ctx->device);
    int nra, nrb;
    CKR(check_states(ctx, a, count, &nra));
    CKR(check_states(ctx, b, count, &nrb));
    for (int64_t i = 0; i < count; i++)
        if (a[i].n != b[i].n) return fail(ctx, CSIM_ERR_ARG, "pair %lld: n differs", (long long)i);
    const int nr = std::max(nra, nrb);
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        csim_state *da, *db;
        int *de, *dp, *dm;
        void* v;
        CKR(dput(ctx, kBufA, a + o, c, &da));
        CKR(dput(ctx, kBufB, b + o, c, &db));
        CKR(dbuf(ctx, kBufEps, c * 4, &v)); de = (int*)v;
        CKR(dbuf(ctx, kBufP, c * 4, &v)); dp = (int*)v;
        CKR(dbuf(ctx, kBufM, c * 4, &v)); dm = (int*)v;
        if (csim::launch_inner_product(launch_of(ctx), nr, (const csim::GState*)da, (const csim::GState*)db, c, de, dp,
                                       dm))
            return fail(ctx, CSIM_ERR_CUDA, "inner product launch failed");
        CKR(dget(ctx, eps + o, de, c));
        CKR(dget(ctx, p + o, dp, c));
        CKR(dget(ctx, m + o, dm, c));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

extern "C" int csim_exponential_sum_exact(csim_ctx* ctx, int64_t count, csim_state* s, int32_t* eps, int32_t* p,
                                          int32_t* m) {
    if (!ctx || count < 0 || (count && (!s || !eps || !p || !m))) return fail(ctx, CSIM_ERR_ARG, "null argument");
    cudaSetDevice(ctx->device);
    int nr;
    CKR(check_states(ctx, s, count, &nr));
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        csim_state* ds;
        int *de, *dp, *dm;
        void* v;
        CKR(dput(ctx, kBufA, s + o, c, &ds));
        CKR(dbuf(ctx, kBufEps, c * 4, &v)); de = (int*)v;
        CKR(dbuf(ctx, kBufP, c * 4, &v)); dp = (int*)v;
        CKR(dbuf(ctx, kBufM, c * 4, &v)); dm = (int*)v;
        if (csim::launch_exp_sum(launch_of(ctx), nr, (csim::GState*)ds, c, de, dp, dm))
            return fail(ctx, CSIM_ERR_CUDA, "exponential sum launch failed");
        CKR(dget(ctx, s + o, ds, c));
        CKR(dget(ctx, eps + o, de, c));
        CKR(dget(ctx, p + o, dp, c));
        CKR(dget(ctx, m + o, dm, c));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

extern "C" int csim_shrink(csim_ctx* ctx, int64_t count, csim_state* s, const uint64_t* xi, const int32_t* alpha,
                           int32_t lazy, int32_t* status) {
    if (!ctx || count < 0 || (count && (!s || !xi || !alpha || !status))) return fail(ctx, CSIM_ERR_ARG, "null argument");
    cudaSetDevice(ctx->device);
    int nr;
    CKR(check_states(ctx, s, count, &nr));
    for (int64_t i = 0; i < count; i++)
        if (alpha[i] < 0) return fail(ctx, CSIM_ERR_ARG, "alpha must be >= 0");
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        csim_state* ds;
        uint64_t* dx;
        int32_t* dal;
        int* dst;
        void* v;
        CKR(dput(ctx, kBufA, s + o, c, &ds));
        CKR(dput(ctx, kBufXi, xi + o, c, &dx));
        CKR(dput(ctx, kBufAlpha, alpha + o, c, &dal));
        CKR(dbuf(ctx, kBufCode, c * 4, &v)); dst = (int*)v;
        if (csim::launch_shrink(launch_of(ctx), nr, (csim::GState*)ds, dx, dal, lazy, c, dst))
            return fail(ctx, CSIM_ERR_CUDA, "shrink launch failed");
        CKR(dget(ctx, s + o, ds, c));
        CKR(dget(ctx, status + o, dst, c));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

extern "C" int csim_measure_pauli(csim_ctx* ctx, int64_t count, csim_state* s, const int32_t* m, const uint64_t* zeta,
                                  const uint64_t* xi, double* norm) {
    if (!ctx || count < 0 || (count && (!s || !m || !zeta || !xi || !norm)))
        return fail(ctx, CSIM_ERR_ARG, "null argument");
    cudaSetDevice(ctx->device);
    int nr;
    CKR(check_states(ctx, s, count, &nr));
    std::vector<int> code((size_t)std::min(count, kBatch));
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        csim_state* ds;
        uint64_t *dx, *dz;
        int32_t* dm;
        int* dc;
        void* v;
        CKR(dput(ctx, kBufA, s + o, c, &ds));
        CKR(dput(ctx, kBufXi, xi + o, c, &dx));
        CKR(dput(ctx, kBufZeta, zeta + o, c, &dz));
        CKR(dput(ctx, kBufAlpha, m + o, c, &dm));
        CKR(dbuf(ctx, kBufCode, c * 4, &v)); dc = (int*)v;
        if (csim::launch_measure(launch_of(ctx), nr, (csim::GState*)ds, dm, dz, dx, c, dc))
            return fail(ctx, CSIM_ERR_CUDA, "measurePauli launch failed");
        CKR(dget(ctx, s + o, ds, c));
        CKR(dget(ctx, code.data(), dc, c));
        CKR(finish(ctx));
        for (int64_t i = 0; i < c; i++) norm[o + i] = code[i] == 0 ? 0.0 : (code[i] == 1 ? 1.0 : pow(2, -0.5));
    }
    return CSIM_OK;
}

extern "C" int csim_extend(csim_ctx* ctx, int64_t count, csim_state* s, const uint64_t* xi) {
    if (!ctx || count < 0 || (count && (!s || !xi))) return fail(ctx, CSIM_ERR_ARG, "null argument");
    cudaSetDevice(ctx->device);
    int nr;
    CKR(check_states(ctx, s, count, &nr));
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        csim_state* ds;
        uint64_t* dx;
        CKR(dput(ctx, kBufA, s + o, c, &ds));
        CKR(dput(ctx, kBufXi, xi + o, c, &dx));
        if (csim::launch_extend(launch_of(ctx), nr, (csim::GState*)ds, dx, c))
            return fail(ctx, CSIM_ERR_CUDA, "extend launch failed");
        CKR(dget(ctx, s + o, ds, c));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

namespace {

int upload_cum(csim_ctx* ctx, int n, double** dcum) {
    double cum[CSIM_MAX_QUBITS + 1];
    cum_table(n, cum);
    return dput(ctx, kBufCum, cum, (size_t)n + 1, dcum);
}

}  // namespace

extern "C" int csim_random_states(csim_ctx* ctx, int32_t n, int64_t count, uint64_t seed, uint64_t first,
                                  csim_state* out) {
    if (!ctx || count < 0 || (count && !out) || n < 1 || n > CSIM_MAX_QUBITS)
        return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        double* dcum;
        void* v;
        CKR(upload_cum(ctx, n, &dcum));
        CKR(dbuf(ctx, kBufA, c * sizeof(csim_state), &v));
        if (csim::launch_random_states(launch_of(ctx), n, c, 0, seed, first + o, nullptr, nullptr, dcum,
                                       (csim::GState*)v, nullptr))
            return fail(ctx, CSIM_ERR_CUDA, "random state launch failed");
        CKR(dget(ctx, out + o, (const csim_state*)v, c));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

extern "C" int csim_random_states_replay(csim_ctx* ctx, int32_t n, int64_t count, const uint32_t* words,
                                         const int64_t* offsets, csim_state* out) {
    if (!ctx || count < 0 || (count && (!out || !words || !offsets)) || n < 1 || n > CSIM_MAX_QUBITS)
        return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    if (count == 0) return CSIM_OK;
    for (int64_t i = 0; i < count; i++)
        if (offsets[i + 1] < offsets[i] || offsets[i] < 0) return fail(ctx, CSIM_ERR_ARG, "offsets not increasing");
    const int64_t nw = offsets[count];
    std::vector<int64_t> rel(count + 1), consumed(count);
    for (int64_t i = 0; i <= count; i++) rel[i] = offsets[i] - offsets[0];
    double* dcum;
    uint32_t* dw;
    int64_t *doff, *dcon;
    void* v;
    CKR(upload_cum(ctx, n, &dcum));
    CKR(dput(ctx, kBufWords, words + offsets[0], (size_t)(nw - offsets[0]), &dw));
    CKR(dput(ctx, kBufOffsets, rel.data(), rel.size(), &doff));
    CKR(dbuf(ctx, kBufConsumed, count * 8, &v)); dcon = (int64_t*)v;
    CKR(dbuf(ctx, kBufA, count * sizeof(csim_state), &v));
    if (csim::launch_random_states(launch_of(ctx), n, count, 1, 0, 0, dw, doff, dcum, (csim::GState*)v, dcon))
        return fail(ctx, CSIM_ERR_CUDA, "random state launch failed");
    CKR(dget(ctx, out, (const csim_state*)v, count));
    CKR(dget(ctx, consumed.data(), dcon, count));
    CKR(finish(ctx));
    for (int64_t i = 0; i < count; i++)
        if (consumed[i] != rel[i + 1] - rel[i])
            return fail(ctx, CSIM_ERR_ARG, "state %lld consumed %lld words, segment holds %lld", (long long)i,
                        (long long)consumed[i], (long long)(rel[i + 1] - rel[i]));
    return CSIM_OK;
}

extern "C" int csim_prep_h(csim_ctx* ctx, int32_t t, int64_t count, const int64_t* idx, csim_state* out) {
    if (!ctx || count < 0 || (count && (!idx || !out)) || t < 1 || t > CSIM_MAX_QUBITS)
        return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    const int64_t lim = (int64_t)1 << ((t + 1) / 2);
    for (int64_t i = 0; i < count; i++)
        if (idx[i] < 0 || idx[i] >= lim) return fail(ctx, CSIM_ERR_ARG, "term index out of range");
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        int64_t* di;
        void* v;
        CKR(dput(ctx, kBufIdx, idx + o, c, &di));
        CKR(dbuf(ctx, kBufA, c * sizeof(csim_state), &v));
        if (csim::launch_prep(launch_of(ctx), t, 1, nullptr, di, c, (csim::GState*)v))
            return fail(ctx, CSIM_ERR_CUDA, "prepH launch failed");
        CKR(dget(ctx, out + o, (const csim_state*)v, c));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

extern "C" int csim_prep_l(csim_ctx* ctx, int32_t t, const uint64_t* L, int32_t k, int64_t count, const int64_t* idx,
                           csim_state* out) {
    if (!ctx || count < 0 || (count && (!idx || !out || !L)) || t < 1 || t > CSIM_MAX_QUBITS || k < 0 || k > 62)
        return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    for (int64_t o = 0; o < count; o += kBatch) {
        const int64_t c = std::min(kBatch, count - o);
        std::vector<uint64_t> cw(c);
        for (int64_t i = 0; i < c; i++) {
            if (idx[o + i] < 0 || idx[o + i] >= ((int64_t)1 << k)) return fail(ctx, CSIM_ERR_ARG, "term index out of range");
            cw[i] = codeword(idx[o + i], L, k) & (t >= 64 ? ~0ull : ((1ull << t) - 1));
        }
        uint64_t* dcw;
        void* v;
        CKR(dput(ctx, kBufCodewords, cw.data(), cw.size(), &dcw));
        CKR(dbuf(ctx, kBufA, c * sizeof(csim_state), &v));
        if (csim::launch_prep(launch_of(ctx), t, 0, dcw, nullptr, c, (csim::GState*)v))
            return fail(ctx, CSIM_ERR_CUDA, "prepL launch failed");
        CKR(dget(ctx, out + o, (const csim_state*)v, c));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

// ---------------------------------------------------------------- hot path
namespace {

// the terms |phi_j>, j in [j0, j0+nj): codewords (|L>) or prepared states (|H^t>)
int stage_terms(csim_ctx* ctx, int t, int exact, const uint64_t* L, int k, int64_t j0, int64_t nj,
                uint64_t** dcw, csim_state** dphis) {
    *dcw = nullptr;
    *dphis = nullptr;
    void* v;
    if (!exact) {
        uint64_t* dL;
        CKR(dput(ctx, kBufL, L, (size_t)k, &dL));
        CKR(dbuf(ctx, kBufCodewords, nj * 8, &v));
        if (csim::launch_codewords(launch_of(ctx), dL, k, j0, nj, (uint64_t*)v))
            return fail(ctx, CSIM_ERR_CUDA, "codeword launch failed");
        *dcw = (uint64_t*)v;
        return 0;
    }
    std::vector<int64_t> idx(nj);
    for (int64_t i = 0; i < nj; i++) idx[i] = j0 + i;
    int64_t* di;
    CKR(dput(ctx, kBufIdx, idx.data(), idx.size(), &di));
    CKR(dbuf(ctx, kBufPhis, nj * sizeof(csim_state), &v));
    if (csim::launch_prep(launch_of(ctx), t, 1, nullptr, di, nj, (csim::GState*)v))
        return fail(ctx, CSIM_ERR_CUDA, "prepH launch failed");
    *dphis = (csim_state*)v;
    return 0;
}

int check_code(csim_ctx* ctx, int t, int exact, const uint64_t* L, int k) {
    if (t < 1 || t > CSIM_MAX_QUBITS) return fail(ctx, CSIM_ERR_ARG, "t=%d out of range 1..64", t);
    if (!exact) {
        if (!L || k < 0 || k > 40) return fail(ctx, CSIM_ERR_ARG, "k=%d out of range 0..40", k);
        const uint64_t tm = t >= 64 ? ~0ull : ((1ull << t) - 1);
        for (int r = 0; r < k; r++)
            if (L[r] & ~tm) return fail(ctx, CSIM_ERR_ARG, "row %d of L has bits beyond t", r);
    } else if ((t + 1) / 2 > 40) {
        return fail(ctx, CSIM_ERR_ARG, "exact decomposition of t=%d is too large", t);
    }
    return 0;
}

}  // namespace

extern "C" int csim_term_products(csim_ctx* ctx, int32_t t, int32_t exact, const uint64_t* L, int32_t k,
                                  int64_t ntheta, const csim_state* theta, int64_t j0, int64_t nj, int32_t* eps,
                                  int32_t* p, int32_t* m) {
    if (!ctx || ntheta < 0 || nj < 0 || j0 < 0 || (ntheta && nj && (!theta || !eps || !p || !m)))
        return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    CKR(check_code(ctx, t, exact, L, k));
    const int64_t chi = exact ? ((int64_t)1 << ((t + 1) / 2)) : ((int64_t)1 << k);
    if (j0 + nj > chi) return fail(ctx, CSIM_ERR_ARG, "term range beyond chi");
    if (ntheta == 0 || nj == 0) return CSIM_OK;
    int nr;
    CKR(check_states(ctx, theta, ntheta, &nr, t));
    // the thread-per-pair kernel needs a symmetric J block (always true of drawn states)
    bool sym = true;
    for (int64_t a = 0; a < ntheta && sym; a++)
        for (int x = 0; x < theta[a].k && sym; x++)
            for (int y = 0; y < theta[a].k; y++)
                if (((theta[a].J[x] >> y) & 1) != ((theta[a].J[y] >> x) & 1)) {
                    sym = false;
                    break;
                }
    uint64_t* dcw;
    csim_state* dphis;
    CKR(stage_terms(ctx, t, exact, L, k, j0, nj, &dcw, &dphis));
    const int64_t rows = std::max<int64_t>(1, std::min<int64_t>(ntheta, (1 << 22) / nj + 1));
    for (int64_t o = 0; o < ntheta; o += rows) {
        const int64_t c = std::min(rows, ntheta - o);
        csim_state* dth;
        void* v;
        CKR(dput(ctx, kBufA, theta + o, c, &dth));
        CKR(dbuf(ctx, kBufEps, c * nj * 4, &v));
        int* de = (int*)v;
        CKR(dbuf(ctx, kBufP, c * nj * 4, &v));
        int* dp = (int*)v;
        CKR(dbuf(ctx, kBufM, c * nj * 4, &v));
        int* dm = (int*)v;
        const int rc = (!exact && ctx->pair_kernel == 0 && sym)
                           ? csim::launch_terms_tp(launch_of(ctx), t, dcw, (const csim::GState*)dth, nullptr, c, j0, nj,
                                                   ctx->per_thread, 2 * t, nullptr, de, dp, dm)
                           : csim::launch_terms(launch_of(ctx), nr, exact ? 1 : 0, dcw, (const csim::GState*)dphis,
                                                (const csim::GState*)dth, nullptr, c, j0, nj, 64, 2 * t, nullptr,
                                                nullptr, de, dp, dm);
        if (rc) return fail(ctx, CSIM_ERR_CUDA, "term launch failed");
        CKR(dget(ctx, eps + o * nj, de, c * nj));
        CKR(dget(ctx, p + o * nj, dp, c * nj));
        CKR(dget(ctx, m + o * nj, dm, c * nj));
        CKR(finish(ctx));
    }
    return CSIM_OK;
}

namespace {

int check_projector(csim_ctx* ctx, const csim_projector* P) {
    if (!P || P->nstabs < 0 || P->nqubits < 0 || P->nqubits > CSIM_MAX_QUBITS)
        return fail(ctx, CSIM_ERR_ARG, "bad projector");
    if (P->nstabs > 0 && (!P->phase || !P->xs || !P->zs)) return fail(ctx, CSIM_ERR_ARG, "bad projector arrays");
    return 0;
}

// Draws `count` states, projects them onto P, sums their terms on the GPU, and
// returns singleProjectorSample's value for each (innerprod.c:88-144).
int sample_values(csim_ctx* ctx, const csim_projector* P, const uint64_t* L, int k, int exact, int64_t count,
                  int rng, uint64_t seed, double* values) {
    const int t = P->nqubits;
    CKR(check_code(ctx, t, exact, L, k));
    if (rng != CSIM_RNG_LIBC && rng != CSIM_RNG_PHILOX) return fail(ctx, CSIM_ERR_ARG, "unknown rng %d", rng);
    if (rng == CSIM_RNG_LIBC && seed != CSIM_SEED_CONTINUE) ctx->lr.seed((uint32_t)seed);
    if (rng == CSIM_RNG_PHILOX && seed != CSIM_SEED_CONTINUE) {
        ctx->philox_seed = seed;
        ctx->philox_next = 0;
    }
    if (count <= 0) return 0;
    const int nr = t > 32 ? 2 : 1;
    const int64_t chi = exact ? ((int64_t)1 << ((t + 1) / 2)) : ((int64_t)1 << k);
    const int P2 = 2 * t;
    const bool tp = !exact && ctx->pair_kernel == 0;
    const int64_t chunk = chunk_for(chi);
    const int64_t nchunks = tp ? csim::terms_tp_blocks(chi, ctx->per_thread) : (chi + chunk - 1) / chunk;

    std::vector<int> hm(P->nstabs);
    for (int r = 0; r < P->nstabs; r++) hm[r] = phase_m(P->phase[r]);
    int* dpm;
    uint64_t *dpz, *dpx;
    CKR(dput(ctx, kBufPm, hm.data(), hm.size(), &dpm));
    CKR(dput(ctx, kBufPz, P->zs, (size_t)P->nstabs, &dpz));
    CKR(dput(ctx, kBufPx, P->xs, (size_t)P->nstabs, &dpx));
    double* dcum;
    CKR(upload_cum(ctx, t, &dcum));
    double hcum[CSIM_MAX_QUBITS + 1];
    cum_table(t, hcum);
    uint64_t* dcw;
    csim_state* dphis;
    CKR(stage_terms(ctx, t, exact, L, k, 0, chi, &dcw, &dphis));

    const int64_t batch = 1 << 14;
    std::vector<uint32_t> words;
    std::vector<int64_t> offs;
    std::vector<int> code;
    std::vector<__int128> acc;
    for (int64_t o = 0; o < count; o += batch) {
        const int64_t c = std::min(batch, count - o);
        void* v;
        CKR(dbuf(ctx, kBufA, c * sizeof(csim_state), &v));
        csim::GState* dth = (csim::GState*)v;
        if (rng == CSIM_RNG_LIBC) {
            words.clear();
            offs.assign(1, 0);
            for (int64_t i = 0; i < c; i++) {
                draw_state_words(ctx->lr, t, hcum, words);
                offs.push_back((int64_t)words.size());
            }
            uint32_t* dw;
            int64_t* doff;
            CKR(dput(ctx, kBufWords, words.data(), words.size(), &dw));
            CKR(dput(ctx, kBufOffsets, offs.data(), offs.size(), &doff));
            CK(cudaEventRecord(ctx->ev[0], ctx->stream));
            if (csim::launch_random_states(launch_of(ctx), t, c, 1, 0, 0, dw, doff, dcum, dth, nullptr))
                return fail(ctx, CSIM_ERR_CUDA, "random state launch failed");
        } else {
            CK(cudaEventRecord(ctx->ev[0], ctx->stream));
            if (csim::launch_random_states(launch_of(ctx), t, c, 0, ctx->philox_seed, ctx->philox_next, nullptr,
                                           nullptr, dcum, dth, nullptr))
                return fail(ctx, CSIM_ERR_CUDA, "random state launch failed");
            ctx->philox_next += c;
        }
        CKR(dbuf(ctx, kBufCode, c * 4, &v));
        int* dcode = (int*)v;
        if (csim::launch_project(launch_of(ctx), nr, dth, c, P->nstabs, dpm, dpz, dpx, dcode))
            return fail(ctx, CSIM_ERR_CUDA, "projection launch failed");
        const size_t nparts = (size_t)c * nchunks * 4;
        CKR(dbuf(ctx, kBufParts, nparts * sizeof(__int128), &v));
        __int128* dpart = (__int128*)v;
        CK(cudaMemsetAsync(dpart, 0, nparts * sizeof(__int128), ctx->stream));
        CK(cudaEventRecord(ctx->ev[1], ctx->stream));
        const int rc = tp ? csim::launch_terms_tp(launch_of(ctx), t, dcw, dth, dcode, c, 0, chi, ctx->per_thread, P2,
                                                  dpart, nullptr, nullptr, nullptr)
                          : csim::launch_terms(launch_of(ctx), nr, exact ? 1 : 0, dcw, (const csim::GState*)dphis, dth,
                                               dcode, c, 0, chi, (int)chunk, P2, dpart, nullptr, nullptr, nullptr,
                                               nullptr);
        if (rc) return fail(ctx, CSIM_ERR_CUDA, "term launch failed");
        CK(cudaEventRecord(ctx->ev[2], ctx->stream));
        CKR(dbuf(ctx, kBufAcc, (size_t)c * 4 * sizeof(__int128), &v));
        __int128* dacc = (__int128*)v;
        if (csim::launch_reduce_parts(launch_of(ctx), dpart, c, nchunks, dacc))
            return fail(ctx, CSIM_ERR_CUDA, "reduce launch failed");
        CK(cudaEventRecord(ctx->ev[3], ctx->stream));
        code.resize(c);
        acc.resize(c * 4);
        CKR(dget(ctx, code.data(), dcode, c));
        CKR(dget(ctx, acc.data(), dacc, c * 4));
        CKR(finish(ctx));
        CKR(stats_batch(ctx));
        const double scale = pow(2, t);
        ctx->stats.states += c;
        for (int64_t i = 0; i < c; i++) {
            if (code[i] < 0) {
                values[o + i] = 0;
                continue;
            }
            ctx->stats.states_live++;
            ctx->stats.pairs += chi;
            double re, im;
            zomega_to_complex(&acc[4 * i], P2, &re, &im);
            const double pf = sqrt_half_power(code[i]);
            const double a = re * pf, b = im * pf;
            values[o + i] = scale * (a * a + b * b);
        }
    }
    return 0;
}

double clifford_sum(const csim_projector* P) {  // innerprod.c:52-62
    double sum = 1;
    for (int i = 0; i < P->nstabs; i++) {
        const double ph = (double)phase_m(P->phase[i]);
        if (ph == 0) sum += 1;
        if (ph == 2) sum -= 1;
    }
    return sum;
}

int cmp_trunc(const void* a, const void* b) {  // innerprod.c:17-19
    return (int)(*(const double*)a - *(const double*)b);
}

}  // namespace

extern "C" int csim_single_projector_samples(csim_ctx* ctx, const csim_projector* P, const uint64_t* L, int32_t k,
                                             int32_t exact, int64_t count, int32_t rng, uint64_t seed,
                                             double* values) {
    if (!ctx || count < 0 || (count && !values)) return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    CKR(check_projector(ctx, P));
    if (P->nqubits < 1) return fail(ctx, CSIM_ERR_ARG, "singleProjectorSample needs t >= 1");
    stats_begin(ctx);
    const int r = sample_values(ctx, P, L, k, exact, count, rng, seed, values);
    stats_end(ctx);
    return r;
}

extern "C" int csim_multi_sampled_projector(csim_ctx* ctx, const csim_projector* P, const uint64_t* L, int32_t k,
                                            int32_t exact, double norm, int32_t samples, int32_t bins, int32_t rng,
                                            uint64_t seed, double* out) {
    if (!ctx || !out || bins < 1 || samples < 0) return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    CKR(check_projector(ctx, P));
    stats_begin(ctx);
    if (P->nstabs == 0) {  // sampledProjector, innerprod.c:47
        *out = pow(norm, 2);
        return CSIM_OK;
    }
    if (P->nqubits == 0) {
        *out = pow(norm, 2) * clifford_sum(P) / (1 + (double)P->nstabs);
        return CSIM_OK;
    }
    std::vector<double> v((size_t)samples * bins);
    CKR(sample_values(ctx, P, L, k, exact, (int64_t)samples * bins, rng, seed, v.data()));
    stats_end(ctx);
    std::vector<double> binv(bins);
    for (int b = 0; b < bins; b++) {
        double total = 0;  // sequential, in draw order (innerprod.c:75-77)
        for (int i = 0; i < samples; i++) total += v[(size_t)b * samples + i];
        binv[b] = total / samples;
    }
    if (bins == 1) {
        *out = binv[0];
        return CSIM_OK;
    }
    qsort(binv.data(), (size_t)bins, sizeof(double), cmp_trunc);
    *out = (bins % 2 == 1) ? binv[(bins - 1) / 2] : (binv[bins / 2] + binv[bins / 2 - 1]) / 2;
    return CSIM_OK;
}

extern "C" int csim_exact_projector(csim_ctx* ctx, const csim_projector* P, const uint64_t* L, int32_t k,
                                    int32_t exact, double norm, double* out) {
    if (!ctx || !out) return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    CKR(check_projector(ctx, P));
    stats_begin(ctx);
    if (P->nstabs == 0) {  // innerprod.c:150
        *out = pow(norm, 2);
        return CSIM_OK;
    }
    const int t = P->nqubits;
    if (t == 0) {
        *out = clifford_sum(P) / (1 + (double)P->nstabs);
        return CSIM_OK;
    }
    CKR(check_code(ctx, t, exact, L, k));
    const int64_t chi = exact ? ((int64_t)1 << ((t + 1) / 2)) : ((int64_t)1 << k);
    if (chi > ((int64_t)1 << 20)) return fail(ctx, CSIM_ERR_ARG, "chi=%lld too large for the exact projector", (long long)chi);
    const int nr = t > 32 ? 2 : 1;
    const int P2 = 2 * t;
    void* v;
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    // the terms phi_j, and theta_i = projected copies of them
    csim_state* dphis;
    if (exact) {
        uint64_t* dcw;
        CKR(stage_terms(ctx, t, 1, L, k, 0, chi, &dcw, &dphis));
    } else {
        uint64_t* dL;
        CKR(dput(ctx, kBufL, L, (size_t)k, &dL));
        CKR(dbuf(ctx, kBufCodewords, chi * 8, &v));
        uint64_t* dcw = (uint64_t*)v;
        if (csim::launch_codewords(launch_of(ctx), dL, k, 0, chi, dcw))
            return fail(ctx, CSIM_ERR_CUDA, "codeword launch failed");
        CKR(dbuf(ctx, kBufPhis, chi * sizeof(csim_state), &v));
        dphis = (csim_state*)v;
        if (csim::launch_prep(launch_of(ctx), t, 0, dcw, nullptr, chi, (csim::GState*)dphis))
            return fail(ctx, CSIM_ERR_CUDA, "prepL launch failed");
    }
    CKR(dbuf(ctx, kBufA, chi * sizeof(csim_state), &v));
    csim::GState* dth = (csim::GState*)v;
    CK(cudaMemcpyAsync(dth, dphis, chi * sizeof(csim_state), cudaMemcpyDeviceToDevice, ctx->stream));
    std::vector<int> hm(P->nstabs);
    for (int r = 0; r < P->nstabs; r++) hm[r] = phase_m(P->phase[r]);
    int* dpm;
    uint64_t *dpz, *dpx;
    CKR(dput(ctx, kBufPm, hm.data(), hm.size(), &dpm));
    CKR(dput(ctx, kBufPz, P->zs, (size_t)P->nstabs, &dpz));
    CKR(dput(ctx, kBufPx, P->xs, (size_t)P->nstabs, &dpx));
    CKR(dbuf(ctx, kBufCode, chi * 4, &v));
    int* dcode = (int*)v;
    if (csim::launch_project(launch_of(ctx), nr, dth, chi, P->nstabs, dpm, dpz, dpx, dcode))
        return fail(ctx, CSIM_ERR_CUDA, "projection launch failed");
    const int64_t chunk = 64, nchunks = (chi + chunk - 1) / chunk;
    const size_t nparts = (size_t)chi * nchunks * 4;
    CKR(dbuf(ctx, kBufParts, nparts * sizeof(__int128), &v));
    __int128* dpart = (__int128*)v;
    CKR(dbuf(ctx, kBufPartsDiag, nparts * sizeof(__int128), &v));
    __int128* dpartd = (__int128*)v;
    CK(cudaMemsetAsync(dpart, 0, nparts * sizeof(__int128), ctx->stream));
    CK(cudaMemsetAsync(dpartd, 0, nparts * sizeof(__int128), ctx->stream));
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    if (csim::launch_terms(launch_of(ctx), nr, 2, nullptr, (const csim::GState*)dphis, dth, dcode, chi, 0, chi,
                           (int)chunk, P2, dpart, dpartd, nullptr, nullptr, nullptr))
        return fail(ctx, CSIM_ERR_CUDA, "term launch failed");
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    CKR(dbuf(ctx, kBufAcc, (size_t)chi * 4 * sizeof(__int128), &v));
    __int128* dacc = (__int128*)v;
    CKR(dbuf(ctx, kBufAccDiag, (size_t)chi * 4 * sizeof(__int128), &v));
    __int128* daccd = (__int128*)v;
    if (csim::launch_reduce_parts(launch_of(ctx), dpart, chi, nchunks, dacc) ||
        csim::launch_reduce_parts(launch_of(ctx), dpartd, chi, nchunks, daccd))
        return fail(ctx, CSIM_ERR_CUDA, "reduce launch failed");
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    std::vector<int> code(chi);
    std::vector<__int128> acc(chi * 4), accd(chi * 4);
    CKR(dget(ctx, code.data(), dcode, chi));
    CKR(dget(ctx, acc.data(), dacc, chi * 4));
    CKR(dget(ctx, accd.data(), daccd, chi * 4));
    CKR(finish(ctx));
    CKR(stats_batch(ctx));
    ctx->stats.states = chi;
    for (int64_t i = 0; i < chi; i++)
        if (code[i] >= 0) {
            ctx->stats.states_live++;
            ctx->stats.pairs += chi - i;
        }
    stats_end(ctx);
    // row i adds 2^{-c_i/2} (diag_i + 2 Re off_i): exact per row in Z[w],
    // rows summed in double in row order like exactProjector's loop
    double tr = 0, ti = 0;
    for (int64_t i = 0; i < chi; i++) {
        if (code[i] < 0) continue;
        const __int128* o = &acc[4 * i];
        const __int128* d = &accd[4 * i];
        // 2 Re(a + b w + c w^2 + d w^3) = 2a + (b - d)(w - w^3)
        const __int128 z[4] = {d[0] + 2 * o[0], d[1] + (o[1] - o[3]), d[2], d[3] - (o[1] - o[3])};
        double re, im;
        zomega_to_complex(z, P2, &re, &im);
        const double pf = sqrt_half_power(code[i]);
        tr += re * pf;
        ti += im * pf;
    }
    *out = sqrt(tr * tr + ti * ti);
    return CSIM_OK;
}

// ---------------------------------------------------------------- decompose
namespace {

int gf2_rank(const uint64_t* rows, int nrows) {
    uint64_t m[CSIM_MAX_QUBITS];
    memcpy(m, rows, sizeof(uint64_t) * (size_t)nrows);
    int rank = 0;
    for (int c = 0; c < 64 && rank < nrows; c++) {
        int piv = -1;
        for (int r = rank; r < nrows; r++)
            if ((m[r] >> c) & 1) {
                piv = r;
                break;
            }
        if (piv < 0) continue;
        std::swap(m[piv], m[rank]);
        for (int r = 0; r < nrows; r++)
            if (r != rank && ((m[r] >> c) & 1)) m[r] ^= m[rank];
        rank++;
    }
    return rank;
}

}  // namespace

extern "C" int csim_decompose(int32_t t, double fidbound, int32_t rank, int32_t fidelity, int32_t force_l,
                              int32_t verbose, int32_t quiet, int32_t* exact, int32_t* k, double* norm,
                              uint64_t* L_out, void* rng_state, FILE* log) {
    if (!exact || !k || !norm || !L_out || !rng_state || t < 0 || t > CSIM_MAX_QUBITS) return CSIM_ERR_ARG;
    LibcRand& lr = *(LibcRand*)rng_state;
    if (t == 0) {
        *exact = 0;
        *norm = 1;
        return CSIM_OK;
    }
    const double v = cos(3.14159265358979323846 / 8);
    *norm = pow(2, floor((float)t / 2) / 2);
    if (t % 2) *norm *= 2 * v;
    if (*exact) return CSIM_OK;
    int forceK = 1;
    if (*k <= 0) {
        forceK = 0;
        *k = (int)ceil(1 - 2 * t * log2(v) - log2(fidbound));
        if (verbose && log) fprintf(log, "Autopicking k = %d to achieve delta = %f.\n", *k, fidbound);
    }
    if (*k > t / 2 && !forceK && !force_l) {
        if (verbose && log) fprintf(log, "k > t/2. Reverting to exact decomposition.\n");
        *exact = 1;
        return CSIM_OK;
    }
    if (*k > t) {
        if (forceK && !quiet && log) fprintf(log, "Can't have k > t. Setting k to %d.\n", t);
        *k = t;
    }
    if (*k > 40) return CSIM_ERR_ARG;
    double inner = 0, Z_L = 0;
    while (inner < 1 - fidbound || forceK) {
        const int kk = *k, bytes = (kk * t + 7) / 8;
        for (int i = 0; i < kk; i++) L_out[i] = 0;
        for (int b = 0; b < bytes; b++) {  // BitMatrixSetRandom over the row-major bit array
            const int byte = lr.next() % 256;
            for (int j = 0; j < 8; j++) {
                const int g = 8 * b + j;
                if (g < kk * t && (byte & (0x80 >> j))) L_out[g / t] |= 1ull << (g % t);
            }
        }
        if (rank && gf2_rank(L_out, kk) < kk) {
            if (!quiet && log) fprintf(log, "L has insufficient rank. Sampling again...\n");
            continue;
        }
        if (fidelity) {
            Z_L = 0;  // Z(L) = sum_x 2^{-|x|/2}, with the reference's integer division
            for (int64_t i = 0; i < ((int64_t)1 << kk); i++) Z_L += pow(2, -popc(codeword(i, L_out, kk)) / 2);
            inner = pow(2, kk) * pow(v, 2 * t) / Z_L;
            if (forceK) {
                if (log) fprintf(log, "delta = 1 - <H^t|L>: %lf\n", 1 - inner);
                break;
            } else if (inner < 1 - fidbound) {
                if (!quiet && log) fprintf(log, "delta = 1 - <H^t|L>: %lf - Not good enough!\n", 1 - inner);
            } else {
                if (!quiet && log) fprintf(log, "delta = 1 - <H^t|L>: %lf\n", 1 - inner);
            }
        } else {
            break;
        }
    }
    if (fidelity) *norm = sqrt(pow(2, *k) * Z_L);
    return CSIM_OK;
}

// ---------------------------------------------------------------- many queries
#include "csim_batch.h"

namespace {

enum BatchBuf {
    kBbL = 100, kBbCodes, kBbCw, kBbPhis, kBbStates, kBbCodesOut, kBbDesc, kBbWords, kBbCum, kBbProj,
    kBbItemsTp, kBbItemsW, kBbPartTp, kBbPartTpD, kBbPartW, kBbPartWD, kBbFirstTp, kBbFirstW, kBbSumTp, kBbSumTpD,
    kBbSumW, kBbSumWD, kBbIdx
};

// one projector evaluation (numerator or denominator) of one query
struct Eval {
    int query, which;       // which: 0 = G', 1 = H'
    int kind;               // 0 host-only value, 1 sampled, 2 exact projector
    double value;           // kind 0 result, filled at the end otherwise
    int64_t s0, ns;         // its states [s0, s0 + ns)
    int t, exact, k, samples, bins;
    double norm;
};

struct QueryPlan {
    int exact, k, noapprox, t;
    double norm;
    uint64_t L[CSIM_MAX_QUBITS];
    int64_t cw_off;       // codeword table offset (exact == 0)
    int64_t phis_off;     // term-state offset (exact == 1, or exact projector)
    int64_t chi;
};

}  // namespace

// the batched executor's buffers follow the single-query ones in the context's pool
static int bbuf(csim_ctx* ctx, int id, size_t bytes, void** out) { return dbuf(ctx, id - 100 + kNumBufs, bytes, out); }

extern "C" int csim_run_queries(csim_ctx* ctx, int64_t nq, const csim_query* q, csim_query_result* r,
                                int32_t batched) {
    if (!ctx || nq < 0 || (nq && (!q || !r))) return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    // ---- per-query host plan: decompose and the noapprox rule (probability.c:146-174)
    std::vector<QueryPlan> plan(nq);
    int first_err = CSIM_OK;
    for (int64_t i = 0; i < nq; i++) {
        csim_query_result& R = r[i];
        R = csim_query_result{};
        QueryPlan& P = plan[i];
        const csim_query& Q = q[i];
        if (Q.t < 0 || Q.t > CSIM_MAX_QUBITS || (Q.rng != CSIM_RNG_LIBC && Q.rng != CSIM_RNG_PHILOX) ||
            check_projector(ctx, &Q.G) || check_projector(ctx, &Q.H) || (Q.G.nstabs && Q.G.nqubits != Q.t) ||
            (Q.H.nstabs && Q.H.nqubits != Q.t)) {
            R.status = fail(ctx, CSIM_ERR_ARG, "query %lld: bad t, rng or projectors", (long long)i);
            if (!first_err) first_err = CSIM_ERR_ARG;
            continue;
        }
        LibcRand ds;
        ds.seed(1);
        P.exact = Q.exact;
        P.k = Q.k;
        P.t = Q.t;
        memset(P.L, 0, sizeof(P.L));
        int rc = csim_decompose(Q.t, Q.fidbound, Q.rank, Q.fidelity, Q.force_l, Q.verbose, Q.quiet, &P.exact, &P.k,
                                &P.norm, P.L, &ds, nullptr);
        if (rc != CSIM_OK) {
            R.status = rc;
            if (!first_err) first_err = rc;
            continue;
        }
        P.noapprox = Q.noapprox;
        if (Q.noapprox == 0 && Q.force_sample == 0) {
            const double terms = P.exact ? pow(2, (Q.t + 1) / 2) : pow(2, P.k);
            if (Q.samples * Q.bins * 2 > (terms - 1)) P.noapprox = 1;
        }
        if (P.noapprox == 0 && (Q.bins < 1 || Q.samples < 0)) {  // the sampler needs bins >= 1
            R.status = fail(ctx, CSIM_ERR_ARG, "query %lld: samples=%d bins=%d", (long long)i, Q.samples, Q.bins);
            if (!first_err) first_err = CSIM_ERR_ARG;
            continue;
        }
        P.chi = Q.t == 0 ? 0 : (P.exact ? ((int64_t)1 << ((Q.t + 1) / 2)) : ((int64_t)1 << P.k));
        R.exact = P.exact;
        R.k = P.k;
        R.noapprox = P.noapprox;
        R.norm = P.norm;
    }

    if (!batched) {  // ---- one query at a time through the single-query entry points
        for (int64_t i = 0; i < nq; i++) {
            if (r[i].status) continue;
            const QueryPlan& P = plan[i];
            const csim_query& Q = q[i];
            int rc;
            int64_t pairs = 0;
            if (P.noapprox == 0) {
                rc = csim_multi_sampled_projector(ctx, &Q.G, P.L, P.k, P.exact, P.norm, Q.samples, Q.bins, Q.rng,
                                                  Q.rng == CSIM_RNG_LIBC ? (uint64_t)(uint32_t)Q.seed : Q.seed,
                                                  &r[i].numerator);
                pairs += ctx->stats.pairs;
                if (rc == CSIM_OK)
                    rc = csim_multi_sampled_projector(ctx, &Q.H, P.L, P.k, P.exact, P.norm, Q.samples, Q.bins, Q.rng,
                                                      CSIM_SEED_CONTINUE, &r[i].denominator);
                pairs += ctx->stats.pairs;
            } else {
                rc = csim_exact_projector(ctx, &Q.G, P.L, P.k, P.exact, P.norm, &r[i].numerator);
                pairs += ctx->stats.pairs;
                if (rc == CSIM_OK) rc = csim_exact_projector(ctx, &Q.H, P.L, P.k, P.exact, P.norm, &r[i].denominator);
                pairs += ctx->stats.pairs;
            }
            r[i].pairs = pairs;
            r[i].status = rc;
            if (rc && !first_err) first_err = rc;
        }
        return first_err;
    }

    // ---- batched: evaluations, states, items
    stats_begin(ctx);
    CK(cudaEventRecord(ctx->ev[0], ctx->stream));
    std::vector<Eval> ev;
    int nmax_tp = 1;
    for (int64_t i = 0; i < nq; i++) {
        if (r[i].status) continue;
        const QueryPlan& P = plan[i];
        const csim_query& Q = q[i];
        for (int w = 0; w < 2; w++) {
            const csim_projector& Pr = w == 0 ? Q.G : Q.H;
            Eval e{};
            e.query = (int)i;
            e.which = w;
            e.t = Q.t;
            e.exact = P.exact;
            e.k = P.k;
            e.samples = Q.samples;
            e.bins = Q.bins;
            e.norm = P.norm;
            if (Pr.nstabs == 0) {  // innerprod.c:47 / :150
                e.kind = 0;
                e.value = pow(P.norm, 2);
            } else if (Q.t == 0) {
                e.kind = 0;
                e.value = (P.noapprox ? 1.0 : pow(P.norm, 2)) * clifford_sum(&Pr) / (1 + (double)Pr.nstabs);
            } else {
                e.kind = P.noapprox ? 2 : 1;
                if (check_code(ctx, Q.t, P.exact, P.L, P.k)) {
                    r[i].status = CSIM_ERR_ARG;
                    if (!first_err) first_err = CSIM_ERR_ARG;
                    break;
                }
                if (e.kind == 2 && P.chi > ((int64_t)1 << 20)) {
                    r[i].status = fail(ctx, CSIM_ERR_ARG, "chi too large for the exact projector");
                    if (!first_err) first_err = CSIM_ERR_ARG;
                    break;
                }
                if (!P.exact) nmax_tp = std::max(nmax_tp, Q.t);
            }
            ev.push_back(e);
        }
    }
    // codeword tables (|L> queries) and term states (prepH queries, and every exact projector)
    std::vector<uint64_t> hL;
    std::vector<csim::CodeDesc> hcodes;
    int64_t cw_total = 0, maxchi = 1;
    for (int64_t i = 0; i < nq; i++) {
        QueryPlan& P = plan[i];
        P.cw_off = -1;
        if (r[i].status || q[i].t == 0 || P.exact) continue;
        P.cw_off = cw_total;
        cw_total += P.chi;
        maxchi = std::max(maxchi, P.chi);
    }
    void* v;
    uint64_t* dL;
    uint64_t* dcw = nullptr;
    if (cw_total) {
        hL.assign(64 * (size_t)nq, 0);
        for (int64_t i = 0; i < nq; i++)
            if (plan[i].cw_off >= 0) memcpy(&hL[64 * (size_t)i], plan[i].L, sizeof(plan[i].L));
        CKR(dput(ctx, kNumBufs + (kBbL - 100), hL.data(), hL.size(), &dL));
        for (int64_t i = 0; i < nq; i++)
            if (plan[i].cw_off >= 0) hcodes.push_back(csim::CodeDesc{dL + 64 * i, plan[i].k, 0, plan[i].cw_off});
        csim::CodeDesc* dcodes;
        CKR(dput(ctx, kNumBufs + (kBbCodes - 100), hcodes.data(), hcodes.size(), &dcodes));
        CKR(bbuf(ctx, kBbCw, (size_t)cw_total * 8, &v));
        dcw = (uint64_t*)v;
        if (csim::launch_codewords_multi(launch_of(ctx), dcodes, (int)hcodes.size(), maxchi, dcw))
            return fail(ctx, CSIM_ERR_CUDA, "codeword launch failed");
    }
    // term states: exact-decomposition terms, and the |L> term states the exact projector starts from
    int64_t phis_total = 0;
    for (int64_t i = 0; i < nq; i++) {
        QueryPlan& P = plan[i];
        P.phis_off = -1;
        if (r[i].status || q[i].t == 0) continue;
        if (P.exact || P.noapprox) {
            P.phis_off = phis_total;
            phis_total += P.chi;
        }
    }
    csim_state* dphis = nullptr;  // term states, as csim_state for the offsets below
    if (phis_total) {
        CKR(bbuf(ctx, kBbPhis, (size_t)phis_total * sizeof(csim_state), &v));
        dphis = (csim_state*)v;
        // prepH term indices 0..chi-1, shared by every exact-decomposition query
        int64_t maxchi_h = 0;
        for (int64_t i = 0; i < nq; i++)
            if (plan[i].phis_off >= 0 && plan[i].exact) maxchi_h = std::max(maxchi_h, plan[i].chi);
        std::vector<int64_t> idx(maxchi_h);
        for (int64_t j = 0; j < maxchi_h; j++) idx[j] = j;
        int64_t* di = nullptr;
        if (maxchi_h) CKR(dput(ctx, kNumBufs + (kBbIdx - 100), idx.data(), idx.size(), &di));
        for (int64_t i = 0; i < nq; i++) {
            const QueryPlan& P = plan[i];
            if (P.phis_off < 0) continue;
            if (P.exact) {
                if (csim::launch_prep(launch_of(ctx), P.t, 1, nullptr, di, P.chi, (csim::GState*)(dphis + P.phis_off)))
                    return fail(ctx, CSIM_ERR_CUDA, "prepH launch failed");
            } else {
                if (csim::launch_prep(launch_of(ctx), P.t, 0, dcw + P.cw_off, nullptr, P.chi, (csim::GState*)(dphis + P.phis_off)))
                    return fail(ctx, CSIM_ERR_CUDA, "prepL launch failed");
            }
        }
    }
    // cumulative tables per t, projector rows per evaluation
    std::vector<double> hcum(65 * 65, 0.0);
    for (int t = 1; t <= 64; t++) cum_table(t, &hcum[65 * t]);
    double* dcum;
    CKR(dput(ctx, kNumBufs + (kBbCum - 100), hcum.data(), hcum.size(), &dcum));
    std::vector<uint64_t> hproj;  // per evaluation: 64 m (as uint64), 64 zeta, 64 xi
    hproj.assign(ev.size() * 192, 0);
    for (size_t e = 0; e < ev.size(); e++) {
        if (ev[e].kind == 0) continue;
        const csim_projector& Pr = ev[e].which == 0 ? q[ev[e].query].G : q[ev[e].query].H;
        int32_t* pm = reinterpret_cast<int32_t*>(&hproj[192 * e]);
        for (int rr = 0; rr < Pr.nstabs && rr < 64; rr++) {
            pm[rr] = phase_m(Pr.phase[rr]);
            hproj[192 * e + 64 + rr] = Pr.zs[rr];
            hproj[192 * e + 128 + rr] = Pr.xs[rr];
        }
        if (Pr.nstabs > 64) {
            r[ev[e].query].status = fail(ctx, CSIM_ERR_ARG, "more than 64 stabilizers");
            ev[e].kind = 0;
            ev[e].value = 0;
            if (!first_err) first_err = CSIM_ERR_ARG;
        }
    }
    uint64_t* dproj;
    CKR(dput(ctx, kNumBufs + (kBbProj - 100), hproj.data(), hproj.size(), &dproj));

    // states: draws (sampled) or copies of term states (exact projector); LIBC words per query
    std::vector<csim::DrawDesc> desc;
    std::vector<uint32_t> words;
    std::vector<int> qlive(nq, 1);
    {
        std::vector<LibcRand> lr(nq);
        std::vector<uint64_t> philox_next(nq, 0);
        for (int64_t i = 0; i < nq; i++) lr[i].seed((uint32_t)q[i].seed);
        for (size_t e = 0; e < ev.size(); e++) {
            Eval& E = ev[e];
            if (E.kind == 0 || r[E.query].status) continue;
            const csim_query& Q = q[E.query];
            const QueryPlan& P = plan[E.query];
            const csim_projector& Pr = E.which == 0 ? Q.G : Q.H;
            E.s0 = (int64_t)desc.size();
            csim::DrawDesc d{};
            d.n = Q.t;
            d.nstabs = Pr.nstabs;
            d.cum = dcum + 65 * Q.t;
            d.pm = reinterpret_cast<const int32_t*>(dproj + 192 * e);
            d.pz = dproj + 192 * e + 64;
            d.px = dproj + 192 * e + 128;
            if (E.kind == 1) {
                E.ns = (int64_t)Q.samples * Q.bins;
                for (int64_t s = 0; s < E.ns; s++) {
                    if (Q.rng == CSIM_RNG_LIBC) {
                        d.mode = 1;
                        d.wbegin = (int64_t)words.size();
                        draw_state_words(lr[E.query], Q.t, &hcum[65 * Q.t], words);
                        d.wend = (int64_t)words.size();
                    } else {
                        d.mode = 0;
                        d.seed = Q.seed;
                        d.id = philox_next[E.query]++;
                    }
                    desc.push_back(d);
                }
            } else {
                E.ns = P.chi;
                d.mode = 2;
                for (int64_t s = 0; s < E.ns; s++) {
                    d.src = (const csim::GState*)(dphis + P.phis_off + s);
                    desc.push_back(d);
                }
            }
        }
    }
    const int64_t nstates = (int64_t)desc.size();
    uint32_t* dwords = nullptr;
    if (!words.empty()) CKR(dput(ctx, kNumBufs + (kBbWords - 100), words.data(), words.size(), &dwords));
    for (auto& d : desc)
        if (d.mode == 1) d.words = dwords;
    csim::DrawDesc* ddesc;
    CKR(dput(ctx, kNumBufs + (kBbDesc - 100), desc.data(), desc.size(), &ddesc));
    CKR(bbuf(ctx, kBbStates, (size_t)std::max<int64_t>(nstates, 1) * sizeof(csim_state), &v));
    csim::GState* dstates = (csim::GState*)v;
    CKR(bbuf(ctx, kBbCodesOut, (size_t)std::max<int64_t>(nstates, 1) * 4, &v));
    int* dcode = (int*)v;
    if (csim::launch_draw_project(launch_of(ctx), ddesc, nstates, dstates, dcode))
        return fail(ctx, CSIM_ERR_CUDA, "draw/project launch failed");

    // work items, grouped by state
    std::vector<csim::PairItem> itp, iw;
    std::vector<int64_t> ftp(nstates + 1, 0), fw(nstates + 1, 0);
    const int per_thread = ctx->per_thread;
    const int64_t span_tp = 64 * (int64_t)per_thread, span_w = 64;
    for (size_t e = 0; e < ev.size(); e++) {
        const Eval& E = ev[e];
        if (E.kind == 0 || r[E.query].status) continue;
        const QueryPlan& P = plan[E.query];
        for (int64_t s = 0; s < E.ns; s++) {
            const int64_t st = E.s0 + s;
            const int64_t jb = E.kind == 2 ? s : 0;  // exact projector row s: terms j >= s
            const int64_t diag = E.kind == 2 ? s : -1;
            ftp[st] = (int64_t)itp.size();
            fw[st] = (int64_t)iw.size();
            if (!P.exact) {
                for (int64_t j = jb; j < P.chi; j += span_tp)
                    itp.push_back(csim::PairItem{st, j, std::min(span_tp, P.chi - j), diag, dcw + P.cw_off, nullptr});
            } else {
                for (int64_t j = jb; j < P.chi; j += span_w)
                    iw.push_back(csim::PairItem{st, j, std::min(span_w, P.chi - j), diag, nullptr,
                                                (const csim::GState*)(dphis + P.phis_off)});
            }
        }
    }
    ftp[nstates] = (int64_t)itp.size();
    fw[nstates] = (int64_t)iw.size();
    // make the range ends monotone: a state's range is [f[s], f[s+1])
    for (int64_t st = nstates - 1; st >= 0; st--) {
        ftp[st] = std::min(ftp[st], ftp[st + 1]);
        fw[st] = std::min(fw[st], fw[st + 1]);
    }
    csim::PairItem *ditp = nullptr, *diw = nullptr;
    int64_t *dftp, *dfw;
    if (!itp.empty()) CKR(dput(ctx, kNumBufs + (kBbItemsTp - 100), itp.data(), itp.size(), &ditp));
    if (!iw.empty()) CKR(dput(ctx, kNumBufs + (kBbItemsW - 100), iw.data(), iw.size(), &diw));
    CKR(dput(ctx, kNumBufs + (kBbFirstTp - 100), ftp.data(), ftp.size(), &dftp));
    CKR(dput(ctx, kNumBufs + (kBbFirstW - 100), fw.data(), fw.size(), &dfw));
    __int128 *dptp, *dptpd, *dpw, *dpwd;
    CKR(bbuf(ctx, kBbPartTp, (itp.size() + 1) * 64, &v)); dptp = (__int128*)v;
    CKR(bbuf(ctx, kBbPartTpD, (itp.size() + 1) * 64, &v)); dptpd = (__int128*)v;
    CKR(bbuf(ctx, kBbPartW, (iw.size() + 1) * 64, &v)); dpw = (__int128*)v;
    CKR(bbuf(ctx, kBbPartWD, (iw.size() + 1) * 64, &v)); dpwd = (__int128*)v;
    CK(cudaEventRecord(ctx->ev[1], ctx->stream));
    if (csim::launch_items_tp(launch_of(ctx), ditp, (int64_t)itp.size(), dstates, dcode, per_thread, nmax_tp, dptp,
                              dptpd) ||
        csim::launch_items_warp(launch_of(ctx), diw, (int64_t)iw.size(), dstates, dcode, dpw, dpwd))
        return fail(ctx, CSIM_ERR_CUDA, "pair launch failed");
    CK(cudaEventRecord(ctx->ev[2], ctx->stream));
    __int128 *dstp, *dstpd, *dsw, *dswd;
    CKR(bbuf(ctx, kBbSumTp, (size_t)(nstates + 1) * 64, &v)); dstp = (__int128*)v;
    CKR(bbuf(ctx, kBbSumTpD, (size_t)(nstates + 1) * 64, &v)); dstpd = (__int128*)v;
    CKR(bbuf(ctx, kBbSumW, (size_t)(nstates + 1) * 64, &v)); dsw = (__int128*)v;
    CKR(bbuf(ctx, kBbSumWD, (size_t)(nstates + 1) * 64, &v)); dswd = (__int128*)v;
    if (csim::launch_reduce_slots(launch_of(ctx), dptp, dftp, nstates, dstp) ||
        csim::launch_reduce_slots(launch_of(ctx), dptpd, dftp, nstates, dstpd) ||
        csim::launch_reduce_slots(launch_of(ctx), dpw, dfw, nstates, dsw) ||
        csim::launch_reduce_slots(launch_of(ctx), dpwd, dfw, nstates, dswd))
        return fail(ctx, CSIM_ERR_CUDA, "reduce launch failed");
    CK(cudaEventRecord(ctx->ev[3], ctx->stream));
    std::vector<int> code(std::max<int64_t>(nstates, 1));
    std::vector<__int128> stp(nstates * 4 + 4), stpd(nstates * 4 + 4), sw(nstates * 4 + 4), swd(nstates * 4 + 4);
    CKR(dget(ctx, code.data(), dcode, nstates));
    CKR(dget(ctx, stp.data(), dstp, nstates * 4));
    CKR(dget(ctx, stpd.data(), dstpd, nstates * 4));
    CKR(dget(ctx, sw.data(), dsw, nstates * 4));
    CKR(dget(ctx, swd.data(), dswd, nstates * 4));
    {
        const int fr = finish(ctx);
        if (fr) return fr;
    }
    CKR(stats_batch(ctx));

    // ---- per-evaluation reductions on the host (innerprod.c:23-84, :148-199)
    std::vector<double> vals;
    for (size_t e = 0; e < ev.size(); e++) {
        Eval& E = ev[e];
        if (E.kind == 0 || r[E.query].status) continue;
        const int P2 = 2 * E.t;
        const int64_t chi = plan[E.query].chi;
        if (E.kind == 1) {
            vals.assign(E.ns, 0.0);
            const double scale = pow(2, E.t);
            for (int64_t s = 0; s < E.ns; s++) {
                const int64_t st = E.s0 + s;
                ctx->stats.states++;
                if (code[st] < 0) continue;
                ctx->stats.states_live++;
                ctx->stats.pairs += chi;
                r[E.query].pairs += chi;
                __int128 z[4];
                for (int qq = 0; qq < 4; qq++) z[qq] = stp[4 * st + qq] + sw[4 * st + qq];
                double re, im;
                zomega_to_complex(z, P2, &re, &im);
                const double pf = sqrt_half_power(code[st]);
                const double a = re * pf, b = im * pf;
                vals[s] = scale * (a * a + b * b);
            }
            std::vector<double> binv(E.bins);
            for (int b = 0; b < E.bins; b++) {
                double total = 0;
                for (int i = 0; i < E.samples; i++) total += vals[(size_t)b * E.samples + i];
                binv[b] = total / E.samples;
            }
            if (E.bins == 1) {
                E.value = binv[0];
            } else {
                qsort(binv.data(), (size_t)E.bins, sizeof(double), cmp_trunc);
                E.value = (E.bins % 2 == 1) ? binv[(E.bins - 1) / 2] : (binv[E.bins / 2] + binv[E.bins / 2 - 1]) / 2;
            }
        } else {
            double tr = 0, ti = 0;
            for (int64_t s = 0; s < E.ns; s++) {
                const int64_t st = E.s0 + s;
                ctx->stats.states++;
                if (code[st] < 0) continue;
                ctx->stats.states_live++;
                ctx->stats.pairs += chi - s;
                r[E.query].pairs += chi - s;
                __int128 o[4], d[4];
                for (int qq = 0; qq < 4; qq++) {
                    o[qq] = stp[4 * st + qq] + sw[4 * st + qq];
                    d[qq] = stpd[4 * st + qq] + swd[4 * st + qq];
                }
                const __int128 z[4] = {d[0] + 2 * o[0], d[1] + (o[1] - o[3]), d[2], d[3] - (o[1] - o[3])};
                double re, im;
                zomega_to_complex(z, P2, &re, &im);
                const double pf = sqrt_half_power(code[st]);
                tr += re * pf;
                ti += im * pf;
            }
            E.value = sqrt(tr * tr + ti * ti);
        }
    }
    for (const Eval& E : ev) {
        if (r[E.query].status) continue;
        if (E.which == 0) r[E.query].numerator = E.value;
        else r[E.query].denominator = E.value;
    }
    stats_end(ctx);
    return first_err;
}
