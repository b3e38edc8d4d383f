// csim_host_common.h — host-side pieces shared by the single-query entry
// points (csim_host.cpp) and the query engine (csim_engine.cpp): the C
// library's rand() sequence, randomStabilizerState's tables, Z[w] -> double
// conversion, the context with its device-buffer pool, error handling and the
// argument checks.
#pragma once

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

namespace csim_host {


// ---------------------------------------------------------------- libc rand()
// The C library's srand()/rand(): additive lagged-Fibonacci r_i = r_{i-3} +
// r_{i-31} (mod 2^32) seeded by the Park–Miller recurrence (Schrage's method),
// first 310 outputs discarded, outputs r_i >> 1 (P. Selinger, "The GLIBC
// pseudo-random number generator").
struct LibcRand {
    uint32_t ring[34];
    int idx;

    LibcRand() { seed(1); }  // rand() before any srand() is seeded with 1

    uint32_t step() {
        const int i31 = idx + 31 >= 34 ? idx - 3 : idx + 31, i3 = idx + 3 >= 34 ? idx - 31 : idx + 3;
        const uint32_t v = ring[i31] + ring[i3];
        ring[idx] = v;
        idx = idx == 33 ? 0 : idx + 1;
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
inline double logeta(int d, int n) {
    if (d == 0) return 0.;
    double product = 0;
    for (int a = 1; a <= d; a++) {
        product += log2(1 - pow(2, d - n - a));
        product -= log2(1 - pow(2, -a));
    }
    return (-d * (d + 1) / 2) + product;
}

inline void cum_table(int n, double* cum) {
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

inline uint64_t codeword(int64_t j, const uint64_t* L, int k) {
    uint64_t x = 0;
    for (int r = 0; r < k; r++)
        if ((j >> (k - 1 - r)) & 1) x ^= L[r];
    return x;
}

// The rand() words randomStabilizerState consumes for one n-qubit state, drawn
// from `lr` in the reference's order.  The lazy shrink loop is simulated on G
// alone to know how many random vectors are drawn (stabilizer.c:736-740).
inline void draw_state_words(LibcRand& lr, int n, const double* cum, std::vector<uint32_t>& words) {
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
    const size_t w0 = words.size();
    words.resize(w0 + (size_t)rest);
    for (int64_t i = 0; i < rest; i++) words[w0 + (size_t)i] = (uint32_t)lr.next();
}

// Zero bound of the "light" part of an ordered codeword table: codewords with
// at most this many zeros run in a launch whose G-column slots are sized for
// it, which leaves shared memory for more resident blocks.  Weights of a
// random code's codewords cluster at t/2, so most terms fall in this part.
inline int light_zeros(int t) { return std::min(t, (3 * t + 4) / 5); }

// Terms per thread per work item of the thread-per-pair kernels when the
// caller leaves it open (0): items of 2048 terms share their top-bit shrinks
// among more pairs, which pays up to t = 52; above that, items of 1024 keep
// more of them resident per SM (measured: t = 24 +5%, t = 40 +1.5%, t = 64
// -3% for 2048).
inline int auto_per_thread(int t) { return t <= 52 ? 32 : 16; }
inline int tp_per_thread(int fixed, int t) { return fixed > 0 ? fixed : auto_per_thread(t); }

// Launch parameters of the thread-per-pair kernels for one t: terms per thread
// per work item (items of 64 * per_thread terms) and the zero bound of the
// light launch.  The defaults are the rules above; a context's autotuner
// (csim_autotune) replaces them per t bucket with the fastest measured pair.
struct TpTune {
    int per_thread = 0;
    int light = 0;
    int kernel = 0;  // 0: block-prefix kernel (k_terms_tp), heavy and light launches; 1: run kernel
                     // (k_terms_runs); 2: block-prefix kernel, one launch per occupancy class; 3: direct
                     // kernel (k_terms_direct), states with many non-pivot coordinates on kernel 0
};
// constraint slots per pair of the direct kernel: states with more non-pivot
// coordinates (n - k) than this go to the block-prefix kernel
inline int direct_slots(int t) { return std::min(t, 8); }
// The direct kernel's light bound: above 32 qubits the table's heavy part
// (more than t - 33 zeros) holds the codewords of at most 32 ones, whose pairs
// have at most 32 live variables; the block-prefix launches of the states
// left to them use the same bound.
inline int direct_light(int t) { return t > 32 ? t - 33 : light_zeros(t); }
inline TpTune default_tune(int t) {
    TpTune r;
    r.per_thread = auto_per_thread(t);
    r.light = light_zeros(t);
    r.kernel = 0;
    return r;
}

// Codeword-order parameter: the top-bit groups of ordered_codewords hold
// 2^11 terms, one or two kernel blocks (items of 2^11 or 2^10 terms)
inline int ordered_prefix_bits(int k, int t) { return std::max(0, std::min(t, k - 11)); }

// The 2^k codewords of L in the order the thread-per-pair kernel walks them in
// a sampled estimator.  First those with more than light_zeros(t) zeros (the
// heavy launch), then the rest (light_split finds the boundary); within each
// part by the top d = ordered_prefix_bits(k, t) bits, then by weight, then by
// value.  A block's consecutive codewords then agree on long top bits, whose
// shrinks the block runs once for all of its pairs (prefix_shrink), and the 32
// pairs of a warp mostly have the same number of shrinks, so the warp's
// predicated loops waste few lanes.  A state's sum over all terms is exact,
// so it does not depend on the order.
inline void ordered_codewords(const uint64_t* L, int k, int t, int lz, std::vector<uint64_t>& out) {
    const int64_t chi = (int64_t)1 << k;
    out.resize((size_t)chi);
    uint64_t x = 0;
    out[0] = 0;
    for (int64_t i = 1; i < chi; i++) {  // Gray code: one row of L per step
        x ^= L[k - 1 - __builtin_ctzll((unsigned long long)i)];
        out[(size_t)i] = x;
    }
    const int wmin = t - lz;
    const int d = ordered_prefix_bits(k, t);
    std::sort(out.begin(), out.end(), [wmin, d, t](uint64_t a, uint64_t b) {
        const int pa = __builtin_popcountll(a), pb = __builtin_popcountll(b);
        const bool ha = pa < wmin, hb = pb < wmin;
        if (ha != hb) return ha;
        const uint64_t ta = d ? a >> (t - d) : 0, tb = d ? b >> (t - d) : 0;
        if (ta != tb) return ta < tb;
        return pa != pb ? pa < pb : a < b;
    });
}

inline void ordered_codewords(const uint64_t* L, int k, int t, std::vector<uint64_t>& out) {
    ordered_codewords(L, k, t, light_zeros(t), out);
}

// First index of an ordered table (heavy part first) from which every codeword
// has at most lz zeros.
inline int64_t light_split(const std::vector<uint64_t>& cw, int t, int lz) {
    const int wmin = t - lz;
    int64_t j = 0;
    while (j < (int64_t)cw.size() && __builtin_popcountll(cw[(size_t)j]) < wmin) j++;
    return j;
}
inline int64_t light_split(const std::vector<uint64_t>& cw, int t) { return light_split(cw, t, light_zeros(t)); }

// The 2^k codewords of L ordered for launches by zero class: bounds[0] = t >
// bounds[1] > ... are the G-slot bounds of the launches; class c holds the
// codewords with at most bounds[c] zeros and more than bounds[c + 1].  Classes
// in order (most zeros first), each ordered as ordered_codewords orders a
// part (top bits, weight, value).  starts[c] = first index of class c.  With
// bounds {t, light_zeros(t)} this is ordered_codewords' order.
inline void ordered_codewords_classes(const uint64_t* L, int k, int t, const std::vector<int>& bounds,
                                      std::vector<uint64_t>& out, std::vector<int64_t>& starts) {
    const int64_t chi = (int64_t)1 << k;
    out.resize((size_t)chi);
    uint64_t x = 0;
    out[0] = 0;
    for (int64_t i = 1; i < chi; i++) {
        x ^= L[k - 1 - __builtin_ctzll((unsigned long long)i)];
        out[(size_t)i] = x;
    }
    const int nc = (int)bounds.size();
    auto cls = [&bounds, nc, t](uint64_t v) {
        const int z = t - __builtin_popcountll(v);
        int c = 0;
        while (c + 1 < nc && z <= bounds[(size_t)c + 1]) c++;
        return c;
    };
    const int d = ordered_prefix_bits(k, t);
    std::sort(out.begin(), out.end(), [&cls, d, t](uint64_t a, uint64_t b) {
        const int ca = cls(a), cb = cls(b);
        if (ca != cb) return ca < cb;
        const uint64_t ta = d ? a >> (t - d) : 0, tb = d ? b >> (t - d) : 0;
        if (ta != tb) return ta < tb;
        const int pa = __builtin_popcountll(a), pb = __builtin_popcountll(b);
        return pa != pb ? pa < pb : a < b;
    });
    starts.assign((size_t)nc + 1, chi);
    for (int64_t i = chi - 1; i >= 0; i--) starts[(size_t)cls(out[(size_t)i])] = i;
    for (int c = nc - 1; c >= 0; c--) starts[(size_t)c] = std::min(starts[(size_t)c], starts[(size_t)c + 1]);
}

// Top bits of [0, n) on which codewords that differ in the bits `dis` agree
// (csim::pc::agree_top's host twin)
inline uint64_t agree_top_host(uint64_t dis, int n) {
    const uint64_t nm = n >= 64 ? ~0ull : ((1ull << n) - 1);
    const uint64_t d = dis & nm;
    if (!d) return nm;
    const int hb = 64 - __builtin_clzll(d);
    return nm & ~(hb >= 64 ? ~0ull : ((1ull << hb) - 1));
}

// The 2^k codewords of L in run order, for the run kernel (k_terms_runs):
// sorted by value, so consecutive codewords agree on long top bits, and cut
// into runs of pt.  Each run is sorted by its codewords' zeros below the
// run's agreed top bits (then by value); runs in which some codeword has more
// than gl such zeros are "heavy".  Heavy runs come first, then the light ones,
// each part ordered by the run's total zeros, so the runs of one warp have
// about the same number of shrinks at each step.  In the table, blocks of 64
// runs: run r of block b occupies positions b * 64 * pt + r + 64 * i.  Returns
// the first position of the light launch (a whole number of blocks; the block
// that holds the last heavy run goes to the heavy launch).  Needs 2^k to be a
// multiple of 64 * pt.
inline int64_t run_ordered_codewords(const uint64_t* L, int k, int t, int pt, int gl, std::vector<uint64_t>& out) {
    const int64_t chi = (int64_t)1 << k;
    std::vector<uint64_t> cw((size_t)chi);
    uint64_t x = 0;
    cw[0] = 0;
    for (int64_t i = 1; i < chi; i++) {
        x ^= L[k - 1 - __builtin_ctzll((unsigned long long)i)];
        cw[(size_t)i] = x;
    }
    std::sort(cw.begin(), cw.end());
    const uint64_t tm = t >= 64 ? ~0ull : ((1ull << t) - 1);
    const int64_t nruns = chi / pt;
    struct Run {
        int64_t first;
        int maxrem, sumrem;
    };
    std::vector<Run> runs((size_t)nruns);
    for (int64_t r = 0; r < nruns; r++) {
        uint64_t* b = &cw[(size_t)(r * pt)];
        uint64_t am = ~0ull, om = 0ull;
        for (int i = 0; i < pt; i++) {
            am &= b[i];
            om |= b[i];
        }
        const uint64_t low = tm & ~agree_top_host(am ^ om, t);
        std::sort(b, b + pt, [low](uint64_t u, uint64_t v) {
            const int ru = __builtin_popcountll(~u & low), rv = __builtin_popcountll(~v & low);
            return ru != rv ? ru < rv : u < v;
        });
        int mx = 0, sm = 0;
        for (int i = 0; i < pt; i++) {
            const int rem = __builtin_popcountll(~b[i] & low);
            mx = std::max(mx, rem);
            sm += rem;
        }
        runs[(size_t)r] = Run{r * pt, mx, sm};
    }
    std::stable_sort(runs.begin(), runs.end(), [gl](const Run& u, const Run& v) {
        const bool hu = u.maxrem > gl, hv = v.maxrem > gl;
        if (hu != hv) return hu;
        return u.sumrem < v.sumrem;
    });
    int64_t nheavy = 0;
    while (nheavy < nruns && runs[(size_t)nheavy].maxrem > gl) nheavy++;
    out.resize((size_t)chi);
    for (int64_t r = 0; r < nruns; r++) {
        const int64_t blk = r / 64, lane = r % 64;
        for (int i = 0; i < pt; i++)
            out[(size_t)(blk * 64 * pt + lane + 64 * i)] = cw[(size_t)(runs[(size_t)r].first + i)];
    }
    return (nheavy + 63) / 64 * 64 * pt;
}

// z0 + z1 w + z2 w^2 + z3 w^3 (w = e^{i pi/4}) times 2^{-P/2}, P even
inline void zomega_to_complex(const __int128* z, int P, double* re, double* im) {
    const double s = 0.70710678118654752440;
    const double r = (double)z[0] + (double)(z[1] - z[3]) * s;
    const double i = (double)z[2] + (double)(z[1] + z[3]) * s;
    *re = std::ldexp(r, -P / 2);
    *im = std::ldexp(i, -P / 2);
}

// terms per work item of the pair kernel: at most 64 items per theta
inline int64_t chunk_for(int64_t chi) { return std::max<int64_t>(256, (chi + 63) / 64); }

inline double sqrt_half_power(int c) {  // projfactor of innerprod.c:104-111: c successive *= 2^{-1/2}
    double pf = 1;
    const double r = pow(2, -0.5);
    for (int i = 0; i < c; i++) pf *= r;
    return pf;
}

}  // namespace csim_host

// ---------------------------------------------------------------- context
enum BufId {
    kBufA, kBufB, kBufEps, kBufP, kBufM, kBufXi, kBufZeta, kBufAlpha, kBufCode, kBufWords, kBufOffsets,
    kBufCum, kBufCodewords, kBufAcc, kBufAccDiag, kBufPhis, kBufIdx, kBufConsumed, kBufPm, kBufPz, kBufPx,
    kBufL, kBufParts, kBufPartsDiag, kBufCwOrdered, kBufRunScratch, kBufCanon, kBufCodeDirect, kBufCodeRest,
    kBufRestCount, kNumBufs
};

class Engine;                     // csim_engine.cpp: the batched query engine
void engine_free(Engine* engine);  // releases it and its device memory

struct csim_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    int* d_err = nullptr;
    int64_t launches = 0;
    std::string last_error;
    void* buf[kNumBufs + 32] = {};
    size_t cap[kNumBufs + 32] = {};
    csim_host::LibcRand lr;
    uint64_t philox_seed = 0;
    uint64_t philox_next = 0;
    csim_stats stats = {};
    int64_t stats_launch0 = 0;
    int pair_kernel = 0;  // CSIM_OPT_PAIR_KERNEL
    int per_thread = 0;  // CSIM_OPT_PER_THREAD; 0 = auto_per_thread(t)
    cudaEvent_t ev[4] = {};
    // pinned staging of host-made uploads (staged_put): four slots, each with the event of its last copy
    void* pin[4] = {};
    size_t pin_cap[4] = {};
    cudaEvent_t pin_ev[4] = {};
    Engine* engine = nullptr;  // created by the first batched csim_run_queries
    std::vector<uint64_t> cw_key;  // (k, rows of L, t, light bound) of the ordered codeword table in kBufCwOrdered
    int64_t cw_split = 0;          // first index of that table whose codewords have <= the light bound's zeros
    std::vector<int> cw_bounds;        // occupancy-class order: the launches' zero bounds
    std::vector<int64_t> cw_starts;    // and the first index of each class
    // autotuner (CSIM_OPT_AUTOTUNE): the tuned launch parameters live in a
    // process-wide table per device (csim_host.cpp), filled a t bucket at a time
    int direct_slots = 0;  // CSIM_OPT_DIRECT_SLOTS; 0 = direct_slots(t)
    int autotune = 1;
    bool tuning = false;      // a tuning pass is running on this context (its trials use `trial`)
    csim_host::TpTune trial;  // the parameters of the trial in progress
};

namespace csim_host {

// The thread-per-pair launch parameters for t on this context: a fixed
// CSIM_OPT_PER_THREAD wins for the item size; otherwise the tuned values of
// this device, tuning t's bucket first when the context's autotuner is on and
// the bucket has not been tuned in this process (csim_host.cpp).  P, L, k:
// the workload about to run, which the tuning trials then use (a synthetic
// one when P is null).  Returns 0 or an error code.
int tune_for(csim_ctx* ctx, int t, TpTune* out, const csim_projector* P = nullptr, const uint64_t* L = nullptr,
             int k = 0);

inline int fail(csim_ctx* ctx, int code, const char* fmt, ...) {
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

inline int dbuf(csim_ctx* ctx, int id, size_t bytes, void** out) {
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
inline int dput(csim_ctx* ctx, int id, const T* src, size_t count, T** out) {
    void* p;
    CKR(dbuf(ctx, id, count * sizeof(T), &p));
    if (count) CK(cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    ctx->stats.h2d_bytes += (int64_t)(count * sizeof(T));
    *out = (T*)p;
    return 0;
}

// dput through pinned staging slot `slot`: an upload from pageable memory first waits for the
// stream, one from pinned memory returns at once, so the host can prepare the next upload
// while the GPU works.  The slot's previous copy must have run before the slot is rewritten;
// alternating slots makes that wait rare.
template <class T>
inline int staged_put(csim_ctx* ctx, int slot, int id, const T* src, size_t count, T** out) {
    void* p;
    const size_t bytes = count * sizeof(T);
    CKR(dbuf(ctx, id, bytes, &p));
    if (ctx->pin_ev[slot]) CK(cudaEventSynchronize(ctx->pin_ev[slot]));
    else CK(cudaEventCreateWithFlags(&ctx->pin_ev[slot], cudaEventDisableTiming));
    if (ctx->pin_cap[slot] < bytes) {
        if (ctx->pin[slot]) cudaFreeHost(ctx->pin[slot]);
        ctx->pin[slot] = nullptr;
        ctx->pin_cap[slot] = 0;
        const size_t c = bytes + bytes / 4;
        if (cudaMallocHost(&ctx->pin[slot], c) != cudaSuccess) {
            ctx->pin[slot] = nullptr;
            return fail(ctx, CSIM_ERR_NOMEM, "cudaMallocHost of %zu bytes failed", c);
        }
        ctx->pin_cap[slot] = c;
    }
    if (count) {
        memcpy(ctx->pin[slot], src, bytes);
        CK(cudaMemcpyAsync(p, ctx->pin[slot], bytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    CK(cudaEventRecord(ctx->pin_ev[slot], ctx->stream));
    ctx->stats.h2d_bytes += (int64_t)bytes;
    *out = (T*)p;
    return 0;
}

template <class T>
inline int dget(csim_ctx* ctx, T* dst, const T* src, size_t count) {
    if (count) CK(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
    ctx->stats.d2h_bytes += (int64_t)(count * sizeof(T));
    return 0;
}

inline void stats_begin(csim_ctx* ctx) {
    ctx->stats = csim_stats{};
    ctx->stats_launch0 = ctx->launches;
}

// adds the event-timed spans of one batch: ev0..ev3 = start, pair kernel start, pair kernel end, end
inline int stats_batch(csim_ctx* ctx) {
    float a = 0, b = 0;
    CK(cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[3]));
    CK(cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]));
    ctx->stats.device_ms += a;
    ctx->stats.pair_kernel_ms += b;
    return 0;
}

inline void stats_end(csim_ctx* ctx) { ctx->stats.kernels = ctx->launches - ctx->stats_launch0; }

inline csim::Launch launch_of(csim_ctx* ctx) { return csim::Launch{ctx->stream, ctx->d_err, &ctx->launches, ctx->num_sms}; }

// waits for the stream, then turns device error flags into a status
inline int finish(csim_ctx* ctx) {
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

inline int check_states(csim_ctx* ctx, const csim_state* s, int64_t count, int* nr_out, int n_expect = -1) {
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


inline int check_projector(csim_ctx* ctx, const csim_projector* P) {
    if (!P || P->nstabs < 0 || P->nqubits < 0 || P->nqubits > CSIM_MAX_QUBITS)
        return fail(ctx, CSIM_ERR_ARG, "bad projector");
    if (P->nstabs > 0 && (!P->phase || !P->xs || !P->zs)) return fail(ctx, CSIM_ERR_ARG, "bad projector arrays");
    return 0;
}

inline int check_code(csim_ctx* ctx, int t, int exact, const uint64_t* L, int k) {
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

inline double clifford_sum(const csim_projector* P) {  // innerprod.c:52-62
    double sum = 1;
    for (int i = 0; i < P->nstabs; i++) {
        const double ph = (double)phase_m(P->phase[i]);
        if (ph == 0) sum += 1;
        if (ph == 2) sum -= 1;
    }
    return sum;
}

inline int cmp_trunc(const void* a, const void* b) {  // innerprod.c:17-19
    return (int)(*(const double*)a - *(const double*)b);
}

// multiSampledProjector's reduction (innerprod.c:23-41, 75-77): the mean of
// each bin of `samples` values in draw order, then the median of the bin
// means as the C library's qsort orders them with the truncating comparator.
inline double median_of_means(const double* v, int samples, int bins) {
    std::vector<double> binv(bins);
    for (int b = 0; b < bins; b++) {
        double total = 0;
        for (int i = 0; i < samples; i++) total += v[(size_t)b * samples + i];
        binv[b] = total / samples;
    }
    if (bins == 1) return binv[0];
    qsort(binv.data(), (size_t)bins, sizeof(double), cmp_trunc);
    return (bins % 2 == 1) ? binv[(bins - 1) / 2] : (binv[bins / 2] + binv[bins / 2 - 1]) / 2;
}

}  // namespace csim_host
