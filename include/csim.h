/*
 * csim.h — C ABI of libcsimgpu.so, the GB300 backend for CircuitSimulator's
 * stabilizer-rank norm-estimation path.
 *
 * Everything here is plain C: pointers, sizes and int status codes.  All
 * pointer arguments are HOST memory unless the name ends in _dev; the library
 * copies to and from the GPU itself.  Nothing returned is allocated by the
 * library (the reference allocates states in the callee and frees them in the
 * caller, libcirc/stabilizer/stabilizer.c:9-51; here the caller owns every
 * buffer).  Each csim_ctx owns its own CUDA stream, device buffers and random
 * generators, so distinct contexts may be used from distinct threads; one
 * context must not be used by two threads at once.
 *
 * Qubit counts are limited to 1..CSIM_MAX_QUBITS (64): one uint64 per row.
 */
#ifndef CSIM_H
#define CSIM_H

#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CSIM_MAX_QUBITS 64

/* ------------------------------------------------------------------ status */
#define CSIM_OK 0
#define CSIM_ERR_ARG (-1)         /* bad argument (size, range, null)          */
#define CSIM_ERR_CUDA (-2)        /* a CUDA runtime call failed                */
#define CSIM_ERR_DEVICE (-3)      /* a kernel flagged an impossible value      */
#define CSIM_ERR_NOMEM (-4)       /* device or host allocation failed          */
#define CSIM_ERR_NODEVICE (-5)    /* no CUDA device / no sm_103 device         */
#define CSIM_ERR_PROTOCOL (-6)    /* malformed backend stdin input             */

/* ------------------------------------------------------------------ types */

/*
 * One stabilizer state, packed.  Replaces struct StabilizerState
 * (libcirc/stabilizer/stabilizer.h:5-16), whose matrices are byte-packed
 * MSB-first bit arrays (libcirc/utils/matrix.c:330-339).
 *
 * Row r of G, Gbar and J is one uint64 whose bit c is column c.
 * D[a] = 2*(2*bit_a(D2) + bit_a(D1)) in {0,2,4,6} (stabilizer.c:55-62).
 * J[a] bit b set means J_ab = 4.  Only rows/columns < n are meaningful;
 * everything above n must be zero.
 */
typedef struct csim_state {
    int32_t n;         /* number of qubits, 1..64                     */
    int32_t k;         /* dimension of the affine space, 0..n         */
    int32_t Q;         /* constant term of q, in Z8                   */
    int32_t reserved0; /* must be 0                                   */
    uint64_t h;        /* shift vector                                */
    uint64_t D1;       /* low bit of D/2                              */
    uint64_t D2;       /* high bit of D/2                             */
    uint64_t reserved1;
    uint64_t G[CSIM_MAX_QUBITS];
    uint64_t Gbar[CSIM_MAX_QUBITS];
    uint64_t J[CSIM_MAX_QUBITS];
} csim_state;

/*
 * A Pauli projector Π = Π_r (1 + i^{phase_r} Z(zeta_r) X(xi_r))/2, in the
 * stdin-protocol encoding (libcirc/utils/comms.c:9-36): phase_r = v in Z4,
 * xs[r] bit c = x-part on qubit c, zs[r] bit c = z-part.  Replaces struct
 * Projector (libcirc/utils/comms.h:4-11).
 */
typedef struct csim_projector {
    int32_t nstabs;
    int32_t nqubits;
    const int32_t *phase;
    const uint64_t *xs;
    const uint64_t *zs;
} csim_projector;

/* Random-state generators for the samplers. */
#define CSIM_RNG_PHILOX 0 /* counter-based, one independent stream per state (GPU)   */
#define CSIM_RNG_LIBC 1   /* the sequence of srand(seed); rand() of the C library:
                             reproduces the reference's draws sample for sample       */
/* Pass as `seed` to continue the context's current stream instead of reseeding
 * (the reference draws the numerator's and the denominator's samples from one
 * stream, libcirc/probability.c:182-198). */
#define CSIM_SEED_CONTINUE UINT64_MAX

typedef struct csim_ctx csim_ctx;

/* ------------------------------------------------------------- context */

/* Opens a context on CUDA device `device`.  Fails with CSIM_ERR_NODEVICE if the
 * device is not an sm_103 part (the kernels are built for sm_103a only).  A
 * context has its own stream, buffers and generators; use it from one thread
 * at a time (threads that share a GPU open one context each, or share a
 * csim_server, which is safe to call from any thread). */
int csim_ctx_create(int device, csim_ctx **out);
void csim_ctx_destroy(csim_ctx *ctx);
/* Message of the last failing call on this context ("" if none). */
const char *csim_last_error(const csim_ctx *ctx);
/* Number of kernels this context has launched so far. */
int64_t csim_launch_count(const csim_ctx *ctx);

/* Measurements of the last estimator call (csim_single_projector_samples,
 * csim_multi_sampled_projector, csim_exact_projector) on this context.  Device
 * times come from CUDA events recorded on the context's stream. */
typedef struct csim_stats {
    double device_ms;        /* first kernel start .. last kernel end, summed over batches */
    double pair_kernel_ms;   /* the (theta, term) pair kernel alone                        */
    int64_t states;          /* random states drawn                                        */
    int64_t states_live;     /* states not annihilated by the projector                    */
    int64_t pairs;           /* inner products computed (live states x terms)              */
    int64_t h2d_bytes;       /* host -> device bytes copied by the call                    */
    int64_t d2h_bytes;       /* device -> host bytes copied by the call                    */
    int64_t kernels;         /* kernels launched by the call                               */
} csim_stats;
int csim_last_stats(const csim_ctx *ctx, csim_stats *out);

/* Positions the context's counter-based generator: the next state drawn with
 * CSIM_RNG_PHILOX and seed CSIM_SEED_CONTINUE is state `first` of stream
 * `seed`.  Lets ranks draw disjoint blocks of one stream (the reference's
 * MPI split of samples, libcirc/innerprod.c:64-83, without changing the draws). */
int csim_rng_position(csim_ctx *ctx, uint64_t seed, uint64_t first);

/* Tuning options (no counterpart in the reference). */
#define CSIM_OPT_PAIR_KERNEL 1 /* |L>-term pairs: 0 = one thread per pair, the tuner's kernel (default); 1 = one warp
                                  per pair; 2 = one thread per pair, block-shared top-bit shrinks; 3 = one thread per
                                  pair, per-thread runs of codewords with shared top-bit shrinks; 4 = as 2, one
                                  launch per occupancy class of the codewords' zero counts; 5 = one thread per
                                  pair, direct restriction of each state's pivot form */
#define CSIM_OPT_PER_THREAD 2  /* |L>-term pairs per thread per work item of the thread-per-pair kernel (1..64; 0 = by t) */
#define CSIM_OPT_DIRECT_SLOTS 4 /* direct kernel: constraint slots per pair (1..64; 0 = min(t, 8)); states with more
                                   non-pivot coordinates (n - k) go to the block-prefix kernel */
#define CSIM_OPT_AUTOTUNE 3    /* 1 (default): tuned thread-per-pair launches, a t bucket tuned on first use; 0: fixed rules */
int csim_set_option(csim_ctx *ctx, int32_t option, int64_t value);

/* The autotuner of the thread-per-pair launches (no counterpart in the
 * reference).  For the t bucket of t ([4b, 4b+3]) it times the sampler's own
 * launches with each candidate -- the direct kernel or the block-prefix
 * kernel (light launch bound ceil(0.6 t) zeros), each with 16 or 32 terms per
 * thread per work item (items of 1024 or 2048 pairs; 32 pairs per warp per
 * step) -- and keeps the fastest for every t of the bucket, for every context
 * on this device in this process.  The trials run projector P and the k-row code L
 * (the workload about to run; P->nqubits == t) on the tuner's own
 * counter-based states, about 2^25 pairs per trial; with P null they run a
 * synthetic workload (ceil(0.7 t) random Pauli rows, a random min(t, 14)-row
 * code).  A bucket is tuned once; with CSIM_OPT_AUTOTUNE on (the default) the
 * first sampler call or batched query at a new t tunes it on its own
 * workload.  The caller's random streams and last statistics are unchanged.
 * Returns the chosen kernel (0 block-prefix with heavy and light launches,
 * 3 direct restriction; 1 per-thread runs and 2 block-prefix with one launch
 * per occupancy class are not tried, only forced), terms per thread, light
 * bound (t - 33 above 32 qubits for the direct kernel, its narrow/wide split)
 * and the pair-kernel milliseconds of the winning trial.
 * Any output pointer may be NULL. */
int csim_autotune(csim_ctx *ctx, int32_t t, const csim_projector *P, const uint64_t *L, int32_t k,
                  int32_t *kernel, int32_t *per_thread, int32_t *light_zeros, double *pair_ms);

/* ----------------------------------------------- stabilizer primitives (batched) */

/* eps/p/m of <a[i]|b[i]> for i < count; value = eps * 2^{p/2} * e^{i pi m/4}.
 * Replaces innerProductExact, libcirc/stabilizer/stabilizer.c:589-659. */
int csim_inner_product_exact(csim_ctx *ctx, int64_t count, const csim_state *a, const csim_state *b,
                             int32_t *eps, int32_t *p, int32_t *m);

/* Exponential sum of each state's quadratic form; states are updated in place
 * exactly as the reference updates them.
 * Replaces exponentialSumExact, libcirc/stabilizer/stabilizer.c:300-481. */
int csim_exponential_sum_exact(csim_ctx *ctx, int64_t count, csim_state *s, int32_t *eps, int32_t *p,
                               int32_t *m);

/* Intersects state i with {x : xi[i].x = alpha[i]}; status 0 EMPTY, 1 SAME, 2 SUCCESS.
 * Replaces shrink, libcirc/stabilizer/stabilizer.c:500-585. */
int csim_shrink(csim_ctx *ctx, int64_t count, csim_state *s, const uint64_t *xi, const int32_t *alpha,
                int32_t lazy, int32_t *status);

/* Projects state i onto (1 + i^{m[i]} Z(zeta[i]) X(xi[i]))/2; norm[i] in {0, 1, 2^-1/2}.
 * Replaces measurePauli, libcirc/stabilizer/stabilizer.c:827-959. */
int csim_measure_pauli(csim_ctx *ctx, int64_t count, csim_state *s, const int32_t *m, const uint64_t *zeta,
                       const uint64_t *xi, double *norm);

/* Replaces extend, libcirc/stabilizer/stabilizer.c:759-825. */
int csim_extend(csim_ctx *ctx, int64_t count, csim_state *s, const uint64_t *xi);

/* count random n-qubit states from the counter-based generator: state i uses
 * stream (seed, first + i).  Same law as randomStabilizerState,
 * libcirc/stabilizer/stabilizer.c:689-756. */
int csim_random_states(csim_ctx *ctx, int32_t n, int64_t count, uint64_t seed, uint64_t first,
                       csim_state *out);

/* count random n-qubit states built from recorded rand() values: state i
 * consumes words[offsets[i] .. offsets[i+1]) in the order the reference's
 * randomStabilizerState calls rand().  Fails with CSIM_ERR_DEVICE if a state
 * needs more words than its segment holds. */
int csim_random_states_replay(csim_ctx *ctx, int32_t n, int64_t count, const uint32_t *words,
                              const int64_t *offsets, csim_state *out);

/* Term idx[i] of the exact decomposition of |H^{(x)t}>.
 * Replaces prepH, libcirc/stateprep.c:36-81. */
int csim_prep_h(csim_ctx *ctx, int32_t t, int64_t count, const int64_t *idx, csim_state *out);

/* Term idx[i] of |L> for the k x t code L (L[r] = row r).
 * Replaces prepL, libcirc/stateprep.c:85-120. */
int csim_prep_l(csim_ctx *ctx, int32_t t, const uint64_t *L, int32_t k, int64_t count, const int64_t *idx,
                csim_state *out);

/* ------------------------------------------------------------- hot path */

/* All pairs <theta[a] | phi_j> for a < ntheta, j0 <= j < j0 + nj, where phi_j is
 * term j of |L> (exact == 0) or of the exact |H^t> decomposition (exact != 0).
 * Outputs are indexed [a * nj + (j - j0)].  This is the inner loop of
 * singleProjectorSample, libcirc/innerprod.c:122-138. */
int csim_term_products(csim_ctx *ctx, int32_t t, int32_t exact, const uint64_t *L, int32_t k,
                       int64_t ntheta, const csim_state *theta, int64_t j0, int64_t nj, int32_t *eps,
                       int32_t *p, int32_t *m);

/* 2^t |projfactor * sum_j <theta|phi_j>|^2 for `count` random states drawn with
 * generator `rng` (seed `seed`), one value per state in draw order.
 * Replaces singleProjectorSample, libcirc/innerprod.c:88-144. */
int csim_single_projector_samples(csim_ctx *ctx, const csim_projector *P, const uint64_t *L, int32_t k,
                                  int32_t exact, int64_t count, int32_t rng, uint64_t seed, double *values);

/* Median of `bins` means of `samples` samples.  Replaces multiSampledProjector
 * and sampledProjector, libcirc/innerprod.c:23-84; with rng == CSIM_RNG_LIBC
 * the states drawn are the reference's for srand(seed). */
int csim_multi_sampled_projector(csim_ctx *ctx, const csim_projector *P, const uint64_t *L, int32_t k,
                                 int32_t exact, double norm, int32_t samples, int32_t bins, int32_t rng,
                                 uint64_t seed, double *out);

/* The reduction of csim_multi_sampled_projector on `bins` x `samples` values in
 * draw order: per-bin means, then their median as the C library's qsort orders
 * them with the reference's truncating comparator (libcirc/innerprod.c:17-41).
 * Host only; lets ranks that each drew a block of states reduce exactly as one
 * process does. */
int csim_median_of_means(const double *values, int32_t samples, int32_t bins, double *out);

/* |sum_{i<=j} (2 - delta_ij) <Pi phi_i | phi_j>| over all chi(chi+1)/2 pairs.
 * Replaces exactProjector, libcirc/innerprod.c:148-261. */
int csim_exact_projector(csim_ctx *ctx, const csim_projector *P, const uint64_t *L, int32_t k,
                         int32_t exact, double norm, double *out);

/* Rows i0 <= i < i1 of csim_exact_projector: re[i - i0] + i im[i - i0] is row
 * i's contribution, (diag_i + 2 Re sum_{j>i} <Pi phi_i|phi_j>) times the row's
 * projection factor (0 for a row the projector annihilates).  The value of
 * csim_exact_projector is |sum of all chi rows|, summed in row order; ranks that
 * each take a range of rows and send them to one rank reproduce it bit for bit.
 * Splits the l-range of exactProjector's MPI loop (libcirc/innerprod.c:169-195)
 * by rows.  Needs nstabs >= 1 and t >= 1. */
int csim_exact_projector_rows(csim_ctx *ctx, const csim_projector *P, const uint64_t *L, int32_t k,
                              int32_t exact, int64_t i0, int64_t i1, double *re, double *im);

/* ------------------------------------------------------------- many queries */

/* One probability query as the backend process receives it: the 13 scalars of
 * the stdin protocol (libcirc/probability.py:249-268), the projectors G' and H',
 * and the sampler's generator and seed (the reference seeds with getpid(),
 * libcirc/probability.c:182). */
typedef struct csim_query {
    int32_t quiet, verbose, noapprox, samples, bins, t, k, exact;
    double fidbound;
    int32_t fidelity, rank, force_l, force_sample;
    csim_projector G, H;
    int32_t rng; /* CSIM_RNG_LIBC or CSIM_RNG_PHILOX */
    int32_t reserved;
    uint64_t seed;
} csim_query;

typedef struct csim_query_result {
    double numerator, denominator; /* the backend's last two output lines */
    double norm;                   /* decompose()'s norm                  */
    int32_t status;                /* CSIM_OK or this query's error        */
    int32_t exact, k, noapprox;    /* decomposition and estimator used     */
    int64_t pairs;                 /* inner products computed              */
    double latency_s;              /* server: submit -> result; else 0     */
} csim_query_result;

/* Runs nq queries, each exactly as the backend process would (decompose, the
 * noapprox rule, then multiSampledProjector or exactProjector on G' and H';
 * libcirc/probability.c:146-216).  batched == 0: one query after another through
 * the single-query entry points above.  batched == 1: the states, projections and
 * (state, term) pairs of all queries share launches.  Each query draws from its
 * own seed, so both modes give the same results.  Returns the first error;
 * per-query status is in r[i].status. */
int csim_run_queries(csim_ctx *ctx, int64_t nq, const csim_query *q, csim_query_result *r, int32_t batched);

/* The backend as a long-lived process: reads back-to-back stdin-protocol
 * inputs until end of input, runs them on a csim_server as they arrive, and
 * writes "<index> <status> <numerator> <denominator>" per query in input
 * order (%.17e).  Seeds are CSIM_SEED + index (process id + index if unset). */
int csim_backend_serve(FILE *in, FILE *out, int device);

/* ------------------------------------------------------------- serving */

/* A query server on one GPU, replacing one backend process per query
 * (libcirc/probability.py:237-244).  A worker thread runs rounds: each round
 * takes the next states of every admitted query, up to round_pairs inner
 * products, and runs them in shared launches while the host prepares the next
 * round.  Queries submitted while others are on the GPU join the next round
 * once their decomposition fits the device-memory budget; decompositions
 * (codeword tables, term states) stay resident and are shared by queries with
 * the same t and code.  Results are the same as csim_run_queries gives. */
typedef struct csim_server csim_server;

typedef struct csim_server_config {
    int32_t device;
    int32_t per_thread;           /* terms per thread per work item (0: by t)  */
    int64_t hbm_budget_bytes;     /* resident decompositions + round buffers   */
    int64_t round_pairs;          /* inner products per round (0: 2^26)        */
    int64_t round_states;         /* states per round (0: 2^16)                */
} csim_server_config;

typedef struct csim_server_stats {
    int64_t submitted, completed, failed, rounds, pairs;
    int64_t resident_bytes, resident_decompositions, queued;
    double device_ms;             /* event-timed device work of all rounds     */
} csim_server_stats;

#define CSIM_PENDING 1            /* csim_poll: not finished yet               */

int csim_server_create(const csim_server_config *cfg, csim_server **out);
/* Copies the query (projector rows included) and returns its ticket. */
int csim_submit(csim_server *s, const csim_query *q, int64_t *ticket);
/* CSIM_OK with *out filled once the query is done, CSIM_PENDING before that;
 * a finished ticket can be polled again until csim_release. */
int csim_poll(csim_server *s, int64_t ticket, csim_query_result *out);
/* Waits up to timeout_s seconds (< 0: no limit); CSIM_PENDING on timeout. */
int csim_wait(csim_server *s, int64_t ticket, double timeout_s, csim_query_result *out);
/* Frees a finished ticket; CSIM_PENDING while a failed query's states are
 * still in a round on the device. */
int csim_release(csim_server *s, int64_t ticket);
int csim_server_get_stats(csim_server *s, csim_server_stats *out);
/* Stops the worker after the rounds in flight; unfinished queries fail. */
void csim_server_destroy(csim_server *s);

/* The sampler above for terms of |L> (exact == 0) with CSIM_RNG_PHILOX and an
 * explicit seed, for callers that must not allocate device memory: a program
 * whose GPU memory is owned by its own pool allocator or pre-planned to the
 * byte, or a component that has been handed no spare device memory.  It
 * calls no cudaMalloc/cudaFree and needs no csim_ctx; its device scratch is
 * one fixed 2.5 MiB array in the library, held by every GPU that loads it.
 * Same values as csim_single_projector_samples(ctx, P, L, k, 0, count,
 * CSIM_RNG_PHILOX, seed, values).  Limits: 1 <= count <= CSIM_STATIC_MAX_STATES,
 * 0 <= k <= CSIM_STATIC_MAX_K, 1 <= P->nstabs <= 64; larger inputs fail with
 * CSIM_ERR_ARG.  The first call on a device looks the array's device address
 * up (cudaGetSymbolAddress), so make that first call before any stream
 * capture.  Calls share the array: calls that overlap on the GPU (from two
 * threads, or two processes' streams on one device) race and must be
 * serialized by the caller.  Runs on the legacy default stream of `device`;
 * the calling thread's current device is the same after the call as before.
 * No counterpart in the reference. */
#define CSIM_STATIC_MAX_STATES 256
#define CSIM_STATIC_MAX_K 16
int csim_single_projector_samples_static(int32_t device, const csim_projector *P, const uint64_t *L, int32_t k,
                                         int64_t count, uint64_t seed, double *values);

/* ------------------------------------------------------------- host side */

/* Chooses the decomposition: exact |H^t> terms, or a random k x t code L
 * (rows returned in L_out, capacity 64).  *exact and *k are in/out exactly as
 * in decompose, libcirc/probability.c:307-415.  Random bits come from the
 * libc-compatible generator state `*rng_state` (see csim_libc_rand_*), which
 * the reference leaves at its unseeded default (seed 1). */
int csim_decompose(int32_t t, double fidbound, int32_t rank, int32_t fidelity, int32_t force_l,
                   int32_t verbose, int32_t quiet, int32_t *exact, int32_t *k, double *norm, uint64_t *L_out,
                   void *rng_state, FILE *log);

/* csim_decompose with the fidelity sum Z(L) = sum_x 2^(-|x|/2) over the 2^k
 * codewords (probability.c:391-398) taken on ctx's GPU, exactly, where the
 * reference's double loop is exact (k + floor(t/2) <= 53); beyond that the
 * host loop reproduces its rounding.  Same outputs as csim_decompose. */
int csim_decompose_on(csim_ctx *ctx, int32_t t, double fidbound, int32_t rank, int32_t fidelity,
                      int32_t force_l, int32_t verbose, int32_t quiet, int32_t *exact, int32_t *k, double *norm,
                      uint64_t *L_out, void *rng_state, FILE *log);

/* Z(L) of the k-row code L on t qubits, on the GPU.  CSIM_ERR_ARG unless
 * k + floor(t/2) <= 53, where the value equals the reference's double sum. */
int csim_fidelity_sum(csim_ctx *ctx, int32_t t, const uint64_t *L, int32_t k, double *Z_L);

/* The C library's srand()/rand() sequence, reproduced as a value type so that
 * each context owns one.  Use csim_libc_rand_size() bytes of storage. */
int64_t csim_libc_rand_size(void);
void csim_libc_rand_seed(void *state, uint32_t seed);
int32_t csim_libc_rand_next(void *state);

/* The whole backend: reads the stdin protocol of libcirc/probability.py:249-272
 * from `in` and writes the reference's output lines (libcirc/probability.c:44-221)
 * to `out`, the last two being numerator and denominator in %.17e.
 * Returns 0 on success. */
int csim_backend_run(FILE *in, FILE *out, int device);

#ifdef __cplusplus
}
#endif

#endif /* CSIM_H */
