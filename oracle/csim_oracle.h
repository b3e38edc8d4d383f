/*
 * csim_oracle.h — CPU restatement of CircuitSimulator's stabilizer-rank
 * estimator, used ONLY as the checker for the CUDA backend (tests/, the
 * smoke check in __graft_entry__.py and bench.py's CPU-baseline leg).  The
 * product never links or calls it.
 *
 * Parity pinned: tests/test_oracle_golden.py checks it against every fixture
 * of the reference's unit tests (tests/units/tests-c/*.txt, converted into
 * tests/golden/) and against per-pair vectors produced by the reference's own
 * C code compiled from source (oracle/_ref, tests/golden/make_golden.py).
 *
 * States use the packed layout of include/csim.h.
 */
#ifndef CSIM_ORACLE_H
#define CSIM_ORACLE_H

#include <stdint.h>
#include "../include/csim.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Random source: the C library's srand/rand sequence restated, or a replay of
 * recorded words. */
typedef struct orc_rng {
    int32_t kind;            /* 0 = libc sequence, 1 = replay              */
    int32_t idx;             /* position in the libc ring                  */
    uint32_t ring[34];       /* last 34 values of the libc recurrence      */
    const uint32_t *words;   /* replay source                              */
    int64_t pos, end;        /* replay cursor / limit                      */
    int32_t overrun;         /* replay asked past `end`                    */
} orc_rng;

void orc_rng_seed(orc_rng *r, uint32_t seed);
void orc_rng_replay(orc_rng *r, const uint32_t *words, int64_t begin, int64_t end);
int32_t orc_rand(orc_rng *r);

/* stabilizer algebra (libcirc/stabilizer/stabilizer.c) */
void orc_state_init(csim_state *s, int n, int k);
void orc_exponential_sum_exact(csim_state *s, int *eps, int *p, int *m);
int orc_shrink(csim_state *s, uint64_t xi, int alpha, int lazy);
void orc_inner_product_exact(const csim_state *a, const csim_state *b, int *eps, int *p, int *m);
void orc_random_state(int n, orc_rng *r, csim_state *out);
double orc_measure_pauli(csim_state *s, int m, uint64_t zeta, uint64_t xi);
void orc_extend(csim_state *s, uint64_t xi);

/* decomposition terms (libcirc/stateprep.c) */
void orc_prep_h(int64_t i, int t, csim_state *out);
void orc_prep_l(int64_t i, int t, const uint64_t *L, int k, csim_state *out);
uint64_t orc_codeword(int64_t i, const uint64_t *L, int k);

/* estimators (libcirc/innerprod.c) */
double orc_single_projector_sample(const csim_projector *P, const uint64_t *L, int k, int exact, orc_rng *r);
double orc_sampled_projector(const csim_projector *P, const uint64_t *L, int k, int exact, double norm,
                             int samples, orc_rng *r);
double orc_multi_sampled_projector(const csim_projector *P, const uint64_t *L, int k, int exact, double norm,
                                   int samples, int bins, orc_rng *r);
double orc_exact_projector(const csim_projector *P, const uint64_t *L, int k, int exact, double norm);

/* decompose (libcirc/probability.c:307-415) */
void orc_decompose(int t, double fidbound, int rank, int fidelity, int forceL, int *exact, int *k,
                   double *norm, uint64_t *L_out, orc_rng *r);

/* projection of a drawn state: returns projfactor (0 if annihilated) */
double orc_project(csim_state *s, const csim_projector *P);

/* All pairs <theta[a]|phi_j>, a < ntheta, j0 <= j < j0+nj, on `threads` host threads.
 * Outputs indexed [a*nj + (j-j0)]. */
void orc_term_products(int t, int exact, const uint64_t *L, int k, int64_t ntheta, const csim_state *theta,
                       int64_t j0, int64_t nj, int32_t *eps, int32_t *p, int32_t *m, int threads);

/* orc_multi_sampled_projector with the pairs on `threads` host threads; same
 * draws, same term order, same value bit for bit.  values[i] (NULL allowed)
 * receives each state's singleProjectorSample value. */
double orc_multi_sampled_projector_mt(const csim_projector *P, const uint64_t *L, int k, int exact, double norm,
                                      int samples, int bins, orc_rng *r, int threads, double *values);

/* One (theta, term-of-|L>) pair by elementary rank-one updates, with the number
 * of packed 64-bit row operations it takes (the roofline's work unit).  Same
 * (eps, p, m) as orc_inner_product_exact with the prepL term of codeword x. */
void orc_pair_rowops(const csim_state *theta, uint64_t x, int *eps, int *p, int *m, int64_t *ops);

#ifdef __cplusplus
}
#endif

#endif
