/*
 * Flat C entry points over the reference's own stabilizer code, compiled from
 * the reference sources into oracle/_ref/libcsimref.so (see oracle/Makefile).
 *
 * Test infrastructure only.  Python tests and the golden-vector generator call
 * these through ctypes to pin the oracle restatement (oracle/csim_oracle.c)
 * and the CUDA kernels against the reference's actual behaviour:
 *   innerProductExact        libcirc/stabilizer/stabilizer.c:589
 *   exponentialSumExact      libcirc/stabilizer/stabilizer.c:300
 *   shrink                   libcirc/stabilizer/stabilizer.c:500
 *   randomStabilizerState    libcirc/stabilizer/stabilizer.c:689
 *   measurePauli / extend    libcirc/stabilizer/stabilizer.c:827 / :759
 *   prepH / prepL            libcirc/stateprep.c:36 / :85
 *   singleProjectorSample    libcirc/innerprod.c:88
 *   multiSampledProjector    libcirc/innerprod.c:23
 *   exactProjector           libcirc/innerprod.c:148
 *   decompose                libcirc/probability.c:307
 *
 * States cross this boundary in the packed layout of include/csim.h
 * (csim_state: one uint64 per row, bit c = column c).
 *
 * rand()/srand() are interposed here (the library is linked -Bsymbolic so the
 * reference objects bind to these definitions): every value is forwarded from
 * the C library's generator and can optionally be recorded, which lets tests
 * replay the exact random words the reference consumed.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <stdint.h>
#include <string.h>

#include "stabilizer.h"
#include "../include/csim.h"

struct StabilizerState *prepH(int i, int t);
struct StabilizerState *prepL(int i, int t, struct BitMatrix *L);
double singleProjectorSample(struct Projector *P, struct BitMatrix *L, int exact);
double multiSampledProjector(struct Projector *P, struct BitMatrix *L, int exact, double norm,
                             int samples, int bins);
double exactProjector(struct Projector *P, struct BitMatrix *L, int exact, double norm);
void decompose(const int t, struct BitMatrix **L, double *norm, int *exact, int *k,
               const double fidbound, const int rank, const int fidelity, const int forceL,
               const int verbose, const int quiet);

/* ------------------------------------------------------------ rand record */
static int (*real_rand)(void);
static void (*real_srand)(unsigned);
static uint32_t *rec_buf;
static int64_t rec_cap, rec_len;

static void bind_real(void) {
    if (!real_rand) {
        real_rand = (int (*)(void))dlsym(RTLD_NEXT, "rand");
        real_srand = (void (*)(unsigned))dlsym(RTLD_NEXT, "srand");
    }
}

int rand(void) {
    bind_real();
    int v = real_rand();
    if (rec_buf && rec_len < rec_cap) rec_buf[rec_len] = (uint32_t)v;
    if (rec_buf) rec_len++;
    return v;
}

void srand(unsigned s) {
    bind_real();
    real_srand(s);
}

void csimref_srand(unsigned s) { srand(s); }
int csimref_rand(void) { return rand(); }

/* Start recording every rand() value into buf (capacity cap). */
void csimref_record_begin(uint32_t *buf, int64_t cap) {
    rec_buf = buf;
    rec_cap = cap;
    rec_len = 0;
}

/* Stop recording; returns how many values were drawn (may exceed cap). */
int64_t csimref_record_end(void) {
    int64_t n = rec_len;
    rec_buf = NULL;
    rec_cap = 0;
    rec_len = 0;
    return n;
}

/* ------------------------------------------------------------ conversions */
static struct StabilizerState *from_packed(const csim_state *s) {
    struct StabilizerState *st = allocStabilizerState(s->n, s->k);
    st->Q = s->Q;
    BitMatrixSetZero(st->G);
    BitMatrixSetZero(st->Gbar);
    for (int i = 0; i < s->n; i++) {
        BitVectorSet(st->h, i, (unsigned)((s->h >> i) & 1));
        BitVectorSet(st->D1, i, (unsigned)((s->D1 >> i) & 1));
        BitVectorSet(st->D2, i, (unsigned)((s->D2 >> i) & 1));
        for (int j = 0; j < s->n; j++) {
            BitMatrixSet(st->G, i, j, (unsigned)((s->G[i] >> j) & 1));
            BitMatrixSet(st->Gbar, i, j, (unsigned)((s->Gbar[i] >> j) & 1));
            BitMatrixSet(st->J, i, j, (unsigned)((s->J[i] >> j) & 1));
        }
    }
    return st;
}

static void to_packed(const struct StabilizerState *st, csim_state *s) {
    memset(s, 0, sizeof(*s));
    s->n = st->n;
    s->k = st->k;
    s->Q = st->Q;
    for (int i = 0; i < st->n; i++) {
        s->h |= (uint64_t)BitVectorGet(st->h, i) << i;
        s->D1 |= (uint64_t)BitVectorGet(st->D1, i) << i;
        s->D2 |= (uint64_t)BitVectorGet(st->D2, i) << i;
        for (int j = 0; j < st->n; j++) {
            s->G[i] |= (uint64_t)BitMatrixGet(st->G, i, j) << j;
            s->Gbar[i] |= (uint64_t)BitMatrixGet(st->Gbar, i, j) << j;
            s->J[i] |= (uint64_t)BitMatrixGet(st->J, i, j) << j;
        }
    }
}

static struct BitVector *vec_from_word(int n, uint64_t w) {
    struct BitVector *v = newBitVector(n);
    for (int i = 0; i < n; i++) BitVectorSet(v, i, (unsigned)((w >> i) & 1));
    return v;
}

static struct BitMatrix *mat_from_rows(int rows, int cols, const uint64_t *w) {
    struct BitMatrix *m = newBitMatrixZero(rows, cols);
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) BitMatrixSet(m, i, j, (unsigned)((w[i] >> j) & 1));
    return m;
}

static struct Projector *proj_from_packed(int nstabs, int nqubits, const int32_t *phase,
                                          const uint64_t *xs, const uint64_t *zs) {
    struct Projector *P = (struct Projector *)malloc(sizeof(struct Projector));
    P->Nstabs = nstabs;
    P->Nqubits = nqubits;
    if (nstabs == 0) return P;
    P->phaseSign = newBitVector(nstabs);
    P->phaseComplex = newBitVector(nstabs);
    P->xs = newBitMatrixZero(nstabs, nqubits > 0 ? nqubits : 1);
    P->zs = newBitMatrixZero(nstabs, nqubits > 0 ? nqubits : 1);
    for (int i = 0; i < nstabs; i++) {
        /* same phase split as libcirc/utils/comms.c:23-25 */
        BitVectorSet(P->phaseComplex, i, (unsigned)(phase[i] % 2));
        BitVectorSet(P->phaseSign, i, (unsigned)((phase[i] / 2) % 2));
        for (int j = 0; j < nqubits; j++) {
            BitMatrixSet(P->xs, i, j, (unsigned)((xs[i] >> j) & 1));
            BitMatrixSet(P->zs, i, j, (unsigned)((zs[i] >> j) & 1));
        }
    }
    return P;
}

static void proj_free(struct Projector *P) {
    if (P->Nstabs > 0) {
        BitVectorFree(P->phaseSign);
        BitVectorFree(P->phaseComplex);
        BitMatrixFree(P->xs);
        BitMatrixFree(P->zs);
    }
    free(P);
}

/* ------------------------------------------------------------ entry points */
void csimref_inner_product_exact(const csim_state *a, const csim_state *b, int *eps, int *p, int *m) {
    struct StabilizerState *s1 = from_packed(a), *s2 = from_packed(b);
    *eps = 0; *p = 0; *m = 0;
    innerProductExact(s1, s2, eps, p, m);
    freeStabilizerState(s1);
    freeStabilizerState(s2);
}

void csimref_exponential_sum_exact(csim_state *a, int *eps, int *p, int *m) {
    struct StabilizerState *s = from_packed(a);
    *eps = 0; *p = 0; *m = 0;
    exponentialSumExact(s, eps, p, m);
    to_packed(s, a);
    freeStabilizerState(s);
}

int csimref_shrink(csim_state *a, uint64_t xi, int alpha, int lazy) {
    struct StabilizerState *s = from_packed(a);
    struct BitVector *v = vec_from_word(a->n, xi);
    int r = shrink(s, v, alpha, lazy);
    to_packed(s, a);
    BitVectorFree(v);
    freeStabilizerState(s);
    return r;
}

double csimref_measure_pauli(csim_state *a, int m, uint64_t zeta, uint64_t xi) {
    struct StabilizerState *s = from_packed(a);
    struct BitVector *z = vec_from_word(a->n, zeta), *x = vec_from_word(a->n, xi);
    double r = measurePauli(s, m, z, x);
    to_packed(s, a);
    BitVectorFree(z);
    BitVectorFree(x);
    freeStabilizerState(s);
    return r;
}

void csimref_extend(csim_state *a, uint64_t xi) {
    struct StabilizerState *s = from_packed(a);
    struct BitVector *x = vec_from_word(a->n, xi);
    extend(s, x);
    to_packed(s, a);
    BitVectorFree(x);
    freeStabilizerState(s);
}

/* Draws one state from the C library's current rand() stream. */
void csimref_random_state(int n, csim_state *out) {
    struct StabilizerState *s = randomStabilizerState(n);
    to_packed(s, out);
    freeStabilizerState(s);
}

void csimref_prep_h(int i, int t, csim_state *out) {
    struct StabilizerState *s = prepH(i, t);
    to_packed(s, out);
    freeStabilizerState(s);
}

void csimref_prep_l(int i, int t, const uint64_t *L, int k, csim_state *out) {
    struct BitMatrix *Lm = mat_from_rows(k, t, L);
    struct StabilizerState *s = prepL(i, t, Lm);
    to_packed(s, out);
    freeStabilizerState(s);
    BitMatrixFree(Lm);
}

double csimref_single_projector_sample(int nstabs, int nqubits, const int32_t *phase, const uint64_t *xs,
                                       const uint64_t *zs, const uint64_t *L, int k, int exact) {
    struct Projector *P = proj_from_packed(nstabs, nqubits, phase, xs, zs);
    struct BitMatrix *Lm = exact ? NULL : mat_from_rows(k, nqubits, L);
    double r = singleProjectorSample(P, Lm, exact);
    if (Lm) BitMatrixFree(Lm);
    proj_free(P);
    return r;
}

double csimref_multi_sampled_projector(int nstabs, int nqubits, const int32_t *phase, const uint64_t *xs,
                                       const uint64_t *zs, const uint64_t *L, int k, int exact, double norm,
                                       int samples, int bins) {
    struct Projector *P = proj_from_packed(nstabs, nqubits, phase, xs, zs);
    struct BitMatrix *Lm = (exact || nqubits == 0) ? NULL : mat_from_rows(k, nqubits, L);
    double r = multiSampledProjector(P, Lm, exact, norm, samples, bins);
    if (Lm) BitMatrixFree(Lm);
    proj_free(P);
    return r;
}

double csimref_exact_projector(int nstabs, int nqubits, const int32_t *phase, const uint64_t *xs,
                               const uint64_t *zs, const uint64_t *L, int k, int exact, double norm) {
    struct Projector *P = proj_from_packed(nstabs, nqubits, phase, xs, zs);
    struct BitMatrix *Lm = (exact || nqubits == 0) ? NULL : mat_from_rows(k, nqubits, L);
    double r = exactProjector(P, Lm, exact, norm);
    if (Lm) BitMatrixFree(Lm);
    proj_free(P);
    return r;
}

/* decompose(); L rows are returned packed in L_out (capacity 64 rows). */
void csimref_decompose(int t, double fidbound, int rank, int fidelity, int forceL, int *exact, int *k,
                       double *norm, uint64_t *L_out) {
    struct BitMatrix *L = NULL;
    decompose(t, &L, norm, exact, k, fidbound, rank, fidelity, forceL, 0, 1);
    if (!*exact && L) {
        for (int i = 0; i < *k; i++) {
            uint64_t w = 0;
            for (int j = 0; j < t; j++) w |= (uint64_t)BitMatrixGet(L, i, j) << j;
            L_out[i] = w;
        }
        BitMatrixFree(L);
    }
}
