/*
 * csim_oracle.c — CPU restatement of CircuitSimulator's stabilizer-rank
 * estimator (libcirc/stabilizer/stabilizer.c, libcirc/stateprep.c,
 * libcirc/innerprod.c, decompose() of libcirc/probability.c).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the CUDA backend is
 * compared with; it is never linked into libcsimgpu.so or gpubackend.
 *
 * It follows the reference algorithm step by step — the same basis changes
 * in the same order, the dense R J R^T update of updateDJ, the same integer
 * quirks — so that its (eps, p, m) triples, states and probabilities are the
 * reference's own.  Only the storage differs: one uint64 per matrix row
 * (bit c = column c) instead of byte-packed MSB-first bit arrays
 * (libcirc/utils/matrix.c:124-146).  Parity is pinned against the reference's
 * unit-test fixtures and against the reference compiled from source
 * (tests/test_oracle_golden.py).
 */
#include "csim_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define BIT(w, i) ((int)(((w) >> (i)) & 1u))
#define ONE(i) (1ULL << (i))

static inline int popc(uint64_t x) { return __builtin_popcountll(x); }
static inline int par(uint64_t x) { return __builtin_popcountll(x) & 1; }

/* ======================================================================
 * Random source.
 * The C library's rand() after srand(seed) is the additive lagged-Fibonacci
 * generator r_i = r_{i-3} + r_{i-31} (mod 2^32) whose first 31 words come from
 * the Park–Miller recurrence r_i = 16807 r_{i-1} mod (2^31-1) (Schrage's
 * method), r_31..r_33 repeat r_0..r_2, the first 310 outputs are discarded,
 * and each output is r_i >> 1 (P. Selinger, "The GLIBC pseudo-random number
 * generator").  The reference draws every random bit through rand()
 * (libcirc/utils/matrix.c:85-92, libcirc/stabilizer/stabilizer.c:669-674,750).
 * ==================================================================== */
static uint32_t rng_step(orc_rng *r) {
    int i = r->idx;
    uint32_t v = r->ring[(i + 31) % 34] + r->ring[(i + 3) % 34];
    r->ring[i] = v;
    r->idx = (i + 1) % 34;
    return v;
}

void orc_rng_seed(orc_rng *r, uint32_t seed) {
    memset(r, 0, sizeof(*r));
    int32_t word = (int32_t)(seed == 0 ? 1u : seed);
    int32_t v[34];
    v[0] = word;
    for (int i = 1; i < 31; i++) {
        int64_t hi = word / 127773, lo = word % 127773;
        word = (int32_t)(16807 * lo - 2836 * hi);
        if (word < 0) word += 2147483647;
        v[i] = word;
    }
    for (int i = 31; i < 34; i++) v[i] = v[i - 31];
    for (int i = 0; i < 34; i++) r->ring[i] = (uint32_t)v[i];
    r->idx = 0;
    for (int i = 34; i < 344; i++) rng_step(r);
}

void orc_rng_replay(orc_rng *r, const uint32_t *words, int64_t begin, int64_t end) {
    memset(r, 0, sizeof(*r));
    r->kind = 1;
    r->words = words;
    r->pos = begin;
    r->end = end;
}

int32_t orc_rand(orc_rng *r) {
    if (r->kind == 1) {
        if (r->pos >= r->end) {
            r->overrun = 1;
            return 0;
        }
        return (int32_t)r->words[r->pos++];
    }
    return (int32_t)(rng_step(r) >> 1);
}

/* random bit vector from ceil(n/8) bytes, MSB of byte b = bit 8b
 * (BitVectorSetRandom, libcirc/utils/matrix.c:85-92; BitVectorGet :124-131) */
static uint64_t random_bits(int n, orc_rng *r) {
    uint64_t w = 0;
    int bytes = (n + 7) / 8;
    for (int b = 0; b < bytes; b++) {
        int byte = orc_rand(r) % 256;
        for (int j = 0; j < 8; j++) {
            int loc = 8 * b + j;
            if (loc < n && (byte & (0x80 >> j))) w |= ONE(loc);
        }
    }
    return w;
}

/* ======================================================================
 * State helpers (stabilizer.c:9-62)
 * ==================================================================== */
void orc_state_init(csim_state *s, int n, int k) {
    memset(s, 0, sizeof(*s));
    s->n = n;
    s->k = k;
    for (int i = 0; i < n; i++) {
        s->G[i] = ONE(i);
        s->Gbar[i] = ONE(i);
    }
}

static inline int getD(const csim_state *s, int i) { return 2 * (2 * BIT(s->D2, i) + BIT(s->D1, i)); }

/* setD stores (val/2) mod 4 as two bits, C truncating division (stabilizer.c:59-62) */
static inline void setD(csim_state *s, int i, int val) {
    int v2 = val / 2;
    int d1 = (v2 % 2) & 1;
    int d2 = (((v2 - v2 % 2) / 2) % 2) & 1;
    s->D1 = (s->D1 & ~ONE(i)) | ((uint64_t)d1 << i);
    s->D2 = (s->D2 & ~ONE(i)) | ((uint64_t)d2 << i);
}

static void identity(uint64_t *R, int n) {
    for (int i = 0; i < n; i++) R[i] = ONE(i);
}

/* updateDJ, stabilizer.c:129-160: D <- R D (+4 for odd lower-triangle
 * R J R^T diagonal terms), J <- R J R^T, all n x n, dense. */
static void updateDJ(csim_state *s, const uint64_t *R) {
    const int n = s->n, k = s->k;
    int Dnew[CSIM_MAX_QUBITS];
    for (int i = 0; i < n; i++) {
        int acc = 0;
        for (int j = 0; j < k; j++) acc += getD(s, j) * BIT(R[i], j);
        Dnew[i] = acc;
    }
    for (int i = 0; i < n; i++) setD(s, i, Dnew[i]);

    for (int a = 0; a < n; a++) {
        const uint64_t r = R[a];
        int val = 0;
        for (int b = 0; b < n; b++)
            if (BIT(r, b)) val += popc(s->J[b] & r & (ONE(b) - 1));
        if (val % 2 == 1) s->D2 ^= ONE(a);
    }

    uint64_t RJ[CSIM_MAX_QUBITS], Jn[CSIM_MAX_QUBITS];
    for (int x = 0; x < n; x++) {
        uint64_t acc = 0;
        for (int b = 0; b < n; b++)
            if (BIT(R[x], b)) acc ^= s->J[b];
        RJ[x] = acc;
    }
    for (int x = 0; x < n; x++) {
        uint64_t w = 0;
        for (int y = 0; y < n; y++)
            if (par(RJ[x] & R[y])) w |= ONE(y);
        Jn[x] = w;
    }
    memcpy(s->J, Jn, sizeof(uint64_t) * (size_t)n);
}

/* updateQD, stabilizer.c:163-177 */
static void updateQD(csim_state *s, uint64_t y) {
    const int k = s->k;
    for (int a = 0; a < k; a++) {
        s->Q += getD(s, a) * BIT(y, a);
        for (int b = a + 1; b < k; b++) s->Q += 4 * BIT(s->J[a], b) * BIT(y, a) * BIT(y, b);
    }
    s->Q = s->Q % 8;
    uint64_t t = 0;
    for (int x = 0; x < s->n; x++)
        if (par(s->J[x] & y)) t |= ONE(x);
    s->D2 ^= t;
}

/* ======================================================================
 * Exponential sum (stabilizer.c:183-481)
 * ==================================================================== */
int orc_assert_failures = 0;

/* 1 + e^{i pi A/4} + e^{i pi B/4} - e^{i pi (A+B)/4} for even A, B (:183-225) */
static void gamma_ab(int *eps, int *p, int *m, int A, int B) {
    static const int lre[4] = {1, 0, -1, 0}, lim[4] = {0, 1, 0, -1};
    if (A % 2 != 0 || B % 2 != 0) orc_assert_failures++;
    int gr = 1 + lre[(A % 8) / 2] + lre[(B % 8) / 2] - lre[((A + B) % 8) / 2];
    int gi = lim[(A % 8) / 2] + lim[(B % 8) / 2] - lim[((A + B) % 8) / 2];
    if (gr == 0 && gi == 0) {
        *eps = 0;
        *p = 0;
        *m = 0;
        return;
    }
    *eps = 1;
    *p = 2;
    if (gr == 0) {
        *m = gi > 0 ? 2 : 6;
    } else if (gr == -2) {
        *m = 4;
    } else {
        if (gi == 2) *m = 1;
        if (gi == 0) *m = 0;
        if (gi == -2) *m = 7;
    }
}

/* 1 + e^{i pi A/4} (:228-255) */
static void partial_gamma(int *eps, int *p, int *m, int A) {
    while (A < 0) A += 8;
    if (A % 2 != 0) orc_assert_failures++;
    *eps = (A % 8 == 4) ? 0 : 1;
    switch (A % 8) {
    case 0: *p = 2; *m = 0; break;
    case 2: *p = 1; *m = 1; break;
    case 4: *p = 0; *m = 0; break;
    case 6: *p = 1; *m = 7; break;
    default: break;
    }
}

/* W_sigma (:258-297) */
static void wsigma(const csim_state *s, int *eps, int *p, int *m, int sigma, int sidx, const int *M, int Ml,
                   const int *Dm, int Dl) {
    if (s->k == 0) {
        *eps = 1;
        *p = 0;
        *m = s->Q;
        return;
    }
    int tEps = 1, tP = 0, tM = s->Q + sigma * getD(s, sidx);
    for (int i = 0; i < Ml; i++) {
        partial_gamma(eps, p, m, getD(s, M[i]) + sigma * (4 * BIT(s->J[M[i]], sidx)));
        if (*eps == 0) {
            *p = 0;
            *m = 0;
            return;
        }
        tEps = 1;
        tP += *p;
        tM = (tM + *m) % 8;
    }
    for (int i = 0; i < Dl; i++) {
        const int a = Dm[2 * i], b = Dm[2 * i + 1];
        gamma_ab(eps, p, m, getD(s, a) + sigma * 4 * BIT(s->J[a], sidx), getD(s, b) + sigma * 4 * BIT(s->J[b], sidx));
        if (*eps == 0) {
            *p = 0;
            *m = 0;
            return;
        }
        tEps = 1;
        tP += *p;
        tM = (tM + *m) % 8;
    }
    *eps = tEps;
    *p = tP;
    *m = tM;
}

void orc_exponential_sum_exact(csim_state *s, int *eps, int *p, int *m) {
    const int n = s->n, k = s->k;
    int S[CSIM_MAX_QUBITS], Sl = 0;
    for (int a = 0; a < k; a++) {
        int d = getD(s, a);
        if (d == 2 || d == 6) S[Sl++] = a;
    }
    uint64_t R[CSIM_MAX_QUBITS];
    if (Sl > 0) {
        const int a = S[0];
        identity(R, n);
        for (int i = 1; i < Sl; i++) R[S[i]] ^= ONE(a);
        updateDJ(s, R);
        identity(R, n); /* identity with columns a and k-1 swapped */
        if (a != k - 1) {
            R[a] = ONE(k - 1);
            R[k - 1] = ONE(a);
        }
        updateDJ(s, R);
        S[0] = k - 1;
        Sl = 1;
    }

    int E[CSIM_MAX_QUBITS], El = 0;
    for (int x = 0; x < k; x++)
        if (Sl == 0 || x != S[0]) E[El++] = x;

    int M[CSIM_MAX_QUBITS], Ml = 0, Dm[2 * CSIM_MAX_QUBITS], Dl = 0;
    while (El > 0) {
        const int a = E[0];
        int b = -1;
        for (int i = 1; i < El; i++)
            if (BIT(s->J[a], E[i])) {
                b = E[i];
                break;
            }
        if (b < 0) { /* monomer {a} */
            M[Ml++] = a;
            for (int i = 0; i < El - 1; i++) E[i] = E[i + 1];
            El--;
        } else { /* dimer {a, b}: basis change clearing J[a,.] and J[b,.] on the rest of E */
            identity(R, n);
            for (int i = 0; i < El; i++) {
                const int e = E[i];
                if (e != a && e != b) {
                    if (BIT(s->J[a], e)) R[e] ^= ONE(b);
                    if (BIT(s->J[b], e)) R[e] ^= ONE(a);
                }
            }
            updateDJ(s, R);
            Dm[2 * Dl] = a;
            Dm[2 * Dl + 1] = b;
            Dl++;
            int w = 0;
            for (int i = 0; i < El; i++)
                if (E[i] != a && E[i] != b) E[w++] = E[i];
            El = w;
        }
    }

    if (Sl == 0) {
        wsigma(s, eps, p, m, 0, 0, M, Ml, Dm, Dl);
        return;
    }
    int e0, p0, m0, e1, p1, m1;
    wsigma(s, &e0, &p0, &m0, 0, S[0], M, Ml, Dm, Dl);
    wsigma(s, &e1, &p1, &m1, 1, S[0], M, Ml, Dm, Dl);
    if (e0 == 0) {
        *eps = e1;
        *p = p1;
        *m = m1;
        return;
    }
    if (e1 == 0) {
        *eps = e0;
        *p = p0;
        *m = m0;
        return;
    }
    if (p0 != p1) { /* the reference prints an error and returns without writing (:457-460) */
        orc_assert_failures++;
        return;
    }
    if ((m1 - m0) % 2 == 1) {
        orc_assert_failures++;
        return;
    }
    partial_gamma(eps, p, m, m1 - m0);
    if (*eps == 0) {
        *p = 0;
        *m = 0;
    } else {
        *p += p0;
        *m = *m + m0 % 8; /* not reduced mod 8 (:477) */
    }
}

/* ======================================================================
 * shrink (stabilizer.c:500-585)
 * ==================================================================== */
int orc_shrink(csim_state *s, uint64_t xi, int alpha, int lazy) {
    const int n = s->n, k = s->k;
    int S[CSIM_MAX_QUBITS], Sl = 0;
    for (int a = 0; a < k; a++)
        if (par(s->G[a] & xi)) S[Sl++] = a;
    const int beta = (alpha + popc(xi & s->h)) % 2;
    if (Sl == 0) return 1 - beta;

    const int i = S[--Sl];
    uint64_t gbar_i = s->Gbar[i];
    uint64_t R[CSIM_MAX_QUBITS];
    for (int t = 0; t < Sl; t++) {
        const int a = S[t];
        s->G[a] ^= s->G[i];
        if (lazy != 1) {
            identity(R, n);
            R[a] |= ONE(i);
            updateDJ(s, R);
        }
        gbar_i ^= s->Gbar[a];
    }
    s->Gbar[i] = gbar_i;

    uint64_t tmp = s->G[i];
    s->G[i] = s->G[k - 1];
    s->G[k - 1] = tmp;
    tmp = s->Gbar[i];
    s->Gbar[i] = s->Gbar[k - 1];
    s->Gbar[k - 1] = tmp;
    if (lazy != 1) {
        identity(R, n);
        R[i] = ONE(k - 1);
        R[k - 1] = ONE(i);
        if (i == k - 1) R[i] = ONE(i);
        updateDJ(s, R);
    }
    if (beta == 1) s->h ^= s->G[k - 1];
    if (lazy != 1) updateQD(s, (uint64_t)beta << (k - 1));
    s->k--;
    return 2;
}

/* ======================================================================
 * innerProductExact (stabilizer.c:589-659)
 * ==================================================================== */
void orc_inner_product_exact(const csim_state *s1, const csim_state *s2, int *eps, int *p, int *m) {
    csim_state st = *s1;
    const int n = s2->n;
    for (int b = s2->k; b < n; b++) {
        const uint64_t v = s2->Gbar[b];
        const int alpha = popc(s2->h & v) % 2;
        *eps = orc_shrink(&st, v, alpha, 0);
        if (*eps == 0) {
            *p = 0;
            *m = 0;
            return;
        }
    }
    uint64_t R[CSIM_MAX_QUBITS];
    memset(R, 0, sizeof(R));
    const uint64_t hh = st.h ^ s2->h;
    uint64_t y = 0;
    for (int a = 0; a < n; a++) {
        const uint64_t g2 = s2->Gbar[a];
        if (par(hh & g2)) y |= ONE(a);
        for (int b = 0; b < n; b++)
            if (par(st.G[b] & g2)) R[b] |= ONE(a);
    }
    csim_state t2 = *s2;
    updateQD(&t2, y);
    updateDJ(&t2, R);
    st.Q -= t2.Q;
    if (st.Q < 0) st.Q += 8;
    for (int i = 0; i < st.n; i++) {
        int val = getD(&st, i) - getD(&t2, i);
        if (val < 0) val += 8;
        setD(&st, i, val);
    }
    for (int i = 0; i < n; i++) st.J[i] ^= t2.J[i];
    orc_exponential_sum_exact(&st, eps, p, m);
    *p -= s1->k + s2->k;
}

/* ======================================================================
 * randomStabilizerState (stabilizer.c:669-756)
 * ==================================================================== */
static double logeta(int d, int n) {
    if (d == 0) return 0.;
    double product = 0;
    for (int a = 1; a <= d; a++) {
        product += log2(1 - pow(2, d - n - a));
        product -= log2(1 - pow(2, -a));
    }
    return (-d * (d + 1) / 2) + product;
}

static double rand_unit(orc_rng *r) {
    double range = 1.0;
    double div = 2147483647 / range;
    return 0. + (orc_rand(r) / div);
}

void orc_random_state(int n, orc_rng *r, csim_state *out) {
    double dist[CSIM_MAX_QUBITS + 1], cum[CSIM_MAX_QUBITS + 1];
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

    double sample = rand_unit(r);
    while (sample == 0.) sample = rand_unit(r);
    int d;
    for (d = 0; d <= n; d++)
        if (sample <= cum[d]) break;
    const int k = n - d;

    orc_state_init(out, n, n);
    while (out->k > k) orc_shrink(out, random_bits(n, r), 0, 1);
    out->h = random_bits(n, r);
    out->D1 = random_bits(n, r);
    out->D2 = random_bits(n, r);
    for (int i = 0; i < k; i++) {
        if (((getD(out, i) * 2) % 8) / 4) out->J[i] |= ONE(i);
        for (int j = 0; j < i; j++) {
            const int val = orc_rand(r);
            if (val & 1) {
                out->J[i] |= ONE(j);
                out->J[j] |= ONE(i);
            }
        }
    }
}

/* ======================================================================
 * extend / measurePauli (stabilizer.c:759-959)
 * ==================================================================== */
void orc_extend(csim_state *s, uint64_t xi) {
    const int n = s->n, k = s->k;
    int S[CSIM_MAX_QUBITS], Sl = 0;
    for (int a = 0; a < n; a++)
        if (par(xi & s->Gbar[a])) S[Sl++] = a;
    int i = -1;
    for (int t = 0; t < Sl; t++)
        if (k <= S[t] && k < n) {
            i = S[t];
            break;
        }
    if (i < 0) return;
    const uint64_t gbar_i = s->Gbar[i];
    uint64_t g_i = s->G[i];
    for (int t = 0; t < Sl; t++) {
        const int a = S[t];
        if (a == i) continue;
        s->Gbar[a] ^= gbar_i;
        g_i ^= s->G[a];
    }
    s->G[i] = g_i;
    uint64_t tmp = s->G[i];
    s->G[i] = s->G[k];
    s->G[k] = tmp;
    tmp = s->Gbar[i];
    s->Gbar[i] = s->Gbar[k];
    s->Gbar[k] = tmp;
    s->k++;
}

double orc_measure_pauli(csim_state *s, int m, uint64_t zeta, uint64_t xi) {
    const int n = s->n, k = s->k;
    uint64_t vXi = 0, vZeta = 0, xiP = 0;
    for (int a = 0; a < k; a++) {
        if (par(s->Gbar[a] & xi)) vXi |= ONE(a);
        if (par(s->G[a] & zeta)) vZeta |= ONE(a);
    }
    for (int a = 0; a < k; a++)
        if (BIT(vXi, a)) xiP ^= s->G[a];

    int w = 2 * m;
    w += 4 * (popc(zeta & s->h) % 2);
    for (int b = 0; b < k; b++) w += getD(s, b) * BIT(vXi, b);
    for (int b = 0; b < k; b++)
        for (int a = 0; a < b; a++) w += 4 * BIT(s->J[a], b) * BIT(vXi, a) * BIT(vXi, b);
    w = w % 8;

    uint64_t eta = 0;
    for (int x = 0; x < n; x++)
        if (par(s->J[x] & vXi)) eta |= ONE(x);
    eta ^= vZeta;

    if (xi == xiP) {
        if (w == 0 || w == 4) {
            uint64_t gam = 0;
            for (int a = 0; a < k; a++)
                if (BIT(eta, a)) gam ^= s->Gbar[a];
            const int alpha = (w / 4 + popc(gam & s->h)) % 2;
            switch (orc_shrink(s, gam, alpha, 0)) {
            case 0: return 0;
            case 1: return 1;
            default: return pow(2, -0.5);
            }
        } else if (w == 2 || w == 6) {
            const int sigma = 2 - w / 2;
            s->Q = (s->Q + sigma) % 8;
            while (s->Q < 0) s->Q += 8;
            for (int a = 0; a < k; a++) {
                int val = getD(s, a) - 2 * sigma * BIT(eta, a);
                while (val < 0) val += 8;
                setD(s, a, val);
            }
            for (int i = 0; i < n; i++)
                if (BIT(eta, i)) s->J[i] ^= eta;
            return pow(2, -0.5);
        }
    }
    orc_extend(s, xi);
    const int newD = 2 * m + 4 * (popc(zeta & xi) % 2) + 4 * (popc(zeta & s->h) % 2);
    const int kk = s->k - 1;
    setD(s, kk, newD);
    s->J[kk] = vZeta;
    for (int x = 0; x < n; x++) s->J[x] = (s->J[x] & ~ONE(kk)) | ((uint64_t)BIT(vZeta, x) << kk);
    if (m % 2 == 1 || m % 2 == -1) s->J[kk] |= ONE(kk);
    else s->J[kk] &= ~ONE(kk);
    return pow(2, -0.5);
}

/* ======================================================================
 * decomposition terms (stateprep.c)
 * ==================================================================== */
/* binrep(i, sz): character j is bit (sz-1-j) of i (stateprep.c:5-32) */
void orc_prep_h(int64_t i, int t, csim_state *out) {
    const int size = (int)ceil((double)t / 2);
    orc_state_init(out, t, t);
    for (int j = 0; j < size; j++) {
        const int bit = (int)((i >> (size - 1 - j)) & 1);
        if (bit == 0 && !(t % 2 && j == size - 1)) {
            out->J[2 * j + 1] |= ONE(2 * j);
            out->J[2 * j] |= ONE(2 * j + 1);
        }
    }
    for (int j = 0; j < size; j++) {
        const int bit = (int)((i >> (size - 1 - j)) & 1);
        if (t % 2 && j == size - 1) {
            if (bit == 1) orc_shrink(out, ONE(t - 1), 0, 0);
            continue;
        }
        if (bit == 1) orc_shrink(out, ONE(2 * j + 1) | ONE(2 * j), 0, 0);
    }
}

uint64_t orc_codeword(int64_t i, const uint64_t *L, int k) {
    uint64_t x = 0;
    for (int j = 0; j < k; j++)
        if ((i >> (k - 1 - j)) & 1) x ^= L[j];
    return x;
}

void orc_prep_l(int64_t i, int t, const uint64_t *L, int k, csim_state *out) {
    const uint64_t x = orc_codeword(i, L, k);
    orc_state_init(out, t, t);
    for (int idx = 0; idx < t; idx++)
        if (!BIT(x, idx)) orc_shrink(out, ONE(idx), 0, 0);
}

/* ======================================================================
 * estimators (innerprod.c)
 * ==================================================================== */
static int phase_m(int v) { return 2 * (((v / 2) % 2) & 1) + ((v % 2) & 1); }

double orc_project(csim_state *s, const csim_projector *P) {
    double projfactor = 1;
    for (int i = 0; i < P->nstabs; i++) {
        const double res = orc_measure_pauli(s, phase_m(P->phase[i]), P->zs[i], P->xs[i]);
        projfactor *= res;
        if (res == 0) return 0;
    }
    return projfactor;
}

/* evalW + ComplexAdd (stabilizer.c:484-488, matrix.c:15-37) */
static void add_w(double *re, double *im, int eps, int p, int m) {
    const double th = 3.14159265358979323846 * (double)m / 4.;
    const double r = eps * pow(2., (double)p / 2.);
    const double zr = (1 * cos(th)) * r, zi = (1 * sin(th)) * r;
    *re += zr;
    *im += zi;
}

static void prep_term(int exact, int64_t j, int t, const uint64_t *L, int k, csim_state *out) {
    if (exact) orc_prep_h(j, t, out);
    else orc_prep_l(j, t, L, k, out);
}

double orc_single_projector_sample(const csim_projector *P, const uint64_t *L, int k, int exact, orc_rng *r) {
    const int t = P->nqubits;
    csim_state th, phi;
    orc_random_state(t, r, &th);
    const double projfactor = orc_project(&th, P);
    if (projfactor == 0) return 0;
    double tr = 0, ti = 0;
    const int size = exact ? (int)pow(2, ceil((double)t / 2)) : (int)pow(2, k);
    for (int i = 0; i < size; i++) {
        int eps = 0, p = 0, m = 0;
        prep_term(exact, i, t, L, k, &phi);
        orc_inner_product_exact(&th, &phi, &eps, &p, &m);
        add_w(&tr, &ti, eps, p, m);
    }
    const double a = tr * projfactor, b = ti * projfactor;
    return pow(2, t) * (a * a + b * b);
}

static double clifford_sum(const csim_projector *P) {
    double sum = 1;
    for (int i = 0; i < P->nstabs; i++) {
        const double ph = (double)phase_m(P->phase[i]);
        if (ph == 0) sum += 1;
        if (ph == 2) sum -= 1;
    }
    return sum;
}

double orc_sampled_projector(const csim_projector *P, const uint64_t *L, int k, int exact, double norm,
                             int samples, orc_rng *r) {
    if (P->nstabs == 0) return pow(norm, 2);
    if (P->nqubits == 0) return pow(norm, 2) * clifford_sum(P) / (1 + (double)P->nstabs);
    double total = 0;
    for (int i = 0; i < samples; i++) total += orc_single_projector_sample(P, L, k, exact, r);
    return total / samples;
}

/* the reference's comparator converts the difference to int (innerprod.c:17-19) */
static int cmp_trunc(const void *a, const void *b) { return (int)(*(const double *)a - *(const double *)b); }

double orc_multi_sampled_projector(const csim_projector *P, const uint64_t *L, int k, int exact, double norm,
                                   int samples, int bins, orc_rng *r) {
    if (bins == 1) return orc_sampled_projector(P, L, k, exact, norm, samples, r);
    double *v = (double *)malloc(sizeof(double) * (size_t)bins);
    for (int i = 0; i < bins; i++) v[i] = orc_sampled_projector(P, L, k, exact, norm, samples, r);
    qsort(v, (size_t)bins, sizeof(double), cmp_trunc);
    double out = (bins % 2 == 1) ? v[(bins - 1) / 2] : (v[bins / 2] + v[bins / 2 - 1]) / 2;
    free(v);
    return out;
}

/* exactProjectorWork (innerprod.c:203-261) */
static void exact_work(int l, const csim_projector *P, const uint64_t *L, int k, int exact, double *re,
                       double *im) {
    const int t = P->nqubits;
    const int chi = exact ? (int)pow(2, ceil((double)t / 2)) : (int)pow(2, k);
    int i = 0;
    while (l >= chi - i) {
        l -= chi - i;
        i += 1;
    }
    const int j = l + i;
    csim_state th, phi;
    prep_term(exact, i, t, L, k, &th);
    const double projfactor = orc_project(&th, P);
    *re = 0;
    *im = 0;
    if (projfactor == 0) return;
    prep_term(exact, j, t, L, k, &phi);
    int eps = 0, p = 0, m = 0;
    orc_inner_product_exact(&th, &phi, &eps, &p, &m);
    double ir = 0, ii = 0;
    add_w(&ir, &ii, eps, p, m);
    if (i == j) {
        *re = ir * projfactor;
        *im = ii * projfactor;
    } else {
        *re = ir * (2 * projfactor);
        *im = 0;
    }
}

double orc_exact_projector(const csim_projector *P, const uint64_t *L, int k, int exact, double norm) {
    if (P->nstabs == 0) return pow(norm, 2);
    if (P->nqubits == 0) return clifford_sum(P) / (1 + (double)P->nstabs);
    const int size = exact ? (int)ceil((double)P->nqubits / 2) : k;
    const int krange = (int)(pow(2, size - 1) * (pow(2, size) + 1));
    double tr = 0, ti = 0;
    for (int l = 0; l < krange; l++) {
        double re, im;
        exact_work(l, P, L, k, exact, &re, &im);
        tr += re;
        ti += im;
    }
    return sqrt(tr * tr + ti * ti);
}

/* ======================================================================
 * decompose (probability.c:307-415)
 * ==================================================================== */
static int gf2_rank(const uint64_t *rows, int nrows) {
    uint64_t m[CSIM_MAX_QUBITS];
    memcpy(m, rows, sizeof(uint64_t) * (size_t)nrows);
    int rank = 0;
    for (int c = 0; c < 64 && rank < nrows; c++) {
        int piv = -1;
        for (int r = rank; r < nrows; r++)
            if (BIT(m[r], c)) {
                piv = r;
                break;
            }
        if (piv < 0) continue;
        uint64_t t = m[piv];
        m[piv] = m[rank];
        m[rank] = t;
        for (int r = 0; r < nrows; r++)
            if (r != rank && BIT(m[r], c)) m[r] ^= m[rank];
        rank++;
    }
    return rank;
}

void orc_decompose(int t, double fidbound, int rank, int fidelity, int forceL, int *exact, int *k,
                   double *norm, uint64_t *L_out, orc_rng *r) {
    if (t == 0) {
        *exact = 0;
        *norm = 1;
        return;
    }
    const double v = cos(3.14159265358979323846 / 8);
    *norm = pow(2, floor((float)t / 2) / 2);
    if (t % 2) *norm *= 2 * v;
    if (*exact) return;
    int forceK = 1;
    if (*k <= 0) {
        forceK = 0;
        *k = (int)ceil(1 - 2 * t * log2(v) - log2(fidbound));
    }
    if (*k > t / 2 && !forceK && !forceL) {
        *exact = 1;
        return;
    }
    if (*k > t) *k = t;
    double inner = 0, Z_L = 0;
    while (inner < 1 - fidbound || forceK) {
        /* BitMatrixSetRandom: ceil(k*t/8) bytes over the row-major bit array */
        const int kk = *k, bytes = (kk * t + 7) / 8;
        for (int i = 0; i < kk; i++) L_out[i] = 0;
        for (int b = 0; b < bytes; b++) {
            const int byte = orc_rand(r) % 256;
            for (int j = 0; j < 8; j++) {
                const int g = 8 * b + j;
                if (g < kk * t && (byte & (0x80 >> j))) L_out[g / t] |= ONE(g % t);
            }
        }
        if (rank && gf2_rank(L_out, kk) < kk) continue;
        if (fidelity) {
            Z_L = 0;
            for (int i = 0; i < (int)pow(2, kk); i++) {
                const int hamming = popc(orc_codeword(i, L_out, kk));
                Z_L += pow(2, -hamming / 2);
            }
            inner = pow(2, kk) * pow(v, 2 * t) / Z_L;
            if (forceK) break;
        } else {
            break;
        }
    }
    if (fidelity) *norm = sqrt(pow(2, *k) * Z_L);
}

/* ======================================================================
 * multi-threaded pair grid (the CPU baseline and the large parity checks)
 * ==================================================================== */
typedef struct {
    int t, exact, k;
    const uint64_t *L;
    int64_t ntheta, j0, nj;
    const csim_state *theta;
    int32_t *eps, *p, *m;
    int64_t next; /* work cursor, guarded by mu */
    pthread_mutex_t mu;
} grid_job;

static void *grid_worker(void *arg) {
    grid_job *g = (grid_job *)arg;
    const int64_t total = g->ntheta * g->nj, chunk = 16;
    csim_state phi;
    for (;;) {
        pthread_mutex_lock(&g->mu);
        const int64_t s = g->next;
        g->next += chunk;
        pthread_mutex_unlock(&g->mu);
        if (s >= total) break;
        const int64_t e = s + chunk < total ? s + chunk : total;
        for (int64_t w = s; w < e; w++) {
            const int64_t a = w / g->nj, j = g->j0 + w % g->nj;
            int eps = 0, p = 0, m = 0;
            prep_term(g->exact, j, g->t, g->L, g->k, &phi);
            orc_inner_product_exact(&g->theta[a], &phi, &eps, &p, &m);
            g->eps[w] = eps;
            g->p[w] = p;
            g->m[w] = m;
        }
    }
    return NULL;
}

void orc_term_products(int t, int exact, const uint64_t *L, int k, int64_t ntheta, const csim_state *theta,
                       int64_t j0, int64_t nj, int32_t *eps, int32_t *p, int32_t *m, int threads) {
    grid_job g = {t, exact, k, L, ntheta, j0, nj, theta, eps, p, m, 0, PTHREAD_MUTEX_INITIALIZER};
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    pthread_t th[256];
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, grid_worker, &g);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
}

/* multiSampledProjector (innerprod.c:23-84) with the pair work on host
 * threads.  States are drawn and projected one after another, consuming rand()
 * exactly as orc_single_projector_sample does (the term loop draws nothing);
 * the (eps, p, m) of every pair come from the threaded grid; then each state's
 * terms are added in term order with the same double arithmetic.  So the value
 * is orc_multi_sampled_projector's, bit for bit.  values[i] (if not NULL)
 * receives state i's singleProjectorSample value. */
double orc_multi_sampled_projector_mt(const csim_projector *P, const uint64_t *L, int k, int exact, double norm,
                                      int samples, int bins, orc_rng *r, int threads, double *values) {
    if (P->nstabs == 0 || P->nqubits == 0) {
        if (values) memset(values, 0, sizeof(double) * (size_t)samples * (size_t)bins);
        return orc_multi_sampled_projector(P, L, k, exact, norm, samples, bins, r);
    }
    const int t = P->nqubits;
    const int64_t total = (int64_t)samples * bins;
    const int64_t size = exact ? (int64_t)pow(2, ceil((double)t / 2)) : (int64_t)pow(2, k);
    double *val = (double *)malloc(sizeof(double) * (size_t)(total > 0 ? total : 1));
    /* states in groups of at most 2^24 pairs */
    int64_t group = ((int64_t)1 << 24) / size;
    if (group < 1) group = 1;
    csim_state *th = (csim_state *)malloc(sizeof(csim_state) * (size_t)group);
    double *pf = (double *)malloc(sizeof(double) * (size_t)group);
    int64_t *live = (int64_t *)malloc(sizeof(int64_t) * (size_t)group);
    csim_state *lth = (csim_state *)malloc(sizeof(csim_state) * (size_t)group);
    int32_t *eps = (int32_t *)malloc(sizeof(int32_t) * (size_t)(group * size));
    int32_t *pp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(group * size));
    int32_t *mm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(group * size));
    for (int64_t o = 0; o < total; o += group) {
        const int64_t c = total - o < group ? total - o : group;
        int64_t nl = 0;
        for (int64_t i = 0; i < c; i++) {
            orc_random_state(t, r, &th[i]);
            pf[i] = orc_project(&th[i], P);
            if (pf[i] != 0) {
                live[nl] = i;
                lth[nl++] = th[i];
            }
            val[o + i] = 0;
        }
        if (nl) orc_term_products(t, exact, L, k, nl, lth, 0, size, eps, pp, mm, threads);
        for (int64_t a = 0; a < nl; a++) {
            double tr = 0, ti = 0;
            for (int64_t j = 0; j < size; j++) add_w(&tr, &ti, eps[a * size + j], pp[a * size + j], mm[a * size + j]);
            const double x = tr * pf[live[a]], y = ti * pf[live[a]];
            val[o + live[a]] = pow(2, t) * (x * x + y * y);
        }
    }
    free(th);
    free(pf);
    free(live);
    free(lth);
    free(eps);
    free(pp);
    free(mm);
    double *bv = (double *)malloc(sizeof(double) * (size_t)bins);
    for (int b = 0; b < bins; b++) {
        double tot = 0;
        for (int i = 0; i < samples; i++) tot += val[(int64_t)b * samples + i];
        bv[b] = tot / samples;
    }
    double out = bv[0];
    if (bins > 1) {
        qsort(bv, (size_t)bins, sizeof(double), cmp_trunc);
        out = (bins % 2 == 1) ? bv[(bins - 1) / 2] : (bv[bins / 2] + bv[bins / 2 - 1]) / 2;
    }
    if (values) memcpy(values, val, sizeof(double) * (size_t)total);
    free(bv);
    free(val);
    return out;
}

/* ======================================================================
 * Elementary-update restatement of one (theta, prepL term) pair, with a
 * count of packed row operations (the roofline's work unit).
 *
 * Same results as orc_inner_product_exact(theta, prepL term) — the tests
 * check this — but each basis change R = I + u e_c^T is applied as rank-one
 * row/column updates instead of updateDJ's dense R J R^T.  One "row-op" is one
 * 64-bit operation on one matrix row or one bit-sliced vector: a bit test or
 * parity of a row, a row XOR, a column-bit update of a row, a row swap, or a
 * bit-sliced D/h/Q update.
 * ==================================================================== */
typedef struct {
    int n, k, Q;
    uint64_t h, D1, D2;
    uint64_t G[CSIM_MAX_QUBITS], J[CSIM_MAX_QUBITS];
} el_state;

static inline int el_getD(const el_state *s, int i) { return 2 * (2 * BIT(s->D2, i) + BIT(s->D1, i)); }

static void el_addD(el_state *s, uint64_t u, int d1, int d2) {
    const uint64_t a1 = d1 ? u : 0, a2 = d2 ? u : 0, c = s->D1 & a1;
    s->D1 ^= a1;
    s->D2 ^= a2 ^ c;
}

/* updateDJ for R = I + u1 e_c1^T + u2 e_c2^T (c2 < 0: absent) */
static void el_applyR(el_state *s, int c1, uint64_t u1, int c2, uint64_t u2, int64_t *ops) {
    const int k = s->k;
    const uint64_t km = k >= 64 ? ~0ULL : (ONE(k) - 1);
    uint64_t row1 = s->J[c1], col1 = 0, row2 = c2 >= 0 ? s->J[c2] : 0, col2 = 0;
    for (int x = 0; x < s->n; x++) {
        col1 |= (uint64_t)BIT(s->J[x], c1) << x;
        if (c2 >= 0) col2 |= (uint64_t)BIT(s->J[x], c2) << x;
    }
    const int d11 = BIT(s->D1, c1), d21 = BIT(s->D2, c1);
    const int d12 = c2 >= 0 ? BIT(s->D1, c2) : 0, d22 = c2 >= 0 ? BIT(s->D2, c2) : 0;
    el_addD(s, u1, d11, d21);
    if (c2 >= 0) el_addD(s, u2, d12, d22);
    s->D1 &= km;
    s->D2 &= km;
    uint64_t flip = u1 & ((col1 & ~((c1 + 1 >= 64) ? ~0ULL : (ONE(c1 + 1) - 1))) | (row1 & (ONE(c1) - 1)));
    if (c2 >= 0) {
        flip ^= u2 & ((col2 & ~((c2 + 1 >= 64) ? ~0ULL : (ONE(c2 + 1) - 1))) | (row2 & (ONE(c2) - 1)));
        const int jc = c1 > c2 ? BIT(row1, c2) : BIT(row2, c1);
        if (jc) flip ^= u1 & u2;
    }
    s->D2 ^= flip;
    for (int x = 0; x < s->n; x++) {
        uint64_t r = s->J[x];
        if (BIT(u1, x)) r ^= row1;
        if (c2 >= 0 && BIT(u2, x)) r ^= row2;
        uint64_t r2 = r;
        if (BIT(r, c1)) r2 ^= u1;
        if (c2 >= 0 && BIT(r, c2)) r2 ^= u2;
        s->J[x] = r2;
    }
    *ops += 2 /* pivot rows */ + popc(u1) + popc(u2) /* row XORs */ + k /* column updates */ + 3 /* D */;
}

static void el_swap(el_state *s, int i, int j, int64_t *ops) {
    const int k = s->k;
    const uint64_t km = k >= 64 ? ~0ULL : (ONE(k) - 1);
    if (i != j) {
        uint64_t t = ((s->D1 >> i) ^ (s->D1 >> j)) & 1;
        s->D1 ^= (t << i) | (t << j);
        t = ((s->D2 >> i) ^ (s->D2 >> j)) & 1;
        s->D2 ^= (t << i) | (t << j);
        uint64_t r = s->J[i];
        s->J[i] = s->J[j];
        s->J[j] = r;
        for (int x = 0; x < s->n; x++) {
            t = ((s->J[x] >> i) ^ (s->J[x] >> j)) & 1;
            s->J[x] ^= (t << i) | (t << j);
        }
        *ops += 2 + k + 2;
    }
    s->D1 &= km;
    s->D2 &= km;
}

static int el_shrink_unit(el_state *s, int q, int64_t *ops) {
    const int k = s->k;
    uint64_t S = 0;
    for (int a = 0; a < k; a++)
        if (BIT(s->G[a], q)) S |= ONE(a);
    *ops += k;
    const int beta = BIT(s->h, q);
    if (!S) return 1 - beta;
    const int i = 63 - __builtin_clzll(S);
    const uint64_t U = S & ~ONE(i);
    for (int a = 0; a < k; a++)
        if (BIT(U, a)) s->G[a] ^= s->G[i];
    *ops += popc(U);
    if (U) el_applyR(s, i, U, -1, 0, ops);
    const int kk = k - 1;
    uint64_t t = s->G[i];
    s->G[i] = s->G[kk];
    s->G[kk] = t;
    *ops += 2;
    el_swap(s, i, kk, ops);
    if (beta) {
        s->h ^= s->G[kk];
        s->Q = (s->Q + el_getD(s, kk)) % 8;
        for (int x = 0; x < s->n; x++)
            if (BIT(s->J[x], kk)) s->D2 ^= ONE(x);
        *ops += 2 + k;
    } else {
        s->Q = s->Q % 8;
    }
    s->k = kk;
    return 2;
}

static void el_partial_gamma(int A, int *e, int *p, int *m) {
    while (A < 0) A += 8;
    *e = (A % 8 == 4) ? 0 : 1;
    switch (A % 8) {
    case 0: *p = 2; *m = 0; break;
    case 2: *p = 1; *m = 1; break;
    case 4: *p = 0; *m = 0; break;
    case 6: *p = 1; *m = 7; break;
    default: orc_assert_failures++; break;
    }
}

static void el_wsigma(const el_state *s, int sigma, int sidx, uint64_t Mm, uint64_t DA, const int *partner, int *e,
                      int *p, int *m, int64_t *ops) {
    if (s->k == 0) {
        *e = 1; *p = 0; *m = s->Q;
        return;
    }
    const int tM0 = s->Q + sigma * el_getD(s, sidx >= 0 ? sidx : 0);
    int P = 0, Ms = 0;
    for (int x = 0; x < s->n; x++) {
        int ee = 1, pp = 0, mm = 0;
        if (BIT(Mm, x)) {
            el_partial_gamma(el_getD(s, x) + sigma * 4 * (sidx >= 0 ? BIT(s->J[x], sidx) : 0), &ee, &pp, &mm);
            (*ops)++;
        } else if (BIT(DA, x)) {
            const int b = partner[x];
            const int js_a = sidx >= 0 ? BIT(s->J[x], sidx) : 0, js_b = sidx >= 0 ? BIT(s->J[b], sidx) : 0;
            gamma_ab(&ee, &pp, &mm, el_getD(s, x) + sigma * 4 * js_a, el_getD(s, b) + sigma * 4 * js_b);
            (*ops)++;
        } else {
            continue;
        }
        if (!ee) {
            *e = 0; *p = 0; *m = 0;
            return;
        }
        P += pp;
        Ms += mm;
    }
    *e = 1;
    *p = P;
    *m = (Mm | DA) ? (tM0 + Ms) % 8 : tM0;
}

static void el_exp_sum(el_state *s, int *eps, int *p, int *m, int64_t *ops) {
    const int k = s->k;
    const uint64_t km = k >= 64 ? ~0ULL : (ONE(k) - 1);
    const uint64_t Sm = s->D1 & km;
    int sidx = -1;
    if (Sm) {
        const int a = __builtin_ctzll(Sm);
        const uint64_t U = Sm & ~ONE(a);
        if (U) el_applyR(s, a, U, -1, 0, ops);
        else {
            s->D1 &= km;
            s->D2 &= km;
        }
        el_swap(s, a, k - 1, ops);
        sidx = k - 1;
    }
    uint64_t E = km & ~(sidx >= 0 ? ONE(sidx) : 0);
    uint64_t Mm = 0, DA = 0;
    int partner[CSIM_MAX_QUBITS] = {0};
    while (E) {
        const int a = __builtin_ctzll(E);
        const uint64_t ra = s->J[a], K = ra & E & ~ONE(a);
        (*ops)++;
        if (!K) {
            Mm |= ONE(a);
            E &= ~ONE(a);
        } else {
            const int b = __builtin_ctzll(K);
            const uint64_t Ep = E & ~ONE(a) & ~ONE(b);
            const uint64_t vb = ra & Ep, va = s->J[b] & Ep;
            if (vb | va) el_applyR(s, b, vb, a, va, ops);
            else {
                s->D1 &= km;
                s->D2 &= km;
            }
            DA |= ONE(a);
            partner[a] = b;
            E = Ep;
        }
    }
    if (sidx < 0) {
        el_wsigma(s, 0, -1, Mm, DA, partner, eps, p, m, ops);
        return;
    }
    int e0, p0, m0, e1, p1, m1;
    el_wsigma(s, 0, sidx, Mm, DA, partner, &e0, &p0, &m0, ops);
    el_wsigma(s, 1, sidx, Mm, DA, partner, &e1, &p1, &m1, ops);
    if (e0 == 0) { *eps = e1; *p = p1; *m = m1; return; }
    if (e1 == 0) { *eps = e0; *p = p0; *m = m0; return; }
    if (p0 != p1 || ((m1 - m0) % 2) != 0) { orc_assert_failures++; return; }
    int ee, pp = 0, mm = 0;
    el_partial_gamma(m1 - m0, &ee, &pp, &mm);
    *eps = ee;
    if (!ee) { *p = 0; *m = 0; }
    else { *p = pp + p0; *m = mm + m0 % 8; }
}

void orc_pair_rowops(const csim_state *theta, uint64_t x, int *eps, int *p, int *m, int64_t *ops) {
    el_state s;
    s.n = theta->n;
    s.k = theta->k;
    s.Q = theta->Q;
    s.h = theta->h;
    s.D1 = theta->D1;
    s.D2 = theta->D2;
    memcpy(s.G, theta->G, sizeof(s.G));
    memcpy(s.J, theta->J, sizeof(s.J));
    const int k1 = s.k, k2 = popc(x);
    uint64_t zeros = ~x & (s.n >= 64 ? ~0ULL : (ONE(s.n) - 1));
    *ops = 0;
    while (zeros) {
        const int q = 63 - __builtin_clzll(zeros);
        zeros &= ~ONE(q);
        *eps = el_shrink_unit(&s, q, ops);
        if (*eps == 0) {
            *p = 0;
            *m = 0;
            return;
        }
    }
    el_exp_sum(&s, eps, p, m, ops);
    *p -= k1 + k2;
}
