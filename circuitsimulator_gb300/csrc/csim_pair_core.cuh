// csim_pair_core.cuh — one (theta, prepL term) pair, the body of the
// thread-per-pair kernel (csim_terms_tp.cu), written once for the device and
// the host: the same functions are compiled into a host-side checker
// (tests/native/tp_host_check.cu) that the CPU tests compare with the oracle.
//
// The pair's J rows and G columns live in caller-provided memory with stride
// `st` words between consecutive indices (the kernel's shared-memory
// [index][thread] layout; 1 on the host).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define CSIM_HD __host__ __device__
#else
#define CSIM_HD
#endif

namespace csim {
namespace pc {

CSIM_HD inline int hd_popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}
// 1-based index of the lowest set bit, 0 for x == 0 (like ffsll)
CSIM_HD inline int hd_ffs64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __ffsll((long long)x);
#else
    return __builtin_ffsll((long long)x);
#endif
}
CSIM_HD inline int hd_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}
CSIM_HD inline uint64_t bit1(int i) { return 1ull << i; }
CSIM_HD inline uint64_t lowmask(int k) { return k >= 64 ? ~0ull : ((1ull << k) - 1ull); }
CSIM_HD inline int getbit(uint64_t w, int i) { return (int)((w >> i) & 1ull); }
CSIM_HD inline uint64_t swapbits(uint64_t w, int i, int j) {
    const uint64_t t = ((w >> i) ^ (w >> j)) & 1ull;
    return w ^ ((t << i) | (t << j));
}

enum : int { kErrRange = 1, kErrExpSum = 4, kErrGamma = 8 };

// partialGamma (stabilizer.c:228-255): 1 + e^{i pi A/4}
CSIM_HD inline void partial_gamma(int A, int& e, int& p, int& m, int& err) {
    while (A < 0) A += 8;
    const int r = A % 8;
    e = (r == 4) ? 0 : 1;
    switch (r) {
    case 0: p = 2; m = 0; break;
    case 2: p = 1; m = 1; break;
    case 4: p = 0; m = 0; break;
    case 6: p = 1; m = 7; break;
    default: err |= kErrGamma; break;
    }
}

// Gamma (stabilizer.c:183-225): 1 + e^{i pi A/4} + e^{i pi B/4} - e^{i pi (A+B)/4}
CSIM_HD inline void gamma_ab(int A, int B, int& e, int& p, int& m, int& err) {
    if ((A % 2) || (B % 2) || A < 0 || B < 0) {
        err |= kErrGamma;
        e = 0; p = 0; m = 0;
        return;
    }
    const int a = (A % 8) / 2, b = (B % 8) / 2, c = ((A + B) % 8) / 2;
    const int gr = 1 + ((a == 0) - (a == 2)) + ((b == 0) - (b == 2)) - ((c == 0) - (c == 2));
    const int gi = ((a == 1) - (a == 3)) + ((b == 1) - (b == 3)) - ((c == 1) - (c == 3));
    if (gr == 0 && gi == 0) {
        e = 0; p = 0; m = 0;
        return;
    }
    e = 1;
    p = 2;
    if (gr == 0) m = gi > 0 ? 2 : 6;
    else if (gr == -2) m = 4;
    else if (gi == 2) m = 1;
    else if (gi == 0) m = 0;
    else if (gi == -2) m = 7;
    else err |= kErrGamma;
}

#define RJ(r) sJ[(size_t)(r) * st]
#define RG(c) sGT[(size_t)(c) * st]

struct PairRegs {
    int k, Q;
    uint64_t h, D1, D2;
};


CSIM_HD inline void tp_add_D(PairRegs& s, uint64_t u, int d1, int d2) {
    const uint64_t a1 = d1 ? u : 0ull, a2 = d2 ? u : 0ull;
    const uint64_t carry = s.D1 & a1;
    s.D1 ^= a1;
    s.D2 ^= a2 ^ carry;
}

// shrink by e_q (alpha = 0) on the thread's pair; returns 0 EMPTY, 1 SAME, 2 SUCCESS.
// `zrem` = zero columns still to be used (only those columns of G are kept).
CSIM_HD inline int tp_shrink(PairRegs& s, uint64_t* sJ, uint64_t* sGT, int st, int q, uint64_t zrem) {
    const int k = s.k;
    const uint64_t km = lowmask(k);
    const uint64_t S = RG(q) & km;
    const int beta = getbit(s.h, q);
    if (!S) return 1 - beta;
    const int i = 63 - hd_clz64(S);
    const uint64_t U = S & ~bit1(i);
    const int kk = k - 1;

    // G (column form): rows in U get the pivot row, then row kk moves into slot i;
    // h gets the pivot row when beta = 1 (stabilizer.c:530-533, 557, 569-573)
    uint64_t z = zrem;
    while (z) {
        const int c = hd_ffs64(z) - 1;
        z &= z - 1;
        uint64_t g = RG(c);
        const uint64_t gi = (g >> i) & 1ull;
        g ^= U & (0ull - gi);
        const uint64_t gk = (g >> kk) & 1ull;
        g = (g & ~bit1(i)) | (gk << i);
        RG(c) = g;
        if (beta) s.h ^= gi << c;
    }

    // J: R = I + U e_i^T (rows, then columns), then the swap i <-> kk; gather the
    // pivot's original column (D2 corrections) and the final column kk (beta term)
    const uint64_t Ji = RJ(i);
    uint64_t colI = 0ull, colK = 0ull;
    for (int x = 0; x < k; x++) {
        uint64_t r = RJ(x);
        colI |= ((r >> i) & 1ull) << x;
        r ^= Ji & (0ull - ((U >> x) & 1ull));
        r ^= U & (0ull - ((r >> i) & 1ull));
        // column swap i <-> kk, row x goes to slot dst; the pivot row lands in
        // slot kk, which the shrink drops, so slot kk is never written (and is
        // still unread when x = i comes first, i < kk)
        const uint64_t tb = ((r >> i) ^ (r >> kk)) & 1ull;
        r ^= (tb << i) | (tb << kk);
        const int dst = (x == kk) ? i : ((x == i) ? kk : x);
        colK |= ((r >> kk) & 1ull) << dst;
        if (dst != kk) RJ(dst) = r;
    }
    // D (eq. 49 + lower-triangle corrections), swap, beta term (updateQD)
    const uint64_t Li = (colI & ~lowmask(i + 1)) | (Ji & lowmask(i));
    tp_add_D(s, U, getbit(s.D1, i), getbit(s.D2, i));
    s.D2 ^= U & Li;
    if (i != kk) {
        s.D1 = swapbits(s.D1, i, kk);
        s.D2 = swapbits(s.D2, i, kk);
    }
    s.D1 &= km;
    s.D2 &= km;
    if (beta) {
        s.Q = (s.Q + 2 * (2 * getbit(s.D2, kk) + getbit(s.D1, kk))) % 8;
        s.D2 ^= colK;
    } else {
        s.Q = s.Q % 8;
    }
    s.k = kk;
    return 2;
}

// W0/W1 accumulators of Wsigma (stabilizer.c:258-297)
struct WAcc {
    int zero, p, m;
};

CSIM_HD inline void tp_factor_mono(WAcc& w, int A, int& err) {
    int e, p = 0, m = 0;
    partial_gamma(A, e, p, m, err);
    if (!e) w.zero = 1;
    w.p += p;
    w.m += m;
}

CSIM_HD inline void tp_factor_dimer(WAcc& w, int A, int B, int& err) {
    int e, p = 0, m = 0;
    gamma_ab(A, B, e, p, m, err);
    if (!e) w.zero = 1;
    w.p += p;
    w.m += m;
}

CSIM_HD inline int tp_getD(const PairRegs& s, int i) {
    return 2 * (2 * getbit(s.D2, i) + getbit(s.D1, i));
}

// exponentialSumExact (stabilizer.c:300-481) on the thread's pair
CSIM_HD inline void tp_exp_sum(PairRegs& s, uint64_t* sJ, int st, int& eps, int& p, int& m, int& err) {
    const int k = s.k;
    const uint64_t km = lowmask(k);
    if (k == 0) {  // Wsigma's k == 0 case
        eps = 1; p = 0; m = s.Q;
        return;
    }
    const uint64_t Sm = s.D1 & km;
    int sidx = -1;
    if (Sm) {
        // R = I + U e_a^T, then swap a <-> k-1 (stabilizer.c:317-336)
        const int a = hd_ffs64(Sm) - 1;
        const uint64_t U = Sm & ~bit1(a);
        const int kk = k - 1;
        const uint64_t Ja = RJ(a), Jk = RJ(kk);  // row a is stored into slot kk before x = kk is read
        uint64_t colA = 0ull;
        for (int x = 0; x < k; x++) {
            uint64_t r = (x == kk) ? Jk : RJ(x);
            colA |= ((r >> a) & 1ull) << x;
            r ^= Ja & (0ull - ((U >> x) & 1ull));
            r ^= U & (0ull - ((r >> a) & 1ull));
            const uint64_t tb = ((r >> a) ^ (r >> kk)) & 1ull;
            r ^= (tb << a) | (tb << kk);
            const int dst = (x == kk) ? a : ((x == a) ? kk : x);
            RJ(dst) = r;
        }
        const uint64_t La = (colA & ~lowmask(a + 1)) | (Ja & lowmask(a));
        tp_add_D(s, U, getbit(s.D1, a), getbit(s.D2, a));
        s.D2 ^= U & La;
        s.D1 = swapbits(s.D1, a, kk) & km;
        s.D2 = swapbits(s.D2, a, kk) & km;
        sidx = kk;
    }
    uint64_t E = km & ~(sidx >= 0 ? bit1(sidx) : 0ull);
    WAcc w0 = {0, 0, 0}, w1 = {0, 0, 0};
    bool any = false;
    while (E) {
        const int a = hd_ffs64(E) - 1;
        const uint64_t ra = RJ(a);
        const uint64_t K = ra & E & ~bit1(a);
        any = true;
        if (!K) {  // monomer {a}: row a is final
            E &= ~bit1(a);
            const int Da = tp_getD(s, a);
            tp_factor_mono(w0, Da, err);
            if (sidx >= 0) tp_factor_mono(w1, Da + 4 * getbit(ra, sidx), err);
            continue;
        }
        const int b = hd_ffs64(K) - 1;
        const uint64_t rb = RJ(b);
        const uint64_t Ep = E & ~bit1(a) & ~bit1(b);
        const uint64_t vb = ra & Ep, va = rb & Ep;
        // dimer {a, b}: rows a and b are final now (D, and their bit sidx)
        {
            const int Da = tp_getD(s, a), Db = tp_getD(s, b);
            tp_factor_dimer(w0, Da, Db, err);
            if (sidx >= 0) tp_factor_dimer(w1, Da + 4 * getbit(ra, sidx), Db + 4 * getbit(rb, sidx), err);
        }
        if (vb | va) {
            // R = I + vb e_b^T + va e_a^T on the rows still in play (Ep); the other
            // rows of R are the identity, so their J rows and D entries stay put
            // except for columns a, b, which nothing reads again.
            uint64_t colA = 0ull, colB = 0ull;
            uint64_t z = Ep;
            while (z) {
                const int x = hd_ffs64(z) - 1;
                z &= z - 1;
                uint64_t r = RJ(x);
                colA |= ((r >> a) & 1ull) << x;
                colB |= ((r >> b) & 1ull) << x;
                r ^= rb & (0ull - ((vb >> x) & 1ull));
                r ^= ra & (0ull - ((va >> x) & 1ull));
                const uint64_t bb = (r >> b) & 1ull, ba = (r >> a) & 1ull;
                r ^= vb & (0ull - bb);
                r ^= va & (0ull - ba);
                RJ(x) = r;
            }
            const int db1 = getbit(s.D1, b), db2 = getbit(s.D2, b), da1 = getbit(s.D1, a), da2 = getbit(s.D2, a);
            tp_add_D(s, vb, db1, db2);
            tp_add_D(s, va, da1, da2);
            const uint64_t Lb = (colB & ~lowmask(b + 1)) | (rb & lowmask(b));
            const uint64_t La = (colA & ~lowmask(a + 1)) | (ra & lowmask(a));
            uint64_t flip = (vb & Lb) ^ (va & La);
            const int jab = (b > a) ? getbit(rb, a) : getbit(ra, b);
            if (jab) flip ^= vb & va;
            s.D2 ^= flip;
        }
        E = Ep;
    }
    // W0 = Wsigma(sigma = 0), W1 = Wsigma(sigma = 1) (stabilizer.c:425-479)
    const int tM0 = s.Q, tM1 = s.Q + (sidx >= 0 ? tp_getD(s, sidx) : 0);
    const int e0 = !w0.zero, p0 = w0.zero ? 0 : w0.p, m0 = w0.zero ? 0 : (any ? (tM0 + w0.m) % 8 : tM0);
    if (sidx < 0) {
        eps = e0; p = p0; m = m0;
        return;
    }
    const int e1 = !w1.zero, p1 = w1.zero ? 0 : w1.p, m1 = w1.zero ? 0 : (any ? (tM1 + w1.m) % 8 : tM1);
    if (e0 == 0) {
        eps = e1; p = p1; m = m1;
        return;
    }
    if (e1 == 0) {
        eps = e0; p = p0; m = m0;
        return;
    }
    if (p0 != p1 || ((m1 - m0) % 2) != 0) {
        err |= kErrExpSum;
        return;
    }
    int ee, pp = 0, mm = 0;
    partial_gamma(m1 - m0, ee, pp, mm, err);
    eps = ee;
    if (!ee) {
        p = 0; m = 0;
    } else {
        p = pp + p0;
        m = mm + m0 % 8;
    }
}



// Adds eps 2^{p/2} w^m, scaled by 2^{P/2}, to z = z0 + z1 w + z2 w^2 + z3 w^3
// (w = e^{i pi/4}, sqrt 2 = w - w^3).  With P = 2n every term of a pair's
// p in [-2n, n] is an integer below 2^96, exact in 128 bits.
CSIM_HD inline void zacc(__int128 (&z)[4], int eps, int p, int m, int P, int& err) {
    if (!eps) return;
    const int q = p + P;
    if (q < 0 || q > 192 || eps != 1) {
        err |= kErrRange;
        return;
    }
    const int mm = ((m % 8) + 8) % 8;
    if ((q & 1) == 0) {
        const __int128 c = (__int128)1 << (q / 2);
        z[mm & 3] += (mm >= 4) ? -c : c;
    } else {
        const __int128 c = (__int128)1 << ((q - 1) / 2);
        const int a = (mm + 1) % 8, b = (mm + 3) % 8;
        z[a & 3] += (a >= 4) ? -c : c;
        z[b & 3] -= (b >= 4) ? -c : c;
    }
}

// One pair: theta's pristine rows in (J, GT-columns-as-row-masks), codeword x.
// The caller provides working memory sJ/sGT (stride st) of n indices each.
CSIM_HD inline void pair_l(int n, int k1, int Q, uint64_t h, uint64_t D1, uint64_t D2, const uint64_t* pJ,
                           const uint64_t* pGT, uint64_t x, uint64_t* sJ, uint64_t* sGT, int st, int& eps, int& p,
                           int& m, int& err) {
    PairRegs s;
    s.k = k1;
    s.Q = Q;
    s.h = h;
    s.D1 = D1;
    s.D2 = D2;
    for (int r = 0; r < k1; r++) RJ(r) = pJ[r];
    uint64_t zeros = ~x & lowmask(n);
    for (uint64_t zz = zeros; zz; zz &= zz - 1) {
        const int c = hd_ffs64(zz) - 1;
        RG(c) = pGT[c];
    }
    eps = 0;
    p = 0;
    m = 0;
    while (zeros) {
        const int q = 63 - hd_clz64(zeros);
        zeros &= ~bit1(q);
        eps = tp_shrink(s, sJ, sGT, st, q, zeros);
        if (eps == 0) {
            p = 0;
            m = 0;
            return;
        }
    }
    tp_exp_sum(s, sJ, st, eps, p, m, err);
    p -= k1 + hd_popc64(x);
}

#undef RJ
#undef RG

}  // namespace pc
}  // namespace csim
