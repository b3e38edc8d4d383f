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

// Warp-uniform loop bounds: on the device every lane of the warp runs the
// same number of iterations (the warp maximum) with its own work predicated,
// so the 32 pairs of a warp stay converged; on the host the bound is the
// pair's own.
CSIM_HD inline int uniform_max(int v) {
#if defined(__CUDA_ARCH__)
    return (int)__reduce_max_sync(0xffffffffu, (unsigned)v);
#else
    return v;
#endif
}

CSIM_HD inline void tp_add_D(PairRegs& s, uint64_t u, int d1, int d2) {
    const uint64_t a1 = d1 ? u : 0ull, a2 = d2 ? u : 0ull;
    const uint64_t carry = s.D1 & a1;
    s.D1 ^= a1;
    s.D2 ^= a2 ^ carry;
}

CSIM_HD inline int tp_getD(const PairRegs& s, int i) { return 2 * (2 * getbit(s.D2, i) + getbit(s.D1, i)); }

// Shrink by e_q (alpha = 0), stabilizer.c:500-585, for a symmetric J.
// `act`: this lane has a shrink to do.  Returns 0 EMPTY, 1 SAME, 2 SUCCESS
// (1 when inactive).  All lanes must call it together.
//
// With R = I + U e_i^T (U = S \ {i}, i = max S) and J symmetric,
//   R J R^T = J + U Ji^T + Ji U^T + J_ii U U^T,
// i.e. row x gets Ji if x in U and U if x in C = Ji ^ (J_ii ? U : 0); then
// basis vectors i and kk = k-1 swap and kk is dropped: row kk moves to slot
// i and every row's bit i becomes its old bit kk = bit x of row kk.  The +4
// corrections of updateDJ are U & Ji, and updateQD's J.y is column kk of the
// result, i.e. C with bit i taken from bit kk of C.
CSIM_HD inline int tp_shrink(PairRegs& s, uint64_t* sJ, uint64_t* sGT, int st, int q, uint64_t zrem, bool act) {
    const int k = s.k;
    const uint64_t km = lowmask(k);
    const uint64_t S = act ? (RG(q) & km) : 0ull;
    const int beta = act ? getbit(s.h, q) : 0;
    const bool upd = S != 0ull;
    const int i = upd ? 63 - hd_clz64(S) : 0;
    const uint64_t U = S & ~bit1(i);
    const int kk = k - 1;

    // G, column form: rows in U get the pivot row, row kk moves to slot i;
    // h gets the pivot row when beta = 1 (stabilizer.c:530-533, 557, 569-573)
    const uint64_t mi = bit1(i), mk = bit1(kk & 63);
    const int nz = upd ? hd_popc64(zrem) : 0;
    const int NZ = uniform_max(nz);
    uint64_t z = zrem, hflip = 0ull;
    for (int t = 0; t < NZ; t++) {
        if (t < nz) {
            const int c = hd_ffs64(z) - 1;
            const uint64_t mc = z & (0ull - z);  // lowest remaining zero column, as a mask
            z ^= mc;
            uint64_t g = RG(c);
            const uint64_t gi = 0ull - (uint64_t)((g & mi) != 0ull);
            g ^= U & gi;
            g = (g & ~mi) | (mi & (0ull - (uint64_t)((g & mk) != 0ull)));
            RG(c) = g;
            hflip |= mc & gi;
        }
    }
    if (beta) s.h ^= hflip;

    // J: rank-two update, then the i <-> kk swap and drop of kk
    const uint64_t Ji = upd ? RJ(i) : 0ull;
    const uint64_t C = Ji ^ (getbit(Ji, i) ? U : 0ull);  // new row (and column) i
    const uint64_t Jk = upd ? (RJ(kk) ^ (getbit(C, kk) ? U : 0ull)) : 0ull;  // new row kk (kk not in U)
    // every row of the lane's block is rewritten (rows i and kk get values that are
    // replaced or dropped just below), so the pass is branch-free; rows at or
    // beyond k are outside the block and never read again
    const int KX = uniform_max(upd ? k : 0);
    if (upd) {
        uint64_t cu = U, cc = C, cj = Jk;
        for (int x = 0; x < KX; x++) {
            uint64_t r = RJ(x);
            r ^= Ji & (0ull - (cu & 1ull));
            r ^= U & (0ull - (cc & 1ull));
            r = (r & ~mi) | (mi & (0ull - (cj & 1ull)));
            RJ(x) = r;
            cu >>= 1;
            cc >>= 1;
            cj >>= 1;
        }
    }
    if (upd && i != kk) RJ(i) = (Jk & ~mi) | (mi & (0ull - ((Jk >> kk) & 1ull)));
    if (upd) {
        // D: eq. 49 and the lower-triangle parities (J[max][min] = Ji by symmetry)
        tp_add_D(s, U, getbit(s.D1, i), getbit(s.D2, i));
        s.D2 ^= U & Ji;
        if (i != kk) {
            s.D1 = swapbits(s.D1, i, kk);
            s.D2 = swapbits(s.D2, i, kk);
        }
        s.D1 &= km;
        s.D2 &= km;
        if (beta) {
            s.Q = (s.Q + tp_getD(s, kk)) % 8;
            s.D2 ^= ((C & ~bit1(i)) | (((C >> kk) & 1ull) << i)) & lowmask(kk);
        } else {
            s.Q = s.Q % 8;
        }
        s.k = kk;
        return 2;
    }
    return act ? 1 - beta : 1;
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

// exponentialSumExact (stabilizer.c:300-481), symmetric J; `act` as for tp_shrink.
CSIM_HD inline void tp_exp_sum(PairRegs& s, uint64_t* sJ, int st, bool act, int& eps, int& p, int& m, int& err) {
    const int k = act ? s.k : 0;
    const uint64_t km = lowmask(k);
    const uint64_t Sm = s.D1 & km;
    int sidx = -1;
    {
        // R = I + U e_a^T, then swap a <-> kk (stabilizer.c:317-336); kk may lie in U
        const bool upd = Sm != 0ull;
        const int a = upd ? hd_ffs64(Sm) - 1 : 0;
        const uint64_t U = Sm & ~bit1(a);
        const int kk = k - 1;
        const uint64_t Ja = upd ? RJ(a) : 0ull;
        const uint64_t C = Ja ^ (getbit(Ja, a) ? U : 0ull);  // new row/column a
        const uint64_t Jk = upd ? (RJ(kk) ^ (getbit(U, kk) ? Ja : 0ull) ^ (getbit(C, kk) ? U : 0ull)) : 0ull;
        const int KX = uniform_max(upd ? k : 0);
        if (upd) {
            // rows a and kk are rewritten below; the pass itself is branch-free
            const uint64_t ma = bit1(a), mk = bit1(kk & 63);
            uint64_t cu = U, cc = C, cj = Jk;
            for (int x = 0; x < KX; x++) {
                uint64_t r = RJ(x);
                r ^= Ja & (0ull - (cu & 1ull));
                r ^= U & (0ull - (cc & 1ull));
                // swap bits a and kk: bit a <- J'[x][kk] = bit x of Jk, bit kk <- J'[x][a] = bit x of C
                r = (r & ~(ma | mk)) | (ma & (0ull - (cj & 1ull))) | (mk & (0ull - (cc & 1ull)));
                RJ(x) = r;
                cu >>= 1;
                cc >>= 1;
                cj >>= 1;
            }
        }
        if (upd && a != kk) {
            RJ(a) = swapbits(Jk, a, kk);
            RJ(kk) = swapbits(C, a, kk);
        } else if (upd) {
            RJ(a) = C;
        }
        if (upd) {
            tp_add_D(s, U, getbit(s.D1, a), getbit(s.D2, a));
            s.D2 ^= U & Ja;
            s.D1 = swapbits(s.D1, a, kk) & km;
            s.D2 = swapbits(s.D2, a, kk) & km;
            sidx = kk;
        }
    }
    uint64_t E = km & ~(sidx >= 0 ? bit1(sidx) : 0ull);
    WAcc w0 = {0, 0, 0}, w1 = {0, 0, 0};
    const bool any = E != 0ull;
    const int NE = uniform_max(hd_popc64(E));
    for (int it = 0; it < NE; it++) {
        const bool live = E != 0ull;
        const int a = live ? hd_ffs64(E) - 1 : 0;
        const uint64_t ra = live ? RJ(a) : 0ull;
        const uint64_t K = ra & E & ~bit1(a);
        const bool dimer = K != 0ull;
        const int b = dimer ? hd_ffs64(K) - 1 : 0;
        const uint64_t rb = dimer ? RJ(b) : 0ull;
        if (live && !dimer) {  // monomer {a}: row a is final
            const int Da = tp_getD(s, a);
            tp_factor_mono(w0, Da, err);
            if (sidx >= 0) tp_factor_mono(w1, Da + 4 * getbit(ra, sidx), err);
        }
        if (dimer) {  // dimer {a, b}: rows a and b are final
            const int Da = tp_getD(s, a), Db = tp_getD(s, b);
            tp_factor_dimer(w0, Da, Db, err);
            if (sidx >= 0) tp_factor_dimer(w1, Da + 4 * getbit(ra, sidx), Db + 4 * getbit(rb, sidx), err);
        }
        const uint64_t Ep = dimer ? (E & ~bit1(a) & ~bit1(b)) : (E & ~bit1(a));
        const uint64_t vb = dimer ? (ra & Ep) : 0ull, va = dimer ? (rb & Ep) : 0ull;
        const bool upd = (vb | va) != 0ull;
        // R = I + vb e_b^T + va e_a^T on the rows still in play (Ep):
        //   row x += vb_x Jb + va_x Ja + Cb_x vb + Ca_x va, with the coefficient
        //   columns Cb = (RJ)[.][b], Ca = (RJ)[.][a] (symmetric J)
        const int jaa = getbit(ra, a), jbb = getbit(rb, b), jab = getbit(ra, b);
        const uint64_t Cb = rb ^ (jbb ? vb : 0ull) ^ (jab ? va : 0ull);
        const uint64_t Ca = ra ^ (jab ? vb : 0ull) ^ (jaa ? va : 0ull);
        const int np = upd ? hd_popc64(Ep) : 0;
        const int NP = uniform_max(np);
        uint64_t zz = Ep;
        for (int t = 0; t < NP; t++) {
            if (t < np) {
                const int x = hd_ffs64(zz) - 1;
                zz &= zz - 1;
                uint64_t r = RJ(x);
                r ^= rb & (0ull - ((vb >> x) & 1ull));
                r ^= ra & (0ull - ((va >> x) & 1ull));
                r ^= vb & (0ull - ((Cb >> x) & 1ull));
                r ^= va & (0ull - ((Ca >> x) & 1ull));
                RJ(x) = r;
            }
        }
        if (upd) {
            const int db1 = getbit(s.D1, b), db2 = getbit(s.D2, b), da1 = getbit(s.D1, a), da2 = getbit(s.D2, a);
            tp_add_D(s, vb, db1, db2);
            tp_add_D(s, va, da1, da2);
            uint64_t flip = (vb & rb) ^ (va & ra);
            if (jab) flip ^= vb & va;
            s.D2 ^= flip;
        }
        if (live) E = Ep;
    }
    if (!act) return;
    if (k == 0) {  // Wsigma's k == 0 case
        eps = 1; p = 0; m = s.Q;
        return;
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

// One pair: theta's pristine J rows and G columns (as row masks), codeword x;
// working memory sJ/sGT (stride st), n indices each.  J must be symmetric.
// `valid` = this lane has a pair (all lanes of a warp call together).
CSIM_HD inline void pair_l(bool valid, int n, int k1, int Q, uint64_t h, uint64_t D1, uint64_t D2, const uint64_t* pJ,
                           const uint64_t* pGT, uint64_t x, uint64_t* sJ, uint64_t* sGT, int st, int& eps, int& p,
                           int& m, int& err) {
    PairRegs s;
    s.k = k1;
    s.Q = Q;
    s.h = h;
    s.D1 = D1;
    s.D2 = D2;
    if (valid)
        for (int r = 0; r < k1; r++) RJ(r) = pJ[r];
    uint64_t zeros = valid ? (~x & lowmask(n)) : 0ull;
    for (uint64_t zz = zeros; zz; zz &= zz - 1) {
        const int c = hd_ffs64(zz) - 1;
        RG(c) = pGT[c];
    }
    eps = 0;
    p = 0;
    m = 0;
    bool alive = valid;
    const int NZ = uniform_max(hd_popc64(zeros));
    for (int it = 0; it < NZ; it++) {
        const bool act = alive && zeros != 0ull;
        const int q = act ? 63 - hd_clz64(zeros) : 0;
        if (act) zeros &= ~bit1(q);
        const int r = tp_shrink(s, sJ, sGT, st, q, zeros, act);
        if (act && r == 0) alive = false;
    }
    tp_exp_sum(s, sJ, st, alive, eps, p, m, err);
    if (alive) p -= k1 + hd_popc64(x);
    else {
        eps = 0;
        p = 0;
        m = 0;
    }
}

#undef RJ
#undef RG

}  // namespace pc
}  // namespace csim
