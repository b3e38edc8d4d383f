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

// J rows are stored in pairs: rows 2p and 2p+1 are adjacent 64-bit slots, so
// one 16-byte access moves both; pair p of a lane is 2*st slots after pair
// p-1.  G columns are single slots st apart.  While every row-space index
// of a pair is below 32 (k <= 32) the arithmetic runs on 32-bit words W
// and only the low halves of the slots are read (the high halves are left
// as they are and never read again).
#define RJ(r) sJ[(size_t)((r) >> 1) * 2 * st + ((r) & 1)]

// 64-bit row arithmetic while the warp's largest k exceeds this.  Builds of
// the host checker set it to 0 to run the 64-bit code on every pair, as a
// lane with k <= 32 does in a warp that still has a larger k.
#ifndef CSIM_TP_WIDE_FROM
#define CSIM_TP_WIDE_FROM 32
#endif
#define RG(c) sGT[(size_t)(c) * st]

struct alignas(16) U64x2 {
    uint64_t a, b;
};

template <class W>
struct WordTraits;
template <>
struct WordTraits<uint64_t> {
    static constexpr int bits = 64;
    CSIM_HD static int popc(uint64_t x) { return hd_popc64(x); }
    CSIM_HD static int ffs(uint64_t x) { return hd_ffs64(x); }
    CSIM_HD static int clz(uint64_t x) { return hd_clz64(x); }
};
template <>
struct WordTraits<uint32_t> {
    static constexpr int bits = 32;
    CSIM_HD static int popc(uint32_t x) {
#if defined(__CUDA_ARCH__)
        return __popc(x);
#else
        return __builtin_popcount(x);
#endif
    }
    CSIM_HD static int ffs(uint32_t x) {
#if defined(__CUDA_ARCH__)
        return __ffs((int)x);
#else
        return __builtin_ffs((int)x);
#endif
    }
    CSIM_HD static int clz(uint32_t x) {
#if defined(__CUDA_ARCH__)
        return __clz((int)x);
#else
        return x ? __builtin_clz(x) : 32;
#endif
    }
};

template <class W>
CSIM_HD inline W wbit(int i) {
    return (W)1 << i;
}
template <class W>
CSIM_HD inline W wlow(int k) {
    return k >= WordTraits<W>::bits ? (W)~(W)0 : (W)(((W)1 << k) - (W)1);
}
template <class W>
CSIM_HD inline int wget(W w, int i) {
    return (int)((w >> i) & (W)1);
}
template <class W>
CSIM_HD inline W wmask(bool b) {  // all ones if b
    return (W)0 - (W)(b ? 1 : 0);
}
// bit reversal, so that a row loop can walk a mask from its top bit down
CSIM_HD inline uint32_t wbrev(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __brev(x);
#else
    uint32_t r = 0;
    for (int i = 0; i < 32; i++) r |= ((x >> i) & 1u) << (31 - i);
    return r;
#endif
}
CSIM_HD inline uint64_t wbrev(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __brevll(x);
#else
    return ((uint64_t)wbrev((uint32_t)x) << 32) | wbrev((uint32_t)(x >> 32));
#endif
}
// all ones if the top bit of x is set (an arithmetic shift)
CSIM_HD inline uint32_t topmask(uint32_t x) { return (uint32_t)((int32_t)x >> 31); }
CSIM_HD inline uint64_t topmask(uint64_t x) { return (uint64_t)((int64_t)x >> 63); }

struct PairRegs {
    int k, Q;
    uint64_t h;       // h at the codeword's zero positions, compact (bit j = j-th zero, descending)
    uint64_t D1, D2;  // row space (k bits)
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

// one row of the shrink's rank-two update + bit move (see tp_shrink)
template <class W>
CSIM_HD inline W shrink_row(W r, W Ji, W U, W mi, W bu, W bc, W bj) {
    r ^= Ji & bu;
    r ^= U & bc;
    return (r & ~mi) | (mi & bj);
}

// Shrink by e_q (alpha = 0), stabilizer.c:500-585, for a symmetric J.
// The zero columns of the pair's codeword are kept compact, in the order they
// are shrunk by (descending q): slot j of sGT holds column q_j of G as a row
// mask and bit j of s.h holds h's bit q_j; no other column or bit of h is
// read again.  This shrinks by slot `q`; slots q+1..nz-1 are the columns of
// the later shrinks.  `act`: this lane has a shrink to do.  Returns 0 EMPTY,
// 1 SAME, 2 SUCCESS (1 when inactive).  All lanes must call it together.
//
// With R = I + U e_i^T (U = S \ {i}, i = max S) and J symmetric,
//   R J R^T = J + U Ji^T + Ji U^T + J_ii U U^T,
// i.e. row x gets Ji if x in U and U if x in C = Ji ^ (J_ii ? U : 0); then
// basis vectors i and kk = k-1 swap and kk is dropped: row kk moves to slot
// i and every row's bit i becomes its old bit kk = bit x of row kk.  The +4
// corrections of updateDJ are U & Ji, and updateQD's J.y is column kk of the
// result, i.e. C with bit i taken from bit kk of C.
template <class W>
CSIM_HD inline int tp_shrink(PairRegs& s, uint64_t* sJ, uint64_t* sGT, int st, int q, int nz, bool act) {
    using T = WordTraits<W>;
    const int k = s.k;
    const W km = wlow<W>(k);
    const W S = act ? ((W)RG(q) & km) : (W)0;
    const int beta = act ? getbit(s.h, q) : 0;
    const bool upd = S != (W)0;
    const int i = upd ? T::bits - 1 - T::clz(S) : 0;
    const W U = S & ~wbit<W>(i);
    const int kk = k - 1;
    const W mi = wbit<W>(i), mk = wbit<W>(kk & (T::bits - 1));

    // G, column form: rows in U get the pivot row, row kk moves to slot i;
    // h gets the pivot row when beta = 1 (stabilizer.c:530-533, 557, 569-573)
    const int nrem = upd ? nz - 1 - q : 0;
    const int NR = uniform_max(nrem);
    uint64_t hflip = 0ull;
    for (int t = 0; t < NR; t++) {
        if (t < nrem) {
            const int c = q + 1 + t;
            W g = (W)RG(c);
            const bool gi = (g & mi) != (W)0;
            g ^= U & wmask<W>(gi);
            g = (g & ~mi) | (mi & wmask<W>((g & mk) != (W)0));
            RG(c) = (uint64_t)g;
            if (gi) hflip |= bit1(c);
        }
    }
    if (beta) s.h ^= hflip;

    // J: rank-two update, then the i <-> kk swap and drop of kk.  In 64-bit
    // mode rows below 32 keep only their low halves current: bit y >= 32 of
    // row x < 32 is bit x of row y (J is symmetric), which rows >= 32 carry in
    // full, so row i's high half is gathered from them when i < 32.
    W Ji = upd ? (W)RJ(i) : (W)0;
    if (sizeof(W) == 8 && upd && i < 32) {
        uint64_t hi = 0ull;
        for (int y = 32; y < k; y++) hi |= (uint64_t)((RJ(y) >> i) & 1ull) << (y - 32);
        Ji = (W)(((uint64_t)(uint32_t)Ji) | (hi << 32));
    }
    const W C = Ji ^ (wget<W>(Ji, i) ? U : (W)0);  // new row (and column) i
    const W Jk = upd ? (W)((W)RJ(kk) ^ (wget<W>(C, kk) ? U : (W)0)) : (W)0;  // new row kk (kk not in U)
    // every row of the lane's block is rewritten (rows i and kk get values that are
    // replaced or dropped just below), so the pass is branch-free; rows at or
    // beyond k are outside the block and never read again
    const int KX = uniform_max(upd ? k : 0);
    if (upd) {
        // two rows per 16-byte access (the pair buffer holds an even number of rows);
        // the coefficient masks walk bit-reversed copies from the top bit down
        const W ru = wbrev(U), rc = wbrev(C), rj = wbrev(Jk);
        int x0 = 0;
        if (sizeof(W) == 8) {
            // rows below 32: 32-bit arithmetic on the low halves; bit i moves only
            // when i < 32 (a high bit of such a row is stale and never read)
            const uint32_t Ji32 = (uint32_t)Ji, U32 = (uint32_t)U, mi32 = i < 32 ? (uint32_t)mi : 0u;
            uint32_t cu = (uint32_t)((uint64_t)ru >> 32), cc = (uint32_t)((uint64_t)rc >> 32),
                     cj = (uint32_t)((uint64_t)rj >> 32);
            const int K32 = KX < 32 ? KX : 32;
#if defined(__CUDA_ARCH__)
#pragma unroll 2
#endif
            for (int x = 0; x < K32; x += 2) {
                U64x2* pr = reinterpret_cast<U64x2*>(&RJ(x));
                U64x2 v = *pr;
                v.a = shrink_row<uint32_t>((uint32_t)v.a, Ji32, U32, mi32, topmask(cu), topmask(cc), topmask(cj));
                cu <<= 1;
                cc <<= 1;
                cj <<= 1;
                v.b = shrink_row<uint32_t>((uint32_t)v.b, Ji32, U32, mi32, topmask(cu), topmask(cc), topmask(cj));
                cu <<= 1;
                cc <<= 1;
                cj <<= 1;
                *pr = v;
            }
            x0 = 32;
        }
        W cu = ru << (x0 & (T::bits - 1)), cc = rc << (x0 & (T::bits - 1)), cj = rj << (x0 & (T::bits - 1));
#if defined(__CUDA_ARCH__)
#pragma unroll 2
#endif
        for (int x = x0; x < KX; x += 2) {
            U64x2* pr = reinterpret_cast<U64x2*>(&RJ(x));
            U64x2 v = *pr;
            v.a = (uint64_t)shrink_row<W>((W)v.a, Ji, U, mi, topmask(cu), topmask(cc), topmask(cj));
            cu <<= 1;
            cc <<= 1;
            cj <<= 1;
            v.b = (uint64_t)shrink_row<W>((W)v.b, Ji, U, mi, topmask(cu), topmask(cc), topmask(cj));
            cu <<= 1;
            cc <<= 1;
            cj <<= 1;
            *pr = v;
        }
    }
    if (upd && i != kk) RJ(i) = (uint64_t)((Jk & ~mi) | (mi & wmask<W>(wget<W>(Jk, kk))));
    if (upd) {
        // D: eq. 49 and the lower-triangle parities (J[max][min] = Ji by symmetry)
        tp_add_D(s, (uint64_t)U, getbit(s.D1, i), getbit(s.D2, i));
        s.D2 ^= (uint64_t)(U & Ji);
        if (i != kk) {
            s.D1 = swapbits(s.D1, i, kk);
            s.D2 = swapbits(s.D2, i, kk);
        }
        s.D1 &= lowmask(k);
        s.D2 &= lowmask(k);
        if (beta) {
            s.Q = (s.Q + tp_getD(s, kk)) % 8;
            s.D2 ^= (uint64_t)(((C & ~mi) | (mi & wmask<W>(wget<W>(C, kk)))) & wlow<W>(kk));
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
template <class W>
CSIM_HD inline void tp_exp_sum(PairRegs& s, uint64_t* sJ, int st, bool act, int& eps, int& p, int& m, int& err) {
    using T = WordTraits<W>;
    const int k = act ? s.k : 0;
    const W km = wlow<W>(k);
    const W Sm = (W)s.D1 & km;
    int sidx = -1;
    {
        // R = I + U e_a^T, then swap a <-> kk (stabilizer.c:317-336); kk may lie in U
        const bool upd = Sm != (W)0;
        const int a = upd ? T::ffs(Sm) - 1 : 0;
        const W U = Sm & ~wbit<W>(a);
        const int kk = k - 1;
        const W Ja = upd ? (W)RJ(a) : (W)0;
        const W C = Ja ^ (wget<W>(Ja, a) ? U : (W)0);  // new row/column a
        const W Jk = upd ? (W)((W)RJ(kk) ^ (wget<W>(U, kk) ? Ja : (W)0) ^ (wget<W>(C, kk) ? U : (W)0)) : (W)0;
        const int KX = uniform_max(upd ? k : 0);
        if (upd) {
            // rows a and kk are rewritten below; the pass itself is branch-free
            const W ma = wbit<W>(a), mk = wbit<W>(kk & (T::bits - 1));
            W cu = wbrev(U), cc = wbrev(C), cj = wbrev(Jk);
            for (int x = 0; x < KX; x++) {
                W r = (W)RJ(x);
                const W bc = topmask(cc);
                r ^= Ja & topmask(cu);
                r ^= U & bc;
                // swap bits a and kk: bit a <- J'[x][kk] = bit x of Jk, bit kk <- J'[x][a] = bit x of C
                r = (r & ~(ma | mk)) | (ma & topmask(cj)) | (mk & bc);
                RJ(x) = (uint64_t)r;
                cu <<= 1;
                cc <<= 1;
                cj <<= 1;
            }
        }
        if (upd && a != kk) {
            RJ(a) = (uint64_t)(W)swapbits((uint64_t)Jk, a, kk);
            RJ(kk) = (uint64_t)(W)swapbits((uint64_t)C, a, kk);
        } else if (upd) {
            RJ(a) = (uint64_t)C;
        }
        if (upd) {
            tp_add_D(s, (uint64_t)U, getbit(s.D1, a), getbit(s.D2, a));
            s.D2 ^= (uint64_t)(U & Ja);
            s.D1 = swapbits(s.D1, a, kk) & lowmask(k);
            s.D2 = swapbits(s.D2, a, kk) & lowmask(k);
            sidx = kk;
        }
    }
    W E = km & ~(sidx >= 0 ? wbit<W>(sidx) : (W)0);
    WAcc w0 = {0, 0, 0}, w1 = {0, 0, 0};
    const bool any = E != (W)0;
    const int NE = uniform_max(T::popc(E));
    for (int it = 0; it < NE; it++) {
        const bool live = E != (W)0;
        const int a = live ? T::ffs(E) - 1 : 0;
        const W ra = live ? (W)RJ(a) : (W)0;
        const W K = ra & E & ~wbit<W>(a);
        const bool dimer = K != (W)0;
        const int b = dimer ? T::ffs(K) - 1 : 0;
        const W rb = dimer ? (W)RJ(b) : (W)0;
        if (live && !dimer) {  // monomer {a}: row a is final
            const int Da = tp_getD(s, a);
            tp_factor_mono(w0, Da, err);
            if (sidx >= 0) tp_factor_mono(w1, Da + 4 * wget<W>(ra, sidx), err);
        }
        if (dimer) {  // dimer {a, b}: rows a and b are final
            const int Da = tp_getD(s, a), Db = tp_getD(s, b);
            tp_factor_dimer(w0, Da, Db, err);
            if (sidx >= 0) tp_factor_dimer(w1, Da + 4 * wget<W>(ra, sidx), Db + 4 * wget<W>(rb, sidx), err);
        }
        const W Ep = dimer ? (E & ~wbit<W>(a) & ~wbit<W>(b)) : (E & ~wbit<W>(a));
        const W vb = dimer ? (ra & Ep) : (W)0, va = dimer ? (rb & Ep) : (W)0;
        const bool upd = (vb | va) != (W)0;
        // R = I + vb e_b^T + va e_a^T on the rows still in play (Ep):
        //   row x += vb_x Jb + va_x Ja + Cb_x vb + Ca_x va, with the coefficient
        //   columns Cb = (RJ)[.][b], Ca = (RJ)[.][a] (symmetric J)
        const int jaa = wget<W>(ra, a), jbb = wget<W>(rb, b), jab = wget<W>(ra, b);
        const W Cb = rb ^ (jbb ? vb : (W)0) ^ (jab ? va : (W)0);
        const W Ca = ra ^ (jab ? vb : (W)0) ^ (jaa ? va : (W)0);
        const int np = upd ? T::popc(Ep) : 0;
        const int NP = uniform_max(np);
        W zz = Ep;
        for (int t = 0; t < NP; t++) {
            if (t < np) {
                const int x = T::ffs(zz) - 1;
                zz &= zz - 1;
                W r = (W)RJ(x);
                r ^= rb & wmask<W>(wget<W>(vb, x));
                r ^= ra & wmask<W>(wget<W>(va, x));
                r ^= vb & wmask<W>(wget<W>(Cb, x));
                r ^= va & wmask<W>(wget<W>(Ca, x));
                RJ(x) = (uint64_t)r;
            }
        }
        if (upd) {
            const int db1 = getbit(s.D1, b), db2 = getbit(s.D2, b), da1 = getbit(s.D1, a), da2 = getbit(s.D2, a);
            tp_add_D(s, (uint64_t)vb, db1, db2);
            tp_add_D(s, (uint64_t)va, da1, da2);
            W flip = (vb & rb) ^ (va & ra);
            if (jab) flip ^= vb & va;
            s.D2 ^= (uint64_t)flip;
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
// working memory sJ/sGT (stride st), n indices each (sJ an even number).
// J must be symmetric.  `valid` = this lane has a pair (all lanes of a warp
// call together).  The row arithmetic is 64-bit while the warp's largest k
// exceeds 32 and 32-bit after that.
CSIM_HD inline void pair_l(bool valid, int n, int k1, int Q, uint64_t h, uint64_t D1, uint64_t D2, const uint64_t* pJ,
                           const uint64_t* pGT, uint64_t x, uint64_t* sJ, uint64_t* sGT, int st, int& eps, int& p,
                           int& m, int& err, int gmax = 64) {
    // sGT has gmax slots: a codeword with more zeros is refused (the caller
    // bounds the zeros of the codewords it passes)
    if (valid && hd_popc64(~x & lowmask(n)) > gmax) {
        err |= kErrRange;
        valid = false;
    }
    PairRegs s;
    s.k = k1;
    s.Q = Q;
    s.h = h;
    s.D1 = D1;
    s.D2 = D2;
    if (valid)
        for (int r = 0; r < k1; r += 2) {
            U64x2 v;
            v.a = pJ[r];
            v.b = pJ[r + 1];
            *reinterpret_cast<U64x2*>(&RJ(r)) = v;
        }
    // the zero columns of x, descending (the order of the shrinks), compact
    int nz = 0;
    uint64_t hz = 0ull;
    for (uint64_t zz = valid ? (~x & lowmask(n)) : 0ull; zz; nz++) {
        const int c = 63 - hd_clz64(zz);
        zz &= ~bit1(c);
        RG(nz) = pGT[c];
        hz |= (uint64_t)getbit(h, c) << nz;
    }
    s.h = hz;
    eps = 0;
    p = 0;
    m = 0;
    bool alive = valid;
    const int NZ = uniform_max(nz);
    for (int it = 0; it < NZ; it++) {
        const bool act = alive && it < nz;
        const bool wide = uniform_max(alive ? s.k : 0) > CSIM_TP_WIDE_FROM;
        const int r = wide ? tp_shrink<uint64_t>(s, sJ, sGT, st, it, nz, act)
                           : tp_shrink<uint32_t>(s, sJ, sGT, st, it, nz, act);
        if (act && r == 0) alive = false;
    }
    if (uniform_max(alive ? s.k : 0) > CSIM_TP_WIDE_FROM) {
        // the 64-bit exponential sum reads whole rows: rebuild the high halves
        // of rows below 32 from the rows >= 32 (J symmetric)
        if (alive && s.k > 32)
            for (int x = 0; x < 32; x++) {
                uint64_t hi = 0ull;
                for (int y = 32; y < s.k; y++) hi |= (uint64_t)((RJ(y) >> x) & 1ull) << (y - 32);
                RJ(x) = (uint64_t)(uint32_t)RJ(x) | (hi << 32);
            }
        tp_exp_sum<uint64_t>(s, sJ, st, alive, eps, p, m, err);
    } else {
        tp_exp_sum<uint32_t>(s, sJ, st, alive, eps, p, m, err);
    }
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
