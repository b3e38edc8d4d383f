// csim_pair_core.cuh — one (theta, prepL term) pair, the body of the
// thread-per-pair kernels (csim_terms_tp.cu, csim_batch_kernels.cu), written
// once for the device and the host: the same functions are compiled into a
// host-side checker (tests/native/tp_host_check.cpp) that the CPU tests
// compare with the oracle.
//
// The pair's J rows and G columns live in caller-provided memory (PairMem)
// with stride `st` 16-byte units between consecutive indices (the kernels'
// shared-memory [index][thread] layout; 1 on the host).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define CSIM_HD __host__ __device__
#define CSIM_HD_INLINE __host__ __device__ __forceinline__
#else
#define CSIM_HD
#define CSIM_HD_INLINE inline
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

// Per-pair working memory, laid out [index][thread] (consecutive indices of
// one lane are `st` 16-byte units apart, so every access is conflict-free for
// whole units):
//   j32  rows 0..31 of J, low 32 bits, four rows per 16-byte unit;
//   j64  rows 32.. of J, all 64 bits, two rows per 16-byte unit;
//   g    the G columns of the codeword's zero positions, one 64-bit slot each.
// Rows below 32 keep only their low halves: bit y >= 32 of such a row is bit
// r of row y (J is symmetric), which the rows >= 32 carry in full; read_row
// gathers it when a whole row is needed.  While k <= 32 (the narrow mode)
// only j32 is used.
struct PairMem {
    uint32_t* j32;
    uint64_t* j64;
    uint64_t* g;
    int st;
};
// Bytes of a block's working memory for `threads` lanes, and lane `lane`'s
// view of it: j32 (32 rows), then j64 (rows 32..nmax-1, an even count), then
// gmax G-column slots, each [index][thread].
CSIM_HD inline size_t pair_mem_bytes(int nmax, int gmax, int threads) {
    const int n64 = nmax > 32 ? (((nmax + 1) & ~1) - 32) : 0;
    return (size_t)threads * (32 * 4 + (size_t)n64 * 8 + (size_t)gmax * 8);
}
CSIM_HD inline PairMem pair_mem(unsigned char* base, int nmax, int threads, int lane) {
    const int n64 = nmax > 32 ? (((nmax + 1) & ~1) - 32) : 0;
    uint32_t* j32 = reinterpret_cast<uint32_t*>(base);
    uint64_t* j64 = reinterpret_cast<uint64_t*>(base + (size_t)threads * 32 * 4);
    uint64_t* g = j64 + (size_t)n64 * threads;
    return PairMem{j32 + 4 * lane, j64 + 2 * lane, g + lane, threads};
}

#define R32(r) M.j32[(size_t)((r) >> 2) * 4 * M.st + ((r) & 3)]
#define R64(r) M.j64[(size_t)(((r) - 32) >> 1) * 2 * M.st + (((r) - 32) & 1)]
#define RG(c) M.g[(size_t)(c) * M.st]

// 64-bit row arithmetic while the warp's largest k exceeds this.  Builds of
// the host checker set it to 0 to run the 64-bit code on every pair, as a
// lane with k <= 32 does in a warp that still has a larger k.
#ifndef CSIM_TP_WIDE_FROM
#define CSIM_TP_WIDE_FROM 32
#endif

struct alignas(16) U64x2 {
    uint64_t a, b;
};
struct alignas(16) U32x4 {
    uint32_t a, b, c, d;
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
// The row masks of a 16-byte unit of four rows: m[i] = topmask(c << i), i < 4.  On the
// GPU one multiply puts bit 31 - i of c at the sign bit of byte 3 - i (copies of the top
// nibble at bits 7, 14, 21, 28, which do not overlap), and one prmt per row replicates
// that byte's sign over the word: one logic op per row instead of two shifts.
CSIM_HD inline void unit_masks(uint32_t c, uint32_t (&m)[4]) {
#ifdef __CUDA_ARCH__
    const uint32_t s = (c >> 28) * 0x10204080u;
    asm("prmt.b32 %0, %1, 0, 0xBBBB;" : "=r"(m[0]) : "r"(s));
    asm("prmt.b32 %0, %1, 0, 0xAAAA;" : "=r"(m[1]) : "r"(s));
    asm("prmt.b32 %0, %1, 0, 0x9999;" : "=r"(m[2]) : "r"(s));
    asm("prmt.b32 %0, %1, 0, 0x8888;" : "=r"(m[3]) : "r"(s));
#else
    for (int i = 0; i < 4; i++) m[i] = topmask(c << i);
#endif
}

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
CSIM_HD inline bool uniform_any(bool v) {
#if defined(__CUDA_ARCH__)
    return __any_sync(0xffffffffu, v) != 0;
#else
    return v;
#endif
}
CSIM_HD inline int uniform_min(int v) {
#if defined(__CUDA_ARCH__)
    return (int)__reduce_min_sync(0xffffffffu, (unsigned)v);
#else
    return v;
#endif
}

// D = 2 (2 D2 + D1) per basis vector; adding u to D row-wise (eq. 49), with the carry
// into D2, on D words of the mode's width (in 32-bit mode k <= 32, so D fits)
template <class W>
CSIM_HD inline void add_D(W& D1, W& D2, W u, int d1, int d2) {
    const W a1 = d1 ? u : (W)0, a2 = d2 ? u : (W)0;
    const W carry = D1 & a1;
    D1 ^= a1;
    D2 ^= a2 ^ carry;
}
template <class W>
CSIM_HD inline int get_D(W D1, W D2, int i) {
    return 2 * (2 * wget<W>(D2, i) + wget<W>(D1, i));
}
template <class W>
CSIM_HD inline W wswap(W w, int i, int j) {
    const W t = ((w >> i) ^ (w >> j)) & (W)1;
    return w ^ ((t << i) | (t << j));
}

// bits 32..k-1 of row r < 32, i.e. bit r of rows 32..k-1
CSIM_HD inline uint64_t gather_hi(const PairMem& M, int r, int k) {
    uint64_t hi = 0ull;
    for (int y = 32; y < k; y++) hi |= ((R64(y) >> r) & 1ull) << (y - 32);
    return hi;
}

// whole row r of J (narrow mode: r < 32 and k <= 32)
template <class W>
CSIM_HD inline W read_row(const PairMem& M, int r, int k) {
    if (sizeof(W) == 4) return (W)R32(r);
    if (r >= 32) return (W)R64(r);
    return (W)((uint64_t)R32(r) | (gather_hi(M, r, k) << 32));
}

// stores row r (a row below 32 keeps its low half)
template <class W>
CSIM_HD inline void write_row(const PairMem& M, int r, W v) {
    if (sizeof(W) == 8 && r >= 32) R64(r) = (uint64_t)v;  // narrow mode: every row is below 32
    else R32(r) = (uint32_t)v;
}

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
CSIM_HD inline int tp_shrink(PairRegs& s, const PairMem& M, int q, int nz, bool act) {
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

    // J: rank-two update, then the i <-> kk swap and drop of kk
    const W Ji = upd ? read_row<W>(M, i, k) : (W)0;
    const W C = Ji ^ (wget<W>(Ji, i) ? U : (W)0);  // new row (and column) i
    const W Jk = upd ? (W)(read_row<W>(M, kk, k) ^ (wget<W>(C, kk) ? U : (W)0)) : (W)0;  // new row kk (kk not in U)
    // every row of the lane's block is rewritten (rows i and kk get values that are
    // replaced or dropped just below), so the pass is branch-free; rows at or
    // beyond k are outside the block and never read again.  The coefficient
    // masks walk bit-reversed copies from the top bit down.
    const int KX = uniform_max(upd ? k : 0);
    if (upd) {
        const W ru = wbrev(U), rc = wbrev(C), rj = wbrev(Jk);
        // rows below 32, four per 16-byte unit, 32-bit; bit i moves only when
        // i < 32 (a high bit of such a row is not stored)
        {
            const uint32_t Ji32 = (uint32_t)Ji, U32 = (uint32_t)U, mi32 = i < 32 ? (uint32_t)mi : 0u;
            const int sh = T::bits - 32;
            uint32_t cu = (uint32_t)(ru >> sh), cc = (uint32_t)(rc >> sh), cj = (uint32_t)(rj >> sh);
            const int K32 = KX < 32 ? KX : 32;
            for (int x = 0; x < K32; x += 4) {
                U32x4* pr = reinterpret_cast<U32x4*>(&R32(x));
                U32x4 v = *pr;
                v.a = shrink_row<uint32_t>(v.a, Ji32, U32, mi32, topmask(cu), topmask(cc), topmask(cj));
                v.b = shrink_row<uint32_t>(v.b, Ji32, U32, mi32, topmask(cu << 1), topmask(cc << 1), topmask(cj << 1));
                v.c = shrink_row<uint32_t>(v.c, Ji32, U32, mi32, topmask(cu << 2), topmask(cc << 2), topmask(cj << 2));
                v.d = shrink_row<uint32_t>(v.d, Ji32, U32, mi32, topmask(cu << 3), topmask(cc << 3), topmask(cj << 3));
                cu <<= 4;
                cc <<= 4;
                cj <<= 4;
                *pr = v;
            }
        }
        // rows 32.. (64-bit mode only), two per 16-byte unit
        if (sizeof(W) == 8) {
            W cu = (W)((uint64_t)ru << 32), cc = (W)((uint64_t)rc << 32), cj = (W)((uint64_t)rj << 32);
            for (int x = 32; x < KX; x += 2) {
                U64x2* pr = reinterpret_cast<U64x2*>(&R64(x));
                U64x2 v = *pr;
                v.a = (uint64_t)shrink_row<W>((W)v.a, Ji, U, mi, topmask(cu), topmask(cc), topmask(cj));
                v.b = (uint64_t)shrink_row<W>((W)v.b, Ji, U, mi, topmask((W)(cu << 1)), topmask((W)(cc << 1)),
                                              topmask((W)(cj << 1)));
                cu <<= 2;
                cc <<= 2;
                cj <<= 2;
                *pr = v;
            }
        }
    }
    if (upd && i != kk) write_row<W>(M, i, (Jk & ~mi) | (mi & wmask<W>(wget<W>(Jk, kk))));
    if (upd) {
        // D: eq. 49 and the lower-triangle parities (J[max][min] = Ji by symmetry)
        W D1 = (W)s.D1, D2 = (W)s.D2;
        add_D<W>(D1, D2, U, wget<W>(D1, i), wget<W>(D2, i));
        D2 ^= U & Ji;
        if (i != kk) {
            D1 = wswap<W>(D1, i, kk);
            D2 = wswap<W>(D2, i, kk);
        }
        D1 &= km;
        D2 &= km;
        if (beta) {
            s.Q = (s.Q + get_D<W>(D1, D2, kk)) % 8;
            D2 ^= ((C & ~mi) | (mi & wmask<W>(wget<W>(C, kk)))) & wlow<W>(kk);
        } else {
            s.Q = s.Q % 8;
        }
        s.D1 = (uint64_t)D1;
        s.D2 = (uint64_t)D2;
        s.k = kk;
        return 2;
    }
    return act ? 1 - beta : 1;
}

// W0/W1 accumulators of Wsigma (stabilizer.c:258-297)
struct WAcc {
    int zero, p, m;
};

// gamma_ab for every A = 2a, B = 2b (a, b mod 4) as one 4-bit code per (a, b)
// at bits 4(4a + b): bit 3 set = zero, else bits 0..2 = m (and p = 2).  Built
// at compile time from the same sums as gamma_ab.
constexpr uint64_t gamma_codes() {
    uint64_t tab = 0;
    for (int a = 0; a < 4; a++)
        for (int b = 0; b < 4; b++) {
            const int c = (a + b) % 4;
            const int gr = 1 + ((a == 0) - (a == 2)) + ((b == 0) - (b == 2)) - ((c == 0) - (c == 2));
            const int gi = ((a == 1) - (a == 3)) + ((b == 1) - (b == 3)) - ((c == 1) - (c == 3));
            int code = 0;
            if (gr == 0 && gi == 0) code = 8;
            else if (gr == 0) code = gi > 0 ? 2 : 6;
            else if (gr == -2) code = 4;
            else if (gi == 2) code = 1;
            else if (gi == 0) code = 0;
            else code = 7;
            tab |= (uint64_t)code << (4 * (4 * a + b));
        }
    return tab;
}
constexpr uint64_t kGammaCodes = gamma_codes();

// one monomer factor partialGamma(A) = 1 + e^{i pi A/4}, A even: r = A mod 8 gives
// 2^{2/2} w^0 (r = 0), 2^{1/2} w^1 (2), 0 (4), 2^{1/2} w^7 (6)
CSIM_HD inline void tp_factor_mono(WAcc& w, int A, int& err) {
    const int r = A & 7;
    if (r & 1) err |= kErrGamma;
    w.zero |= (r == 4);
    w.p += r == 0 ? 2 : (r == 4 ? 0 : 1);
    w.m += r == 2 ? 1 : (r == 6 ? 7 : 0);
}

// one dimer factor Gamma(A, B), A and B even and non-negative (kGammaCodes)
CSIM_HD inline void tp_factor_dimer(WAcc& w, int A, int B, int& err) {
    if (((A | B) & 1) || A < 0 || B < 0) err |= kErrGamma;
    const int idx = 4 * ((A & 7) >> 1) + ((B & 7) >> 1);
    const uint32_t half = (idx & 8) ? (uint32_t)(kGammaCodes >> 32) : (uint32_t)kGammaCodes;
    const int code = (int)((half >> (4 * (idx & 7))) & 15u);
    const int z = code >> 3;
    w.zero |= z;
    w.p += z ? 0 : 2;
    w.m += z ? 0 : (code & 7);
}

// exponentialSumExact (stabilizer.c:300-481), symmetric J; `act` as for tp_shrink.
template <class W>
CSIM_HD inline void tp_exp_sum(PairRegs& s, const PairMem& M, bool act, int& eps, int& p, int& m, int& err) {
    using T = WordTraits<W>;
    const int k = act ? s.k : 0;
    const W km = wlow<W>(k);
    W D1 = (W)s.D1, D2 = (W)s.D2;
    const W Sm = D1 & km;
    int sidx = -1;
    {
        // R = I + U e_a^T, then swap a <-> kk (stabilizer.c:317-336); kk may lie in U
        const bool upd = Sm != (W)0;
        const int a = upd ? T::ffs(Sm) - 1 : 0;
        const W U = Sm & ~wbit<W>(a);
        const int kk = k - 1;
        const W Ja = upd ? read_row<W>(M, a, k) : (W)0;
        const W C = Ja ^ (wget<W>(Ja, a) ? U : (W)0);  // new row/column a
        const W Jk =
            upd ? (W)(read_row<W>(M, kk, k) ^ (wget<W>(U, kk) ? Ja : (W)0) ^ (wget<W>(C, kk) ? U : (W)0)) : (W)0;
        const int KX = uniform_max(upd ? k : 0);
        if (upd) {
            // every row: rank-two update, then bit a <- J'[x][kk] = bit x of Jk and
            // bit kk <- J'[x][a] = bit x of C (rows a and kk are rewritten below)
            const W ma = wbit<W>(a), mk = wbit<W>(kk & (T::bits - 1));
            const W ru = wbrev(U), rc = wbrev(C), rj = wbrev(Jk);
            {
                const uint32_t Ja32 = (uint32_t)Ja, U32 = (uint32_t)U;
                const uint32_t ma32 = a < 32 ? (uint32_t)ma : 0u, mk32 = kk < 32 ? (uint32_t)mk : 0u;
                const int sh = T::bits - 32;
                uint32_t cu = (uint32_t)(ru >> sh), cc = (uint32_t)(rc >> sh), cj = (uint32_t)(rj >> sh);
                const int K32 = KX < 32 ? KX : 32;
                for (int x = 0; x < K32; x++) {
                    uint32_t r = R32(x);
                    const uint32_t bc = topmask(cc);
                    r ^= Ja32 & topmask(cu);
                    r ^= U32 & bc;
                    r = (r & ~(ma32 | mk32)) | (ma32 & topmask(cj)) | (mk32 & bc);
                    R32(x) = r;
                    cu <<= 1;
                    cc <<= 1;
                    cj <<= 1;
                }
            }
            if (sizeof(W) == 8) {
                W cu = (W)((uint64_t)ru << 32), cc = (W)((uint64_t)rc << 32), cj = (W)((uint64_t)rj << 32);
                for (int x = 32; x < KX; x++) {
                    W r = (W)R64(x);
                    const W bc = topmask(cc);
                    r ^= Ja & topmask(cu);
                    r ^= U & bc;
                    r = (r & ~(ma | mk)) | (ma & topmask(cj)) | (mk & bc);
                    R64(x) = (uint64_t)r;
                    cu <<= 1;
                    cc <<= 1;
                    cj <<= 1;
                }
            }
        }
        if (upd && a != kk) {
            write_row<W>(M, a, wswap<W>(Jk, a, kk));
            write_row<W>(M, kk, wswap<W>(C, a, kk));
        } else if (upd) {
            write_row<W>(M, a, C);
        }
        if (upd) {
            add_D<W>(D1, D2, U, wget<W>(D1, a), wget<W>(D2, a));
            D2 ^= U & Ja;
            D1 = wswap<W>(D1, a, kk) & km;
            D2 = wswap<W>(D2, a, kk) & km;
            sidx = kk;
        }
    }
    W E = km & ~(sidx >= 0 ? wbit<W>(sidx) : (W)0);
    // rows updated in each pass besides those still in play: in 64-bit mode
    // the row sidx >= 32, whose bits give the bit sidx of rows below 32
    const W keep = (sizeof(W) == 8 && sidx >= 32) ? wbit<W>(sidx) : (W)0;
    WAcc w0 = {0, 0, 0}, w1 = {0, 0, 0};
    const bool any = E != (W)0;
    // at most popc(E) steps; a dimer retires two rows, so the warp is usually
    // done well before that, and a step with no lane in play changes nothing
    const int NE = uniform_max(T::popc(E));
    for (int it = 0; it < NE; it++) {
        if (uniform_max(E != (W)0 ? 1 : 0) == 0) break;
        const bool live = E != (W)0;
        const int a = live ? T::ffs(E) - 1 : 0;
        const W ra = live ? read_row<W>(M, a, k) : (W)0;
        const W K = ra & E & ~wbit<W>(a);
        const bool dimer = K != (W)0;
        const int b = dimer ? T::ffs(K) - 1 : 0;
        const W rb = dimer ? read_row<W>(M, b, k) : (W)0;
        if (live && !dimer) {  // monomer {a}: row a is final
            const int Da = get_D<W>(D1, D2, a);
            tp_factor_mono(w0, Da, err);
            if (sidx >= 0) tp_factor_mono(w1, Da + 4 * wget<W>(ra, sidx), err);
        }
        if (dimer) {  // dimer {a, b}: rows a and b are final
            const int Da = get_D<W>(D1, D2, a), Db = get_D<W>(D1, D2, b);
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
        {
            // every row from the warp's lowest row in play up to its highest: rows
            // below 32 four per 16-byte unit in 32-bit, rows from 32 up two per unit
            // in 64-bit; coefficient masks by sign shift.  A row outside Ep gets
            // vb_x = va_x = 0, i.e. at most its own update of the columns in vb
            // and va: such rows (finished rows, a, b, rows at or beyond k) are
            // never read again, and the row sidx kept for 64-bit mode is updated
            // as it should be.
            const W zm = upd ? (Ep | keep) : (W)0;
            const int lo = zm ? T::ffs(zm) - 1 : T::bits, hi = zm ? T::bits - T::clz(zm) : 0;
            const int X0 = uniform_min(lo) & ~3, X1 = uniform_max(hi);
            const W rvb = wbrev(vb), rva = wbrev(va), rcb = wbrev(Cb), rca = wbrev(Ca);
            {
                const int sh = T::bits - 32;
                const int s0 = X0 < 32 ? X0 : 0;
                const uint32_t rb32 = (uint32_t)rb, ra32 = (uint32_t)ra, vb32 = (uint32_t)vb, va32 = (uint32_t)va;
                uint32_t cvb = (uint32_t)(rvb >> sh) << s0, cva = (uint32_t)(rva >> sh) << s0,
                         ccb = (uint32_t)(rcb >> sh) << s0, cca = (uint32_t)(rca >> sh) << s0;
                const int X1a = X1 < 32 ? X1 : 32;
                for (int x = X0; x < X1a; x += 4) {
                    U32x4* pr = reinterpret_cast<U32x4*>(&R32(x));
                    U32x4 v = *pr;
                    v.a ^= (rb32 & topmask(cvb)) ^ (ra32 & topmask(cva)) ^ (vb32 & topmask(ccb)) ^
                           (va32 & topmask(cca));
                    v.b ^= (rb32 & topmask(cvb << 1)) ^ (ra32 & topmask(cva << 1)) ^ (vb32 & topmask(ccb << 1)) ^
                           (va32 & topmask(cca << 1));
                    v.c ^= (rb32 & topmask(cvb << 2)) ^ (ra32 & topmask(cva << 2)) ^ (vb32 & topmask(ccb << 2)) ^
                           (va32 & topmask(cca << 2));
                    v.d ^= (rb32 & topmask(cvb << 3)) ^ (ra32 & topmask(cva << 3)) ^ (vb32 & topmask(ccb << 3)) ^
                           (va32 & topmask(cca << 3));
                    cvb <<= 4;
                    cva <<= 4;
                    ccb <<= 4;
                    cca <<= 4;
                    *pr = v;
                }
            }
            if (sizeof(W) == 8) {
                const int x0 = X0 > 32 ? (X0 & ~1) : 32;
                const int s1 = x0 & (T::bits - 1);
                W cvb = rvb << s1, cva = rva << s1, ccb = rcb << s1, cca = rca << s1;
                for (int x = x0; x < X1; x += 2) {
                    U64x2* pr = reinterpret_cast<U64x2*>(&R64(x));
                    U64x2 v = *pr;
                    v.a ^= (uint64_t)((rb & topmask(cvb)) ^ (ra & topmask(cva)) ^ (vb & topmask(ccb)) ^
                                      (va & topmask(cca)));
                    v.b ^= (uint64_t)((rb & topmask((W)(cvb << 1))) ^ (ra & topmask((W)(cva << 1))) ^
                                      (vb & topmask((W)(ccb << 1))) ^ (va & topmask((W)(cca << 1))));
                    cvb <<= 2;
                    cva <<= 2;
                    ccb <<= 2;
                    cca <<= 2;
                    *pr = v;
                }
            }
        }
        if (upd) {
            const int db1 = wget<W>(D1, b), db2 = wget<W>(D2, b), da1 = wget<W>(D1, a), da2 = wget<W>(D2, a);
            add_D<W>(D1, D2, vb, db1, db2);
            add_D<W>(D1, D2, va, da1, da2);
            W flip = (vb & rb) ^ (va & ra);
            if (jab) flip ^= vb & va;
            D2 ^= flip;
        }
        if (live) E = Ep;
    }
    if (!act) return;
    if (k == 0) {  // Wsigma's k == 0 case
        eps = 1; p = 0; m = s.Q;
        return;
    }
    // W0 = Wsigma(sigma = 0), W1 = Wsigma(sigma = 1) (stabilizer.c:425-479)
    const int tM0 = s.Q, tM1 = s.Q + (sidx >= 0 ? get_D<W>(D1, D2, sidx) : 0);
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

// The part of a pair after its start state is in M and s: the shrinks by the
// nz zero columns in M's slots (descending positions), then the exponential
// sum; p is corrected by theta's own k (k0) and the weight of x, as
// innerProductExact's p - k1 - k2 (stabilizer.c:659).  All lanes of a warp call
// it together; `valid` = this lane has a pair.
CSIM_HD inline void pair_finish(PairRegs& s, int nz, bool valid, const PairMem& M, uint64_t x, int k0, int& eps,
                                int& p, int& m, int& err) {
    eps = 0;
    p = 0;
    m = 0;
    bool alive = valid;
    const int NZ = uniform_max(nz);
    for (int it = 0; it < NZ; it++) {
        const bool act = alive && it < nz;
        const bool wide = uniform_max(alive ? s.k : 0) > CSIM_TP_WIDE_FROM;
        const int r = wide ? tp_shrink<uint64_t>(s, M, it, nz, act) : tp_shrink<uint32_t>(s, M, it, nz, act);
        if (act && r == 0) alive = false;
    }
    if (uniform_max(alive ? s.k : 0) > CSIM_TP_WIDE_FROM) tp_exp_sum<uint64_t>(s, M, alive, eps, p, m, err);
    else tp_exp_sum<uint32_t>(s, M, alive, eps, p, m, err);
    if (alive) p -= k0 + hd_popc64(x);
    else {
        eps = 0;
        p = 0;
        m = 0;
    }
}

// One pair: theta's J rows and G columns (as row masks), codeword x; working
// memory M (see PairMem: 32 rows in j32, rows 32..n-1 in j64, gmax G-column
// slots).  J must be symmetric.  `valid` = this lane has a pair (all lanes of
// a warp call together).  The row arithmetic is 64-bit while the warp's
// largest k exceeds 32 and 32-bit after that.
//
// `done`: top bits of [0, n) whose shrinks the state passed in has already
// been through (prefix_shrink); the state's k is then k1 and theta's own is
// k0.  Without them (done = 0, k0 < 0) the state is theta's.
CSIM_HD inline void pair_l(bool valid, int n, int k1, int Q, uint64_t h, uint64_t D1, uint64_t D2, const uint64_t* pJ,
                           const uint64_t* pGT, uint64_t x, const PairMem& M, int& eps, int& p, int& m, int& err,
                           int gmax = 64, uint64_t done = 0ull, int k0 = -1) {
    const uint64_t zeros_all = ~x & lowmask(n) & ~done;
    // the G-column slots hold gmax columns: a codeword with more zeros is
    // refused (the caller bounds the zeros of the codewords it passes)
    if (valid && hd_popc64(zeros_all) > gmax) {
        err |= kErrRange;
        valid = false;
    }
    PairRegs s;
    s.k = k1;
    s.Q = Q;
    s.h = h;
    s.D1 = D1;
    s.D2 = D2;
    if (valid) {
        for (int r = 0; r < k1 && r < 32; r++) R32(r) = (uint32_t)pJ[r];
        for (int r = 32; r < k1; r++) R64(r) = pJ[r];
    }
    // the zero columns of x, descending (the order of the shrinks), compact
    int nz = 0;
    uint64_t hz = 0ull;
    for (uint64_t zz = valid ? zeros_all : 0ull; zz; nz++) {
        const int c = 63 - hd_clz64(zz);
        zz &= ~bit1(c);
        RG(nz) = pGT[c];
        hz |= (uint64_t)getbit(h, c) << nz;
    }
    s.h = hz;
    pair_finish(s, nz, valid, M, x, k0 < 0 ? k1 : k0, eps, p, m, err);
}

// The shrinks that every pair of theta with a codeword that agrees with x0 on
// the top bits `pm` of [0, n) starts with: those by the zero bits of x0 in
// pm, in descending order, as pair_l runs them.  In: theta's J rows pJ, G
// columns pGT (row masks), h, D1, D2, Q, k.  Out, in place: the state after
// those shrinks, with the G columns and h bits of the positions below pm (J
// rows and G columns masked to the new k).  Returns 0 if a shrink found the
// projection empty (every such pair is then 0), else 1.  Every lane of one
// warp calls it; the `act` lanes (up to two per warp, each with its own group
// state pJ/pGT and its own working memory M with room for 64 G columns) do
// the work, and only they write.
CSIM_HD inline int prefix_shrink(bool act, int n, uint64_t pm, uint64_t x0, int& k, int& Q, uint64_t& h,
                                 uint64_t& D1, uint64_t& D2, uint64_t* pJ, uint64_t* pGT, const PairMem& M) {
    const uint64_t pz = act ? (~x0 & pm & lowmask(n)) : 0ull;
    const int npz = hd_popc64(pz);
    const int nlow = hd_popc64(lowmask(n) & ~pm);  // pm is a top mask: positions 0..nlow-1 stay
    PairRegs s;
    s.k = k;
    s.Q = Q;
    s.D1 = D1;
    s.D2 = D2;
    int nslot = 0;
    uint64_t hz = 0ull;
    if (act) {
        for (int r = 0; r < k && r < 32; r++) R32(r) = (uint32_t)pJ[r];
        for (int r = 32; r < k; r++) R64(r) = pJ[r];
        // slots: the prefix zeros (the shrinks here), then every position below pm
        for (uint64_t zz = pz; zz; nslot++) {
            const int c = 63 - hd_clz64(zz);
            zz &= ~bit1(c);
            RG(nslot) = pGT[c];
            hz |= (uint64_t)getbit(h, c) << nslot;
        }
        for (int c = nlow - 1; c >= 0; c--, nslot++) {
            RG(nslot) = pGT[c];
            hz |= (uint64_t)getbit(h, c) << nslot;
        }
    }
    s.h = hz;
    bool alive = act;
    const int NQ = uniform_max(npz);
    for (int q = 0; q < NQ; q++) {
        const bool a = alive && q < npz;
        const bool wide = uniform_max(a ? s.k : 0) > CSIM_TP_WIDE_FROM;
        const int r = wide ? tp_shrink<uint64_t>(s, M, q, nslot, a) : tp_shrink<uint32_t>(s, M, q, nslot, a);
        if (a && r == 0) alive = false;
    }
    if (!act) return 1;
    if (!alive) return 0;
    const int k2 = s.k;
    const uint64_t km = lowmask(k2);
    for (int r = 0; r < k2; r++) pJ[r] = read_row<uint64_t>(M, r, k2) & km;
    uint64_t h2 = 0ull;
    for (int c = 0; c < n; c++) {
        if (c < nlow) {
            const int slot = npz + nlow - 1 - c;
            pGT[c] = RG(slot) & km;
            h2 |= (uint64_t)getbit(s.h, slot) << c;
        } else {
            pGT[c] = 0ull;  // a prefix position: no pair shrinks by it again
        }
    }
    k = k2;
    Q = s.Q;
    h = h2;
    D1 = s.D1;
    D2 = s.D2;
    return 1;
}

// ---------------------------------------------------------------- per-thread runs
// A thread that takes a run of codewords agreeing on the top bits pm of
// [0, n) runs the shrinks by their common zeros in pm once (run_prefix) and
// starts each of its pairs from that state (pair_from_run).  The state lives
// in the thread's run memory RS: a PairMem with a G slot for every position
// (the kernel keeps it in global memory; the host checker on the stack).
struct RunState {
    int k, Q, alive, npz, nlow, pad;
    uint64_t h;  // h at the slots (bit s = slot s)
    uint64_t D1, D2;
    uint64_t pm;  // the run's agreed top bits, whose shrinks are done
};

#define S32(r) RS.j32[(size_t)((r) >> 2) * 4 * RS.st + ((r) & 3)]
#define S64(r) RS.j64[(size_t)(((r) - 32) >> 1) * 2 * RS.st + (((r) - 32) & 1)]
#define SG(c) RS.g[(size_t)(c) * RS.st]

// Loads theta (J rows pJ, G columns pGT as row masks, scalars) into RS with
// the slots laid out as prefix_shrink lays them: the zeros of x0 in pm
// (descending), then every position below pm (descending, position c at slot
// npz + nlow - 1 - c), and runs the shrinks by those zeros: the shrinks every
// pair of the run starts with, in the order pair_l runs them.  Every lane of a
// warp calls it; `act` = this lane has a run.  out.alive = 0 if a shrink
// found the projection empty (every pair of the run is then 0).
CSIM_HD inline void run_prefix(bool act, int n, uint64_t pm, uint64_t x0, int k, int Q, uint64_t h, uint64_t D1,
                               uint64_t D2, const uint64_t* pJ, const uint64_t* pGT, const PairMem& RS, RunState& out) {
    const uint64_t pz = act ? (~x0 & pm & lowmask(n)) : 0ull;
    const int npz = hd_popc64(pz);
    const int nlow = hd_popc64(lowmask(n) & ~pm);
    PairRegs s;
    s.k = k;
    s.Q = Q;
    s.D1 = D1;
    s.D2 = D2;
    int nslot = 0;
    uint64_t hz = 0ull;
    if (act) {
        for (int r = 0; r < k && r < 32; r++) S32(r) = (uint32_t)pJ[r];
        for (int r = 32; r < k; r++) S64(r) = pJ[r];
        for (uint64_t zz = pz; zz; nslot++) {
            const int c = 63 - hd_clz64(zz);
            zz &= ~bit1(c);
            SG(nslot) = pGT[c];
            hz |= (uint64_t)getbit(h, c) << nslot;
        }
        for (int c = nlow - 1; c >= 0; c--, nslot++) {
            SG(nslot) = pGT[c];
            hz |= (uint64_t)getbit(h, c) << nslot;
        }
    }
    s.h = hz;
    bool alive = act;
    const int NQ = uniform_max(npz);
    for (int q = 0; q < NQ; q++) {
        const bool a = alive && q < npz;
        const bool wide = uniform_max(a ? s.k : 0) > CSIM_TP_WIDE_FROM;
        const int r = wide ? tp_shrink<uint64_t>(s, RS, q, nslot, a) : tp_shrink<uint32_t>(s, RS, q, nslot, a);
        if (a && r == 0) alive = false;
    }
    out.k = s.k;
    out.Q = s.Q;
    out.alive = alive ? 1 : 0;
    out.npz = npz;
    out.nlow = nlow;
    out.pad = 0;
    out.h = s.h;
    out.D1 = s.D1;
    out.D2 = s.D2;
    out.pm = pm;
}

// One pair of a run: the run's state (rs, RS) copied into the pair's working
// memory M -- J rows, and the G columns and h bits of x's zeros below the
// run's prefix, in descending order -- then pair_finish.  k0: theta's own k.
// Same (eps, p, m) as pair_l on theta.  All lanes of a warp call it together.
CSIM_HD inline void pair_from_run(bool valid, int n, const RunState& rs, const PairMem& RS, uint64_t x,
                                  const PairMem& M, int& eps, int& p, int& m, int& err, int gmax, int k0) {
    const uint64_t zeros = ~x & lowmask(n) & ~rs.pm;
    if (valid && hd_popc64(zeros) > gmax) {
        err |= kErrRange;
        valid = false;
    }
    valid = valid && rs.alive;
    PairRegs s;
    s.k = rs.k;
    s.Q = rs.Q;
    s.D1 = rs.D1;
    s.D2 = rs.D2;
    // J rows, whole 16-byte units: four 32-bit rows below 32, two 64-bit rows from 32 up
    const int K = uniform_max(valid ? s.k : 0);
    const int u32 = ((K < 32 ? K : 32) + 3) / 4, u64 = K > 32 ? (K - 32 + 1) / 2 : 0;
    for (int u = 0; u < u32; u++)
        if (valid && 4 * u < s.k)
            *reinterpret_cast<U32x4*>(&R32(4 * u)) = *reinterpret_cast<const U32x4*>(&S32(4 * u));
    for (int u = 0; u < u64; u++)
        if (valid && 32 + 2 * u < s.k)
            *reinterpret_cast<U64x2*>(&R64(32 + 2 * u)) = *reinterpret_cast<const U64x2*>(&S64(32 + 2 * u));
    int nz = 0;
    uint64_t hz = 0ull;
    const int base = rs.npz + rs.nlow - 1;
    for (uint64_t zz = valid ? zeros : 0ull; zz; nz++) {
        const int c = 63 - hd_clz64(zz);
        zz &= ~bit1(c);
        RG(nz) = SG(base - c);
        hz |= (uint64_t)getbit(rs.h, base - c) << nz;
    }
    s.h = hz;
    pair_finish(s, nz, valid, M, x, k0, eps, p, m, err);
}

#undef S32
#undef S64
#undef SG

// ---------------------------------------------------------------- direct restriction
// <theta|phi_x> = 2^{-(k + |x|)/2} sum over {u : h + uG has no 1 outside x} of
// w^{q(u)}: an exponential sum of theta's form over the u whose image vanishes
// on x's zero positions.  canon_theta rewrites theta once so that its
// variables are k pivot coordinates P of the affine space (the image is
// y_P = v, the other coordinates affine in v), the form re-expressed in v by
// the same elementary substitutions the reference's basis changes make
// (stabilizer.c:129-177).  A pair then needs no shrink for a zero of x at a
// pivot coordinate: that variable is simply absent.  Only the zeros of x at
// the d = n - k non-pivot coordinates are constraints (md_shrink), after which
// the form over the remaining variables goes to the exponential sum
// (md_exp_sum).  Both run on rows indexed by variable under a live mask F;
// pair_direct first renumbers x's live variables 0..f-1 (direct_compact).
// The result is the same complex number as innerProductExact's; eps and p are
// equal, m is equal mod 8 (the reference's unreduced m depends on its basis).
// CSIM_COUNT_ROWS(r): the direct path touched r rows of J or constraint
// masks for one pair (each row read, copied or updated once).  A host build
// that measures the path's work per pair defines it; it is empty otherwise.
#ifndef CSIM_COUNT_ROWS
#define CSIM_COUNT_ROWS(r) ((void)0)
#endif

struct Canon {
    uint64_t P;       // pivot coordinates: the variables
    uint64_t D1, D2;  // the form's D, at each variable's coordinate
    uint64_t bm;      // right-hand side bit of each non-pivot coordinate's constraint
    int Q, k, n, pad;
};

// A state's pivot form as the direct kernels read it (canon_theta): the
// scalars, each coordinate's J row and each non-pivot coordinate's variables.
struct CanonG {
    Canon cs;
    uint64_t Jc[64];
    uint64_t acol[64];
};

// (D1, D2) += (d1, d2) on the bits of u, with the carry into D2 (D = 2 (2 D2 + D1) mod 8)
CSIM_HD inline void add_D64(uint64_t& D1, uint64_t& D2, uint64_t u, int d1, int d2) {
    const uint64_t a1 = d1 ? u : 0ull, a2 = d2 ? u : 0ull, c = D1 & a1;
    D1 ^= a1;
    D2 ^= a2 ^ c;
}
// the same in the words of the exponential sum's mode
template <class W>
CSIM_HD_INLINE void add_Dw(W& D1, W& D2, W u, int d1, int d2) {
    const W a1 = d1 ? u : (W)0, a2 = d2 ? u : (W)0, c = D1 & a1;
    D1 ^= a1;
    D2 ^= a2 ^ c;
}

// theta (n qubits, k, Q, h, D1, D2, G rows, J rows as in csim_state) in pivot
// coordinates.  Jc[c], acol[c] for c < n: J row of variable c (0 for a
// non-pivot c), and for a non-pivot c the mask of variables its coordinate
// depends on (0 for a pivot).  Sequential (one thread); run once per theta.
CSIM_HD inline void canon_theta(int n, int k, int Q, uint64_t h, uint64_t D1, uint64_t D2, const uint64_t* G,
                                const uint64_t* J, uint64_t* Jc, uint64_t* acol, Canon& out) {
    const uint64_t nm = lowmask(n), km = lowmask(k);
    uint64_t g[64], Jv[64];
    int piv[64];
    D1 &= km;
    D2 &= km;
    for (int a = 0; a < k; a++) {
        g[a] = G[a] & nm;
        Jv[a] = J[a] & km;
    }
    // Gauss-Jordan on the rows of G.  Row b += row a is the substitution
    // u_a = u'_a + u'_b; all rows b of a pivot step at once form the rank-two
    // update R J R^T with U = B (rows in B get J_a, rows in C get B), with
    // D_b += D_a + 4 J_ab (tp_shrink's update without the swap).
    for (int a = 0; a < k; a++) {
        const int pc = g[a] ? hd_ffs64(g[a]) - 1 : 0;
        piv[a] = pc;
        uint64_t B = 0ull;
        for (int b = 0; b < k; b++)
            if (b != a && getbit(g[b], pc)) B |= bit1(b);
        if (!B) continue;
        for (int b = 0; b < k; b++)
            if (getbit(B, b)) g[b] ^= g[a];
        const uint64_t Ja = Jv[a], C = Ja ^ (getbit(Ja, a) ? B : 0ull);
        for (int x = 0; x < k; x++) Jv[x] ^= (getbit(B, x) ? Ja : 0ull) ^ (getbit(C, x) ? B : 0ull);
        add_D64(D1, D2, B, getbit(D1, a), getbit(D2, a));
        D2 ^= B & Ja;
    }
    // shift v = u + w, w_a = h at a's pivot, so that y_{piv a} = v_a
    uint64_t wv = 0ull;
    for (int a = 0; a < k; a++)
        if (getbit(h, piv[a])) {
            wv |= bit1(a);
            Q = (Q + 2 * (2 * getbit(D2, a) + getbit(D1, a))) & 7;
            D2 ^= (uint64_t)getbit(D1, a) << a;  // D_a -> -D_a
            D2 ^= Jv[a] & ~bit1(a) & km;          // D_b += 4 J_ab
        }
    // to coordinate indexing
    uint64_t P = 0ull;
    for (int a = 0; a < k; a++) P |= bit1(piv[a]);
    auto map = [&](uint64_t v) {
        uint64_t r = 0ull;
        for (int a = 0; a < k; a++)
            if (getbit(v, a)) r |= bit1(piv[a]);
        return r;
    };
    for (int c = 0; c < 64; c++) {
        Jc[c] = 0ull;
        acol[c] = 0ull;
    }
    for (int a = 0; a < k; a++) Jc[piv[a]] = map(Jv[a]);
    uint64_t bm = 0ull;
    for (int c = 0; c < n; c++) {
        if (getbit(P, c)) continue;
        uint64_t av = 0ull;
        for (int a = 0; a < k; a++)
            if (getbit(g[a], c)) av |= bit1(a);
        acol[c] = map(av);
        if ((getbit(h, c) ^ (hd_popc64(wv & av) & 1)) != 0) bm |= bit1(c);
    }
    out.P = P;
    out.D1 = map(D1);
    out.D2 = map(D2);
    out.bm = bm;
    out.Q = Q;
    out.k = k;
    out.n = n;
    out.pad = 0;
}

// whole row r of J with F-indexed rows (rows below 32 keep their low halves;
// bit y >= 32 of such a row is bit r of row y, for y < KP)
template <class W>
CSIM_HD inline W md_read_row(const PairMem& M, int r, int KP) {
    if (sizeof(W) == 4) return (W)R32(r);
    if (r >= 32) return (W)R64(r);
    return (W)((uint64_t)R32(r) | (gather_hi(M, r, KP) << 32));
}

// Rows [0, KX) of J: row x ^= (U_x ? Ji : 0) ^ (C_x ? U : 0), the rank-two
// update R J R^T of the substitution of variable i, rows below 32 in 32 bits
template <class W>
CSIM_HD inline void md_rank2(const PairMem& M, int KX, W Ji, W U, W C) {
    using T = WordTraits<W>;
    const W ru = wbrev(U), rc = wbrev(C);
    {
        const uint32_t Ji32 = (uint32_t)Ji, U32 = (uint32_t)U;
        const int sh = T::bits - 32;
        uint32_t cu = (uint32_t)(ru >> sh), cc = (uint32_t)(rc >> sh);
        const int K32 = KX < 32 ? KX : 32;
        for (int x = 0; x < K32; x += 4) {
            U32x4* pr = reinterpret_cast<U32x4*>(&R32(x));
            U32x4 v = *pr;
            uint32_t mu[4], mc[4];
            unit_masks(cu, mu);
            unit_masks(cc, mc);
            v.a ^= (Ji32 & mu[0]) ^ (U32 & mc[0]);
            v.b ^= (Ji32 & mu[1]) ^ (U32 & mc[1]);
            v.c ^= (Ji32 & mu[2]) ^ (U32 & mc[2]);
            v.d ^= (Ji32 & mu[3]) ^ (U32 & mc[3]);
            cu <<= 4;
            cc <<= 4;
            *pr = v;
        }
    }
    if (sizeof(W) == 8) {
        W cu = (W)((uint64_t)ru << 32), cc = (W)((uint64_t)rc << 32);
        for (int x = 32; x < KX; x += 2) {
            U64x2* pr = reinterpret_cast<U64x2*>(&R64(x));
            U64x2 v = *pr;
            v.a ^= (uint64_t)((Ji & topmask(cu)) ^ (U & topmask(cc)));
            v.b ^= (uint64_t)((Ji & topmask((W)(cu << 1))) ^ (U & topmask((W)(cc << 1))));
            cu <<= 2;
            cc <<= 2;
            *pr = v;
        }
    }
}

// One constraint (slot q of M's G slots: a mask of variables, right-hand side
// bit q of s.h): sum over its live variables of v = rhs.  Substitutes its
// highest live variable i by the others (rows of J, D, and the later slots'
// masks and right-hand sides), adds the shift when rhs = 1, and drops i from
// F.  Returns 0 EMPTY (no live variable, rhs 1), 1 SAME (none, rhs 0), 2
// SUCCESS; 1 when inactive.  All lanes of a warp call it together.
template <class W>
CSIM_HD inline int md_shrink(PairRegs& s, uint64_t& F, const PairMem& M, int q, int nz, bool act) {
    using T = WordTraits<W>;
    const W S = act ? (W)(RG(q) & F) : (W)0;
    const int beta = act ? getbit(s.h, q) : 0;
    const bool upd = S != (W)0;
    const int i = upd ? T::bits - 1 - T::clz(S) : 0;
    const W U = S & ~wbit<W>(i);
    const W mi = wbit<W>(i);
    const int KP = upd ? 64 - hd_clz64(F) : 0;
    // later constraints: a_c += (a_c)_i U; rhs_c += (a_c)_i rhs
    const int nrem = upd ? nz - 1 - q : 0;
    const int NR = uniform_max(nrem);
    uint64_t hflip = 0ull;
    for (int t = 0; t < NR; t++) {
        if (t < nrem) {
            const int c = q + 1 + t;
            uint64_t g = RG(c);
            const bool gi = getbit(g, i) != 0;
            g ^= (uint64_t)U & (gi ? ~0ull : 0ull);
            RG(c) = g;
            if (gi) hflip |= bit1(c);
        }
    }
    if (beta) s.h ^= hflip;
    const W Ji = upd ? md_read_row<W>(M, i, KP) : (W)0;
    const W C = Ji ^ (wget<W>(Ji, i) ? U : (W)0);  // new row (and column) i
    const int KX = uniform_max(KP);
    if (upd) CSIM_COUNT_ROWS(nrem + 1 + KP);
    if (upd) md_rank2<W>(M, KX, Ji, U, C);
    if (upd) {
        uint64_t D1 = s.D1, D2 = s.D2;
        add_D64(D1, D2, (uint64_t)U, getbit(D1, i), getbit(D2, i));
        D2 ^= (uint64_t)(U & Ji);
        if (beta) {
            s.Q = (s.Q + 2 * (2 * getbit(D2, i) + getbit(D1, i))) & 7;
            D2 ^= (uint64_t)C & F & ~(uint64_t)mi;
        }
        s.D1 = D1;
        s.D2 = D2;
        F &= ~(uint64_t)mi;
        return 2;
    }
    return act ? 1 - beta : 1;
}
// The factors md_exp_sum's elimination has folded into W0 and W1 (bit 0 and
// bit 1 of `zero` and `m4`).  Every variable it eliminates has D/2 even (the
// first substitution leaves D1 only at sidx, and no step changes D1), so D is
// 4 D2 there, and 4 (D2 ^ J_x,sidx) in W1's form.  A monomer factor
// 1 + w^D is then 2 or 0 and a dimer factor Gamma is 2 or -2: each step adds
// 2 to p, a monomer with D = 4 makes the sum zero and a dimer with both D = 4
// adds 4 to m.
struct MdAcc {
    int zero, m4, steps;
};

// One step of md_exp_sum's elimination: the monomer or dimer of the highest
// row in E, its factors folded into w, the rest of E updated.  E and keep are
// carried in 64-bit words between steps, so the sum can go on in 32-bit words
// once no lane has a row in play at or above 32.
template <class W>
CSIM_HD_INLINE void md_exp_step(const PairMem& M, uint64_t& E64, uint64_t keep64, int sidx, W& D2, MdAcc& w) {
    using T = WordTraits<W>;
    W E = (W)E64;
    const W keep = (W)keep64;
    const bool live = E != (W)0;
    const W es = sidx >= 0 ? wbit<W>(sidx) : (W)0;
    const int KP = live ? 64 - hd_clz64((uint64_t)(E | keep | es)) : 0;
    const int a = live ? T::bits - 1 - T::clz(E) : 0;
    const W ra = live ? md_read_row<W>(M, a, KP) : (W)0;
    const W K = ra & E;  // J_aa = D1_a = 0: bit a of row a is clear
    const bool dimer = K != (W)0;
    const int b = dimer ? T::bits - 1 - T::clz(K) : 0;
    const W rb = dimer ? md_read_row<W>(M, b, KP) : (W)0;
    // D2 of a and b in W0's form (bit 0) and W1's (bit 1)
    const int da2 = wget<W>(D2, a), db2 = dimer ? wget<W>(D2, b) : 0;
    const int fa = (da2 ? 3 : 0) ^ ((ra & es) != (W)0 ? 2 : 0);
    const int fb = (db2 ? 3 : 0) ^ ((rb & es) != (W)0 ? 2 : 0);
    if (live) {
        w.steps++;
        if (dimer) w.m4 ^= fa & fb;
        else w.zero |= fa;
    }
    const W Ep = dimer ? (E & ~wbit<W>(a) & ~wbit<W>(b)) : (E & ~wbit<W>(a));
    const W vb = dimer ? (ra & Ep) : (W)0, va = dimer ? (rb & Ep) : (W)0;
    const bool upd = (vb | va) != (W)0;
    // Rows a and b are not read again, so only rows x of Ep change, and only in the columns still
    // read (Ep and sidx).  Since J_ab = 1 for a dimer, R J R^T there is the symmetric rank-two
    // update x ^= (vb_x ? Pm : 0) ^ (va_x ? Qm : 0) (vb_x = J_ax, va_x = J_bx), column sidx
    // included through bit sidx of rows a and b.  The full update also adds J_bb vb to Pm and
    // J_aa va to Qm; J's diagonal is D1 (J_xx = D/2 mod 2, kept so by every substitution), which
    // is 0 at a and b.
    const W Pm = va ^ (rb & es);
    const W Qm = vb ^ (ra & es);
    {
        // rows from 0: the warp's lowest row in play is nearly always 0 after the renumbering,
        // and finding it costs more than the rows it would skip
        const W zm = upd ? Ep : (W)0;
        const int hi = zm ? T::bits - T::clz(zm) : 0;
        const int X1 = uniform_max(hi);
        if (live) CSIM_COUNT_ROWS((dimer ? 2 : 1) + (upd ? hi - (T::ffs(zm) - 1) : 0));
        const W rvb = wbrev(vb), rva = wbrev(va);  // row x's bits at bit T::bits - 1 - x
        {
            const int sh = T::bits - 32;
            const uint32_t P32 = (uint32_t)Pm, Q32 = (uint32_t)Qm;
            uint32_t cvb = (uint32_t)(rvb >> sh), cva = (uint32_t)(rva >> sh);
            const int X1a = X1 < 32 ? X1 : 32;
            for (int x = 0; x < X1a; x += 4) {
                U32x4* pr = reinterpret_cast<U32x4*>(&R32(x));
                U32x4 v = *pr;
                uint32_t mb[4], ma[4];
                unit_masks(cvb, mb);
                unit_masks(cva, ma);
                v.a ^= (P32 & mb[0]) ^ (Q32 & ma[0]);
                v.b ^= (P32 & mb[1]) ^ (Q32 & ma[1]);
                v.c ^= (P32 & mb[2]) ^ (Q32 & ma[2]);
                v.d ^= (P32 & mb[3]) ^ (Q32 & ma[3]);
                cvb <<= 4;
                cva <<= 4;
                *pr = v;
            }
        }
        if (sizeof(W) == 8) {
            W cvb = rvb << (32 & (T::bits - 1)), cva = rva << (32 & (T::bits - 1));  // rows from 32
            for (int x = 32; x < X1; x += 2) {
                U64x2* pr = reinterpret_cast<U64x2*>(&R64(x));
                U64x2 v = *pr;
                v.a ^= (uint64_t)((Pm & topmask(cvb)) ^ (Qm & topmask(cva)));
                v.b ^= (uint64_t)((Pm & topmask((W)(cvb << 1))) ^ (Qm & topmask((W)(cva << 1))));
                cvb <<= 2;
                cva <<= 2;
                *pr = v;
            }
            // a row sidx >= 32 holds column sidx of the rows below 32
            if (keep && upd)
                R64(sidx) ^= (uint64_t)((wget<W>(rb, sidx) ? vb : (W)0) ^ (wget<W>(ra, sidx) ? va : (W)0));
        }
    }
    // the dimer's D update of the rows in Ep: D1 is zero at a and b, so only D2 changes, and the
    // full update's terms vb & rb and va & ra are both ra & rb & Ep, so they cancel
    if (upd) D2 ^= (db2 ? vb : (W)0) ^ (da2 ? va : (W)0) ^ (vb & va);
    if (live) E = Ep;
    E64 = (uint64_t)E;
}

// exponentialSumExact (stabilizer.c:300-481) of the form over the live
// variables F (rows indexed by variable, F marking the live ones): first the
// substitution that leaves one variable (sidx, the lowest with D odd) with D
// odd, then monomers and dimers taken from the highest live row down, so the
// rows still in play shrink towards row 0.  W0/W1 and their combination as in
// tp_exp_sum.  `act` as for md_shrink.
template <class W>
CSIM_HD inline void md_exp_sum(PairRegs& s, const PairMem& M, uint64_t F, bool act, int& eps, int& p, int& m,
                               int& err) {
    using T = WordTraits<W>;
    const W Fw = act ? (W)F : (W)0;
    W D1 = (W)s.D1, D2 = (W)s.D2;  // bits of live variables only (all below 32 in 32-bit mode)
    const W Sm = D1 & Fw;
    int sidx = -1;
    int KP = Fw ? 64 - hd_clz64((uint64_t)Fw) : 0;
    {
        const bool upd = Sm != (W)0;
        const int a = upd ? T::ffs(Sm) - 1 : 0;
        const W U = Sm & ~wbit<W>(a);
        const W Ja = upd ? md_read_row<W>(M, a, KP) : (W)0;
        const W C = Ja ^ U;  // J_aa = D1_a = 1 at the substituted variable
        const int KX = uniform_max(upd ? KP : 0);
        if (upd && U != (W)0) md_rank2<W>(M, KX, Ja, U, C);
        if (upd) CSIM_COUNT_ROWS(U != (W)0 ? 1 + KP : 1);
        if (upd) {
            add_Dw<W>(D1, D2, U, wget<W>(D1, a), wget<W>(D2, a));
            D2 ^= U & Ja;
            sidx = a;
        }
    }
    W E = Fw & ~(sidx >= 0 ? wbit<W>(sidx) : (W)0);
    if ((D1 & E) != (W)0) err |= kErrGamma;  // MdAcc's premise
    // in 64-bit mode the row sidx >= 32 stays updated: its bits are bit sidx of the rows below 32
    const W keep = (sizeof(W) == 8 && sidx >= 32) ? wbit<W>(sidx) : (W)0;
    MdAcc acc = {0, 0, 0};
    const bool any = E != (W)0;
    const int NE = uniform_max(T::popc(E));
    uint64_t E64 = (uint64_t)E;
    int it = 0;
    for (; it < NE; it++) {
        if (!uniform_any(E64 != 0ull)) break;
        // rows below 32 alone (and sidx below 32): on in 32-bit words
        if (sizeof(W) == 8 && uniform_max(64 - hd_clz64(E64 | (sidx >= 0 ? bit1(sidx) : 0ull))) <= CSIM_TP_WIDE_FROM)
            break;
        md_exp_step<W>(M, E64, (uint64_t)keep, sidx, D2, acc);
    }
    if (sizeof(W) == 8 && it < NE) {
        // the rest of E and sidx lie below 32 (or E is empty): steps in 32-bit words, which leave
        // the D bits from 32 up as they are
        uint32_t d2 = (uint32_t)D2;
        for (; it < NE; it++) {
            if (!uniform_any(E64 != 0ull)) break;
            md_exp_step<uint32_t>(M, E64, 0ull, sidx, d2, acc);
        }
        D2 = (D2 & ~(W)0xffffffffu) | (W)d2;
    }
    if (!act) return;
    const WAcc w0 = {acc.zero & 1, 2 * acc.steps, 4 * (acc.m4 & 1)};
    const WAcc w1 = {(acc.zero >> 1) & 1, 2 * acc.steps, 4 * ((acc.m4 >> 1) & 1)};
    if (Fw == (W)0) {  // Wsigma's k == 0 case
        eps = 1;
        p = 0;
        m = s.Q;
        return;
    }
    const int tM0 = s.Q, tM1 = s.Q + (sidx >= 0 ? 2 * (2 * wget<W>(D2, sidx) + wget<W>(D1, sidx)) : 0);
    const int e0 = !w0.zero, p0 = w0.zero ? 0 : w0.p, m0 = w0.zero ? 0 : (any ? (tM0 + w0.m) % 8 : tM0);
    if (sidx < 0) {
        eps = e0;
        p = p0;
        m = m0;
        return;
    }
    const int e1 = !w1.zero, p1 = w1.zero ? 0 : w1.p, m1 = w1.zero ? 0 : (any ? (tM1 + w1.m) % 8 : tM1);
    if (e0 == 0) {
        eps = e1;
        p = p1;
        m = m1;
        return;
    }
    if (e1 == 0) {
        eps = e0;
        p = p0;
        m = m0;
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
        p = 0;
        m = 0;
    } else {
        p = pp + p0;
        m = mm + m0 % 8;
    }
}

// The bits of words at the ones of a fixed 32-bit mask m, packed to the low
// end in order: the parallel-suffix compress of Hacker's Delight (Warren,
// 2nd ed., section 7-4).  compress_net computes the move masks of m once;
// compress32 then moves a word's bits right by 1, 2, 4, ...  R rounds move a
// bit by up to 2^R - 1, which is enough when m has no bit at or above 2^R.
struct CompressNet {
    uint32_t m, mv[5];
    uint32_t keep0;  // m & ~mv[0]: the bits of m that stay in round 0
};
template <int R>
CSIM_HD_INLINE CompressNet compress_net(uint32_t m) {
    CompressNet c;
    c.m = m;
    uint32_t mk = ~m << 1;  // ones where the count of zeros to the right changes parity
#pragma unroll
    for (int i = 0; i < R; i++) {
        uint32_t mp = mk ^ (mk << 1);  // prefix parity of mk: the bits that move by 2^i this round
#pragma unroll
        for (int j = 1; j < R; j++) mp ^= mp << (1 << j);
        const uint32_t mv = mp & m;
        c.mv[i] = mv;
        m = (m ^ mv) | (mv >> (1 << i));
        mk &= ~mp;
    }
    c.keep0 = R > 0 ? c.m & ~c.mv[0] : c.m;
    return c;
}
template <int R>
CSIM_HD_INLINE uint32_t compress32(uint32_t x, const CompressNet& c) {
    if (R == 0) return x & c.m;
    // round 0 with the mask by m folded in (mv[0] lies within m)
    x = (x & c.keep0) | ((x & c.mv[0]) >> 1);
#pragma unroll
    for (int i = 1; i < R; i++) {
        const uint32_t t = x & c.mv[i];
        x = (x ^ t) | (t >> (1 << i));
    }
    return x;
}
// x << s within 32 bits, 0 for s == 32
CSIM_HD_INLINE uint32_t shl32_upto32(uint32_t x, int s) {
#if defined(__CUDA_ARCH__)
    return __funnelshift_lc(0u, x, (unsigned)s);
#else
    return s >= 32 ? 0u : x << s;
#endif
}

// Four words' low bytes (kLanes 4: into one word, byte q from word q) or two
// words' low 16-bit halves (kLanes 2: into two words), and back (lane q of
// the packed words, zero-extended).  Byte permutes on the GPU.
template <int kLanes>
CSIM_HD_INLINE void pack_lanes(const uint32_t (&h)[4], uint32_t (&out)[2]) {
#ifdef __CUDA_ARCH__
    if (kLanes == 4) {
        out[0] = __byte_perm(__byte_perm(h[0], h[1], 0x0040), __byte_perm(h[2], h[3], 0x0040), 0x5410);
    } else {
        out[0] = __byte_perm(h[0], h[1], 0x5410);
        out[1] = __byte_perm(h[2], h[3], 0x5410);
    }
#else
    if (kLanes == 4) {
        out[0] = (h[0] & 0xFFu) | ((h[1] & 0xFFu) << 8) | ((h[2] & 0xFFu) << 16) | ((h[3] & 0xFFu) << 24);
    } else {
        out[0] = (h[0] & 0xFFFFu) | (h[1] << 16);
        out[1] = (h[2] & 0xFFFFu) | (h[3] << 16);
    }
#endif
}
template <int kLanes>
CSIM_HD_INLINE uint32_t unpack_lane(const uint32_t (&c)[2], int q) {
#ifdef __CUDA_ARCH__
    if (kLanes == 4) return __byte_perm(c[0], 0u, 0x4440u | (unsigned)q);
    return __byte_perm(c[q >> 1], 0u, (q & 1) ? 0x4432u : 0x4410u);
#else
    if (kLanes == 4) return (c[0] >> (8 * q)) & 0xFFu;
    return (c[q >> 1] >> (16 * (q & 1))) & 0xFFFFu;
#endif
}

// How pair_direct compresses a pair's words, by the warp's live coordinates:
// all below 32 (kCompactLow); some at or above 32 but at most 32 live
// variables in every lane, so every compressed word fits 32 bits
// (kCompactSplit: each half by its own net, the high net with RHI rounds for
// coordinates below 32 + 2^RHI); more than 32 live variables in some lane
// (kCompactWide: 64-bit words, rows from 32 up whole).
enum { kCompactLow = 0, kCompactSplit = 1, kCompactWide = 2 };

template <int MODE, int RHI>
CSIM_HD_INLINE uint64_t compress_word(uint64_t x, const CompressNet& lo, const CompressNet& hi, int plo) {
    const uint32_t l = compress32<5>((uint32_t)x, lo);
    if (MODE == kCompactLow) return l;
    const uint32_t h = compress32<RHI>((uint32_t)(x >> 32), hi);
    if (MODE == kCompactSplit) return l | shl32_upto32(h, plo);
    return l | ((uint64_t)h << plo);
}

// The compacted form of one pair (pair_direct): live variable i is the i-th
// coordinate of F0.  Writes J rows 0..f-1 (rows below 32 as their low halves,
// four to a 16-byte unit; rows from 32 up whole, kCompactWide only), the
// constraint masks of the zeros N at non-pivot coordinates (descending) with
// their right-hand sides in hz, and D.  Rows from f up to the warp's largest
// f, within the last 16-byte unit, get words that no step reads.
template <int MODE, int RHI>
CSIM_HD_INLINE void direct_compact(const Canon& cs, const uint64_t* Jc, const uint64_t* acol, uint64_t F0, int f,
                                   uint64_t N, const PairMem& M, PairRegs& s, int& nz, uint64_t& hz) {
    const CompressNet nlo = compress_net<5>((uint32_t)F0);
    const CompressNet nhi = MODE == kCompactLow ? nlo : compress_net<RHI>((uint32_t)(F0 >> 32));
    const int plo = MODE == kCompactLow ? 0 : WordTraits<uint32_t>::popc((uint32_t)F0);
    s.D1 = compress_word<MODE, RHI>(cs.D1, nlo, nhi, plo);
    s.D2 = compress_word<MODE, RHI>(cs.D2, nlo, nhi, plo);
    const int fmax = uniform_max(f);
    uint32_t rl = (uint32_t)F0, rh = (uint32_t)(F0 >> 32);  // live coordinates not yet taken
    // with at most 8 (RHI 3) or 16 (RHI 4) live high coordinates, the high parts of a unit's
    // rows share compresses, four bytes or two 16-bit halves to a word: the move masks repeated
    // in each lane move every lane's bits within it
    constexpr int kLanes = RHI == 3 ? 4 : (RHI == 4 ? 2 : 1);
    constexpr uint32_t kLaneMask = kLanes == 4 ? 0xFFu : 0xFFFFu;
    constexpr uint32_t kRepeat = kLanes == 4 ? 0x01010101u : 0x00010001u;
    const bool pack = MODE == kCompactSplit && kLanes > 1;
    CompressNet nrep = nhi;
    if (pack) {
        nrep.m = (nhi.m & kLaneMask) * kRepeat;
#pragma unroll
        for (int i = 0; i < RHI && i < 5; i++) nrep.mv[i] = (nhi.mv[i] & kLaneMask) * kRepeat;
        nrep.keep0 = nrep.m & ~nrep.mv[0];
    }
    for (int u = 0; 4 * u < (fmax < 32 ? fmax : 32); u++) {
        uint32_t w[4];
        uint32_t hi[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const bool inlo = MODE == kCompactLow || rl != 0u;
            const int c = inlo ? WordTraits<uint32_t>::ffs(rl) - 1 : 31 + WordTraits<uint32_t>::ffs(rh);
            if (inlo) rl &= rl - 1u;
            else rh &= rh - 1u;
            const uint64_t row = Jc[c & 63];
            if (pack) {
                w[q] = compress32<5>((uint32_t)row, nlo);
                hi[q] = (uint32_t)(row >> 32);
            } else {
                w[q] = (uint32_t)compress_word<MODE, RHI>(row, nlo, nhi, plo);
            }
        }
        if (pack) {
            uint32_t hb[2], hc[2];
            pack_lanes<kLanes>(hi, hb);
#pragma unroll
            for (int g = 0; g < 4 / kLanes; g++) hc[g] = compress32<RHI>(hb[g], nrep);
#pragma unroll
            for (int q = 0; q < 4; q++) w[q] |= shl32_upto32(unpack_lane<kLanes>(hc, q), plo);
        }
        if (4 * u < f) {
            U32x4 v;
            v.a = w[0];
            v.b = w[1];
            v.c = w[2];
            v.d = w[3];
            *reinterpret_cast<U32x4*>(&R32(4 * u)) = v;
        }
    }
    if (MODE == kCompactWide)
        for (int r = 32; r < fmax; r += 2) {  // whole rows from 32 up
            uint64_t w[2];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const bool inlo = rl != 0u;
                const int c = inlo ? WordTraits<uint32_t>::ffs(rl) - 1 : 31 + WordTraits<uint32_t>::ffs(rh);
                if (inlo) rl &= rl - 1u;
                else rh &= rh - 1u;
                w[q] = compress_word<MODE, RHI>(Jc[c & 63], nlo, nhi, plo);
            }
            if (r < f) {
                U64x2 v;
                v.a = w[0];
                v.b = w[1];
                *reinterpret_cast<U64x2*>(&R64(r)) = v;
            }
        }
    CSIM_COUNT_ROWS(f);
    nz = 0;
    hz = 0ull;
    for (uint64_t zz = N; zz; nz++) {
        const int c = 63 - hd_clz64(zz);
        zz &= ~bit1(c);
        RG(nz) = compress_word<MODE, RHI>(acol[c], nlo, nhi, plo);
        hz |= (uint64_t)getbit(cs.bm, c) << nz;
    }
    CSIM_COUNT_ROWS(nz);
}

// One pair by direct restriction: theta in pivot coordinates (cs, Jc rows,
// acol non-pivot masks), codeword x; working memory M with `rows` J rows (at
// least x's live variables) and at least as many G slots as x has zeros at
// non-pivot coordinates (dslots).  The live variables
// F = x & P are renumbered 0..f-1 in coordinate order (rows, their bits, the
// constraint masks and D compressed by F), so the constraints and the
// exponential sum run on f rows with nothing dead in between, in 32-bit words
// while the warp's f stays at or below 32.  The renumbering keeps the order of
// the variables, so each step eliminates the same variable as on coordinate
// indices.  Same eps and p as pair_l, m equal mod 8.  All lanes of a warp call
// it together.
CSIM_HD inline void pair_direct(bool valid, int n, const Canon& cs, const uint64_t* Jc, const uint64_t* acol,
                                uint64_t x, const PairMem& M, int& eps, int& p, int& m, int& err, int dslots, int k0,
                                int rows) {
    const uint64_t nm = lowmask(n);
    const uint64_t N0 = ~x & ~cs.P & nm;
    if (valid && (hd_popc64(N0) > dslots || hd_popc64(x & cs.P) > rows)) {
        err |= kErrRange;
        valid = false;
    }
    const uint64_t F0 = valid ? x & cs.P : 0ull;
    const uint64_t N = valid ? N0 : 0ull;
    const int f = hd_popc64(F0);
    PairRegs s;
    s.k = 0;
    s.Q = cs.Q;
    int nz;
    uint64_t hz;
    // the warp's highest live coordinate (+ 1) and largest live count choose the compress
    const int top = uniform_max(F0 ? 64 - hd_clz64(F0) : 0);
    if (top <= 32) direct_compact<kCompactLow, 0>(cs, Jc, acol, F0, f, N, M, s, nz, hz);
    else if (uniform_max(f) > 32) direct_compact<kCompactWide, 5>(cs, Jc, acol, F0, f, N, M, s, nz, hz);
    else if (top <= 40) direct_compact<kCompactSplit, 3>(cs, Jc, acol, F0, f, N, M, s, nz, hz);
    else if (top <= 48) direct_compact<kCompactSplit, 4>(cs, Jc, acol, F0, f, N, M, s, nz, hz);
    else direct_compact<kCompactSplit, 5>(cs, Jc, acol, F0, f, N, M, s, nz, hz);
    uint64_t F = lowmask(f);
    s.h = hz;
    eps = 0;
    p = 0;
    m = 0;
    bool alive = valid;
    const int NZ = uniform_max(nz);
    for (int it = 0; it < NZ; it++) {
        const bool act = alive && it < nz;
        const bool wide = uniform_max(act && F ? 64 - hd_clz64(F) : 0) > CSIM_TP_WIDE_FROM;
        const int r = wide ? md_shrink<uint64_t>(s, F, M, it, nz, act) : md_shrink<uint32_t>(s, F, M, it, nz, act);
        if (act && r == 0) alive = false;
    }
    const int KF = uniform_max(alive && F ? 64 - hd_clz64(F) : 0);  // highest live coordinate of the warp, + 1
    if (KF > CSIM_TP_WIDE_FROM) md_exp_sum<uint64_t>(s, M, F, alive, eps, p, m, err);
    else md_exp_sum<uint32_t>(s, M, F, alive, eps, p, m, err);
    if (alive) p -= k0 + hd_popc64(x);
    else {
        eps = 0;
        p = 0;
        m = 0;
    }
}

// Top bits of [0, n) on which codewords that differ in the bits `dis` agree
CSIM_HD inline uint64_t agree_top(uint64_t dis, int n) {
    const uint64_t d = dis & lowmask(n);
    return lowmask(n) & ~lowmask(64 - hd_clz64(d));
}

#undef R32
#undef R64
#undef RG

}  // namespace pc
}  // namespace csim
