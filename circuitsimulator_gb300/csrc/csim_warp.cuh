// csim_warp.cuh — warp-cooperative stabilizer-state algebra for sm_103a.
//
// One warp holds one stabilizer state (CircuitSimulator's struct
// StabilizerState, libcirc/stabilizer/stabilizer.h:5-16) with lane l owning
// rows l and l+32 of G, Gbar and J as uint64 words (bit c = column c).  The
// vectors h, D1, D2 and the scalars n, k, Q are warp-uniform.  Rows >= n are
// kept zero.  NR = rows per lane (1 for n <= 32, 2 for n <= 64).
//
// Every routine reproduces the reference's result bit for bit, including
// the parts of the state outside the k x k block, but replaces the
// reference's dense O(n^3) basis change updateDJ (stabilizer.c:129-160) by
// the equivalent O(1)-per-lane update for the elementary matrices R that
// shrink and exponentialSumExact actually use:
//     R = I + u1 e_c1^T + u2 e_c2^T   (pivot columns c1, c2 not in u1, u2)
// and row/column swaps.  Over GF(2) the composite of shrink's |S|-1
// successive updateDJ calls (stabilizer.c:540-545) equals one such R with
// u1 = S \ {i}, c1 = i, and the +4 corrections D2[a] ^= J[max(a,i)][min(a,i)]
// read entries no earlier step changes, so the result is identical.
#pragma once

#include <cstdint>

namespace csim {

constexpr unsigned kFull = 0xffffffffu;

// device error flags (OR-ed into the per-launch error word)
enum : int {
    kErrRange = 1,        // p or k outside the range a normalized state allows
    kErrReplay = 2,       // a replayed state needed more rand() words than given
    kErrExpSum = 4,       // exponentialSumExact's "p0 != p1" / "odd m1-m0" branch
    kErrGamma = 8,        // partialGamma/Gamma given an odd argument (reference asserts)
    kErrArg = 16,         // bad per-item argument (n out of range ...)
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint64_t bit1(int i) { return 1ull << i; }
__device__ __forceinline__ uint64_t lowmask(int k) { return k >= 64 ? ~0ull : ((1ull << k) - 1ull); }
__device__ __forceinline__ int getbit(uint64_t w, int i) { return (int)((w >> i) & 1ull); }
__device__ __forceinline__ int par64(uint64_t w) { return __popcll(w) & 1; }
__device__ __forceinline__ uint64_t swapbits(uint64_t w, int i, int j) {
    const uint64_t t = ((w >> i) ^ (w >> j)) & 1ull;
    return w ^ ((t << i) | (t << j));
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
    const uint32_t lo = __shfl_sync(kFull, (uint32_t)v, src);
    const uint32_t hi = __shfl_sync(kFull, (uint32_t)(v >> 32), src);
    return ((uint64_t)hi << 32) | lo;
}

__device__ __forceinline__ uint64_t shfl_xor64(uint64_t v, int m) {
    const uint32_t lo = __shfl_xor_sync(kFull, (uint32_t)v, m);
    const uint32_t hi = __shfl_xor_sync(kFull, (uint32_t)(v >> 32), m);
    return ((uint64_t)hi << 32) | lo;
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// ------------------------------------------------------------------ state
template <int NR>
struct WS {
    int n, k, Q;
    uint64_t h, D1, D2;
    uint64_t G[NR], B[NR], J[NR];  // B = Gbar
};

template <int NR>
__device__ __forceinline__ int row_of(int slot) {
    return lane_id() + 32 * slot;
}

// broadcast row idx (uniform) of a lane-distributed matrix
template <int NR>
__device__ __forceinline__ uint64_t row_get(const uint64_t (&m)[NR], int idx) {
    uint64_t v = m[0];
    if constexpr (NR == 2) v = (idx >= 32) ? m[1] : m[0];
    return shfl64(v, idx & 31);
}

template <int NR>
__device__ __forceinline__ void row_set(uint64_t (&m)[NR], int idx, uint64_t v) {
    if ((idx & 31) == lane_id()) {
        if constexpr (NR == 2) {
            if (idx >= 32) m[1] = v;
            else m[0] = v;
        } else {
            m[0] = v;
        }
    }
}

template <int NR>
__device__ __forceinline__ void row_swap(uint64_t (&m)[NR], int i, int j) {
    if (i == j) return;
    const uint64_t ri = row_get<NR>(m, i), rj = row_get<NR>(m, j);
    row_set<NR>(m, i, rj);
    row_set<NR>(m, j, ri);
}

// mask over rows x: bit c of row x
template <int NR>
__device__ __forceinline__ uint64_t ballot_bit(const uint64_t (&m)[NR], int c) {
    uint64_t r = __ballot_sync(kFull, (unsigned)((m[0] >> c) & 1ull));
    if constexpr (NR == 2) r |= (uint64_t)__ballot_sync(kFull, (unsigned)((m[1] >> c) & 1ull)) << 32;
    return r;
}

// mask over rows x: parity(row_x & v)
template <int NR>
__device__ __forceinline__ uint64_t ballot_par(const uint64_t (&m)[NR], uint64_t v) {
    uint64_t r = __ballot_sync(kFull, (unsigned)par64(m[0] & v));
    if constexpr (NR == 2) r |= (uint64_t)__ballot_sync(kFull, (unsigned)par64(m[1] & v)) << 32;
    return r;
}

// XOR of the rows selected by mask
template <int NR>
__device__ __forceinline__ uint64_t xor_rows(const uint64_t (&m)[NR], uint64_t mask) {
    const int l = lane_id();
    uint64_t acc = getbit(mask, l) ? m[0] : 0ull;
    if constexpr (NR == 2) acc ^= getbit(mask, l + 32) ? m[1] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc ^= shfl_xor64(acc, o);
    return acc;
}

template <int NR>
__device__ __forceinline__ uint64_t ballot_i(int pred0, int pred1) {
    uint64_t r = __ballot_sync(kFull, (unsigned)pred0);
    if constexpr (NR == 2) r |= (uint64_t)__ballot_sync(kFull, (unsigned)pred1) << 32;
    return r;
}

template <int NR>
__device__ __forceinline__ bool any_row_nonzero(const uint64_t (&m)[NR]) {
    uint64_t v = m[0];
    if constexpr (NR == 2) v |= m[1];
    return __any_sync(kFull, v != 0ull) != 0;
}

template <int NR>
__device__ __forceinline__ int getD(const WS<NR>& s, int i) {
    return 2 * (2 * getbit(s.D2, i) + getbit(s.D1, i));
}

// setD (stabilizer.c:59-62) stores (val/2) mod 4 with C truncating division
template <int NR>
__device__ __forceinline__ void setD(WS<NR>& s, int i, int val) {
    const int v2 = val / 2;
    const int d1 = (v2 % 2) & 1;
    const int d2 = (((v2 - v2 % 2) / 2) % 2) & 1;
    s.D1 = (s.D1 & ~bit1(i)) | ((uint64_t)d1 << i);
    s.D2 = (s.D2 & ~bit1(i)) | ((uint64_t)d2 << i);
}

// D[x] += d (d in {0,2,4,6} as bits d1, d2) for rows in u, mod 8, bit-sliced
template <int NR>
__device__ __forceinline__ void add_D(WS<NR>& s, uint64_t u, int d1, int d2) {
    const uint64_t a1 = d1 ? u : 0ull, a2 = d2 ? u : 0ull;
    const uint64_t carry = s.D1 & a1;
    s.D1 ^= a1;
    s.D2 ^= a2 ^ carry;
}

// ------------------------------------------------------------------ basis changes
// updateDJ (stabilizer.c:129-160) for R = I + u1 e_c1^T + u2 e_c2^T (c2 < 0: absent).
// Requires c1, c2 < k and u1, u2 subsets of [0,k) \ {c1, c2}.
template <int NR>
__device__ __forceinline__ void apply_R(WS<NR>& s, int c1, uint64_t u1, int c2, uint64_t u2) {
    const uint64_t km = lowmask(s.k);
    const uint64_t row1 = row_get<NR>(s.J, c1), col1 = ballot_bit<NR>(s.J, c1);
    uint64_t row2 = 0ull, col2 = 0ull;
    if (c2 >= 0) {
        row2 = row_get<NR>(s.J, c2);
        col2 = ballot_bit<NR>(s.J, c2);
    }
    // eq. 49: D <- R D (rows >= k become 0)
    const int d11 = getbit(s.D1, c1), d21 = getbit(s.D2, c1);
    int d12 = 0, d22 = 0;
    if (c2 >= 0) {
        d12 = getbit(s.D1, c2);
        d22 = getbit(s.D2, c2);
    }
    add_D<NR>(s, u1, d11, d21);
    if (c2 >= 0) add_D<NR>(s, u2, d12, d22);
    s.D1 &= km;
    s.D2 &= km;
    // + diag(R J R^T) lower-triangle parity, into D2
    uint64_t flip = u1 & ((col1 & ~lowmask(c1 + 1)) | (row1 & lowmask(c1)));
    if (c2 >= 0) {
        flip ^= u2 & ((col2 & ~lowmask(c2 + 1)) | (row2 & lowmask(c2)));
        const int jc = (c1 > c2) ? getbit(row1, c2) : getbit(row2, c1);
        if (jc) flip ^= u1 & u2;
    }
    s.D2 ^= flip;
    // eq. 50: J <- R J R^T
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        uint64_t r = s.J[sl];
        if (getbit(u1, x)) r ^= row1;
        if (c2 >= 0 && getbit(u2, x)) r ^= row2;
        uint64_t r2 = r;
        if (getbit(r, c1)) r2 ^= u1;
        if (c2 >= 0 && getbit(r, c2)) r2 ^= u2;
        s.J[sl] = r2;
    }
}

// updateDJ for the permutation swapping basis vectors i and j (both < k)
template <int NR>
__device__ __forceinline__ void apply_swap(WS<NR>& s, int i, int j) {
    const uint64_t km = lowmask(s.k);
    if (i != j) {
        s.D1 = swapbits(s.D1, i, j);
        s.D2 = swapbits(s.D2, i, j);
        row_swap<NR>(s.J, i, j);
#pragma unroll
        for (int sl = 0; sl < NR; sl++) s.J[sl] = swapbits(s.J[sl], i, j);
    }
    s.D1 &= km;
    s.D2 &= km;
}

// dense updateDJ for a general R (lane-distributed rows), stabilizer.c:129-160
template <int NR>
__device__ void update_dj_dense(WS<NR>& s, const uint64_t (&R)[NR]) {
    const int n = s.n;
    const uint64_t km = lowmask(s.k);
    int v[NR];
#pragma unroll
    for (int sl = 0; sl < NR; sl++)
        v[sl] = (__popcll(R[sl] & s.D1 & km) + 2 * __popcll(R[sl] & s.D2 & km)) & 3;
    const uint64_t nd1 = ballot_i<NR>(v[0] & 1, NR == 2 ? (v[NR - 1] & 1) : 0);
    const uint64_t nd2 = ballot_i<NR>((v[0] >> 1) & 1, NR == 2 ? ((v[NR - 1] >> 1) & 1) : 0);
    int fl[NR];
    uint64_t RJ[NR];
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        fl[sl] = 0;
        RJ[sl] = 0ull;
    }
    for (int b = 0; b < n; b++) {
        const uint64_t jb = row_get<NR>(s.J, b);
#pragma unroll
        for (int sl = 0; sl < NR; sl++)
            if (getbit(R[sl], b)) {
                fl[sl] += __popcll(jb & R[sl] & lowmask(b));
                RJ[sl] ^= jb;
            }
    }
    const uint64_t flip = ballot_i<NR>(fl[0] & 1, NR == 2 ? (fl[NR - 1] & 1) : 0);
    s.D1 = nd1;
    s.D2 = nd2 ^ flip;
    uint64_t Jn[NR];
#pragma unroll
    for (int sl = 0; sl < NR; sl++) Jn[sl] = 0ull;
    for (int y = 0; y < n; y++) {
        const uint64_t ry = row_get<NR>(R, y);
#pragma unroll
        for (int sl = 0; sl < NR; sl++) Jn[sl] |= (uint64_t)par64(RJ[sl] & ry) << y;
    }
#pragma unroll
    for (int sl = 0; sl < NR; sl++) s.J[sl] = Jn[sl];
}

// updateQD (stabilizer.c:163-177) for a general y
template <int NR>
__device__ void update_qd(WS<NR>& s, uint64_t y) {
    const uint64_t km = lowmask(s.k);
    int quad = 0;
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        if (x < s.k && getbit(y, x)) quad += __popcll(s.J[sl] & y & km & ~lowmask(x + 1));
    }
    quad = warp_sum(quad);
    const int lin = 2 * __popcll(s.D1 & y & km) + 4 * __popcll(s.D2 & y & km);
    s.Q = (s.Q + lin + 4 * quad) % 8;
    s.D2 ^= ballot_par<NR>(s.J, y);
}

// ------------------------------------------------------------------ shrink
// shrink (stabilizer.c:500-585).  LAZY skips the D/J/Q updates; TRACK_B keeps
// Gbar up to date (it is dead in the term-product inner loop).
template <int NR, bool LAZY, bool TRACK_B>
__device__ __forceinline__ int shrink_core(WS<NR>& s, uint64_t S, int beta) {
    if (S == 0ull) return 1 - beta;
    const int i = 63 - __clzll((long long)S);
    const uint64_t U = S & ~bit1(i);
    const uint64_t gi = row_get<NR>(s.G, i);
#pragma unroll
    for (int sl = 0; sl < NR; sl++)
        if (getbit(U, row_of<NR>(sl))) s.G[sl] ^= gi;
    if (!LAZY && U) apply_R<NR>(s, i, U, -1, 0ull);
    if (!LAZY && !U) {  // updateDJ is still called |S|-1 = 0 times: nothing to do
    }
    if (TRACK_B) {
        const uint64_t bi = row_get<NR>(s.B, i) ^ xor_rows<NR>(s.B, U);
        row_set<NR>(s.B, i, bi);
    }
    const int kk = s.k - 1;
    row_swap<NR>(s.G, i, kk);
    if (TRACK_B) row_swap<NR>(s.B, i, kk);
    if (!LAZY) apply_swap<NR>(s, i, kk);
    if (beta) s.h ^= row_get<NR>(s.G, kk);
    if (!LAZY) {
        if (beta) {
            s.Q = (s.Q + getD<NR>(s, kk)) % 8;
            s.D2 ^= ballot_bit<NR>(s.J, kk);
        } else {
            s.Q = s.Q % 8;
        }
    }
    s.k = kk;
    return 2;
}

template <int NR, bool LAZY, bool TRACK_B>
__device__ __forceinline__ int shrink(WS<NR>& s, uint64_t xi, int alpha) {
    const uint64_t S = ballot_par<NR>(s.G, xi) & lowmask(s.k);
    const int beta = (alpha + __popcll(xi & s.h)) % 2;
    return shrink_core<NR, LAZY, TRACK_B>(s, S, beta);
}

// shrink by the unit vector e_q with alpha = 0
template <int NR, bool TRACK_B>
__device__ __forceinline__ int shrink_unit(WS<NR>& s, int q) {
    const uint64_t S = ballot_bit<NR>(s.G, q) & lowmask(s.k);
    return shrink_core<NR, false, TRACK_B>(s, S, getbit(s.h, q));
}

// ------------------------------------------------------------------ exponential sum
// partialGamma (stabilizer.c:228-255): 1 + e^{i pi A/4}
__device__ __forceinline__ void partial_gamma(int A, int& e, int& p, int& m, int& err) {
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
__device__ __forceinline__ void gamma_ab(int A, int B, int& e, int& p, int& m, int& err) {
    if ((A % 2) || (B % 2) || A < 0 || B < 0) {
        err |= kErrGamma;
        e = 0; p = 0; m = 0;
        return;
    }
    const int a = (A % 8) / 2, b = (B % 8) / 2, c = ((A + B) % 8) / 2;
    // re/im of i^q for q = 0..3: (1,0) (0,1) (-1,0) (0,-1)
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

// W_sigma (stabilizer.c:258-297) as a warp reduction: monomers Mm, dimers
// (a in DA, partner[a] = b).  The reference accumulates p and m in order and
// stops at the first zero factor; sums mod 8 make the order irrelevant.
template <int NR>
__device__ void wsigma(const WS<NR>& s, int sigma, int sidx, uint64_t Mm, uint64_t DA, const int (&partner)[NR],
                       int& e, int& p, int& m, int& err) {
    if (s.k == 0) {
        e = 1; p = 0; m = s.Q;
        return;
    }
    const uint64_t cs = (sigma && sidx >= 0) ? ballot_bit<NR>(s.J, sidx) : 0ull;
    const int tM0 = s.Q + sigma * getD<NR>(s, sidx >= 0 ? sidx : 0);
    int zero = 0, P = 0, Ms = 0;
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        if (getbit(Mm, x)) {
            int ee, pp = 0, mm = 0;
            partial_gamma(getD<NR>(s, x) + sigma * 4 * getbit(cs, x), ee, pp, mm, err);
            if (!ee) zero = 1;
            P += pp;
            Ms += mm;
        }
        if (getbit(DA, x)) {
            const int b = partner[sl];
            int ee, pp = 0, mm = 0;
            gamma_ab(getD<NR>(s, x) + sigma * 4 * getbit(cs, x), getD<NR>(s, b) + sigma * 4 * getbit(cs, b), ee, pp,
                     mm, err);
            if (!ee) zero = 1;
            P += pp;
            Ms += mm;
        }
    }
    zero = __any_sync(kFull, zero);
    P = warp_sum(P);
    Ms = warp_sum(Ms);
    if (zero) {
        e = 0; p = 0; m = 0;
        return;
    }
    e = 1;
    p = P;
    m = (Mm | DA) ? (tM0 + Ms) % 8 : tM0;
}

// exponentialSumExact (stabilizer.c:300-481); modifies s like the reference.
// eps/p/m are left untouched on the reference's error-return path.
template <int NR>
__device__ void exp_sum(WS<NR>& s, int& eps, int& p, int& m, int& err) {
    const int k = s.k;
    const uint64_t km = lowmask(k);
    const uint64_t Sm = s.D1 & km;  // D[a] in {2, 6}
    int sidx = -1;
    if (Sm) {
        const int a = __ffsll((long long)Sm) - 1;
        const uint64_t U = Sm & ~bit1(a);
        if (U) apply_R<NR>(s, a, U, -1, 0ull);
        else {
            s.D1 &= km;  // updateDJ with R = I still clears D beyond k
            s.D2 &= km;
        }
        apply_swap<NR>(s, a, k - 1);
        sidx = k - 1;
    }
    uint64_t E = km & ~(sidx >= 0 ? bit1(sidx) : 0ull);
    uint64_t Mm = 0ull, DA = 0ull;
    int partner[NR];
#pragma unroll
    for (int sl = 0; sl < NR; sl++) partner[sl] = 0;
    while (E) {
        const int a = __ffsll((long long)E) - 1;
        const uint64_t ra = row_get<NR>(s.J, a);
        const uint64_t K = ra & E & ~bit1(a);
        if (!K) {
            Mm |= bit1(a);
            E &= ~bit1(a);
        } else {
            const int b = __ffsll((long long)K) - 1;
            const uint64_t Ep = E & ~bit1(a) & ~bit1(b);
            const uint64_t rb = row_get<NR>(s.J, b);
            const uint64_t vb = ra & Ep, va = rb & Ep;
            if (vb | va) apply_R<NR>(s, b, vb, a, va);
            else {
                s.D1 &= km;
                s.D2 &= km;
            }
            DA |= bit1(a);
#pragma unroll
            for (int sl = 0; sl < NR; sl++)
                if (row_of<NR>(sl) == a) partner[sl] = b;
            E = Ep;
        }
    }
    if (sidx < 0) {
        wsigma<NR>(s, 0, -1, Mm, DA, partner, eps, p, m, err);
        return;
    }
    int e0, p0, m0, e1, p1, m1;
    wsigma<NR>(s, 0, sidx, Mm, DA, partner, e0, p0, m0, err);
    wsigma<NR>(s, 1, sidx, Mm, DA, partner, e1, p1, m1, err);
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
    if (ee == 0) {
        p = 0; m = 0;
    } else {
        p = pp + p0;
        m = mm + m0 % 8;  // not reduced mod 8 (stabilizer.c:477)
    }
}

// ------------------------------------------------------------------ inner product
// innerProductExact (stabilizer.c:589-659); st is a working copy of state1.
template <int NR>
__device__ void inner_product(WS<NR> st, const WS<NR>& s2, int k1, int& eps, int& p, int& m, int& err) {
    const int n = s2.n;
    for (int b = s2.k; b < n; b++) {
        const uint64_t v = row_get<NR>(s2.B, b);
        const int alpha = __popcll(s2.h & v) % 2;
        eps = shrink<NR, false, false>(st, v, alpha);
        if (eps == 0) {
            p = 0; m = 0;
            return;
        }
    }
    // R[b][a] = G_b . G2bar_a,  y_a = (h + h2) . G2bar_a
    const bool trivial = (s2.Q == 0) && (s2.D1 == 0ull) && (s2.D2 == 0ull) && !any_row_nonzero<NR>(s2.J);
    WS<NR> t2 = s2;
    if (!trivial) {
        const uint64_t y = ballot_par<NR>(s2.B, st.h ^ s2.h);
        uint64_t R[NR];
#pragma unroll
        for (int sl = 0; sl < NR; sl++) R[sl] = 0ull;
        for (int a = 0; a < n; a++) {
            const uint64_t g2a = row_get<NR>(s2.B, a);
#pragma unroll
            for (int sl = 0; sl < NR; sl++) R[sl] |= (uint64_t)par64(st.G[sl] & g2a) << a;
        }
        update_qd<NR>(t2, y);
        update_dj_dense<NR>(t2, R);
    }
    st.Q -= t2.Q;
    if (st.Q < 0) st.Q += 8;
    {  // D <- (D - D2temp) mod 8 on all n entries, bit-sliced on D/2 mod 4
        const uint64_t a0 = st.D1, a1 = st.D2, b0 = t2.D1, b1 = t2.D2;
        const uint64_t borrow = ~a0 & b0;
        st.D1 = (a0 ^ b0) & lowmask(n);
        st.D2 = (a1 ^ b1 ^ borrow) & lowmask(n);
    }
#pragma unroll
    for (int sl = 0; sl < NR; sl++) st.J[sl] ^= t2.J[sl];
    exp_sum<NR>(st, eps, p, m, err);
    p -= k1 + s2.k;
}

// ------------------------------------------------------------------ measurePauli
// extend (stabilizer.c:759-825)
template <int NR>
__device__ void extend(WS<NR>& s, uint64_t xi) {
    const int n = s.n, k = s.k;
    const uint64_t S = ballot_par<NR>(s.B, xi) & lowmask(n);
    const uint64_t T = (k < n) ? (S & ~lowmask(k)) : 0ull;
    if (!T) return;
    const int i = __ffsll((long long)T) - 1;
    const uint64_t newS = S & ~bit1(i);
    const uint64_t gbar_i = row_get<NR>(s.B, i);
    const uint64_t g_i = row_get<NR>(s.G, i) ^ xor_rows<NR>(s.G, newS);
#pragma unroll
    for (int sl = 0; sl < NR; sl++)
        if (getbit(newS, row_of<NR>(sl))) s.B[sl] ^= gbar_i;
    row_set<NR>(s.G, i, g_i);
    row_swap<NR>(s.G, i, k);
    row_swap<NR>(s.B, i, k);
    s.k = k + 1;
}

// measurePauli (stabilizer.c:827-959).  Returns 0 (result 0), 1 (result 1) or
// 2 (result 2^{-1/2}); the host turns codes into the reference's doubles.
// -1 flags the impossible extend-without-growth case.
template <int NR>
__device__ int measure_pauli(WS<NR>& s, int m, uint64_t zeta, uint64_t xi) {
    const int n = s.n, k = s.k;
    const uint64_t km = lowmask(k);
    const uint64_t vXi = ballot_par<NR>(s.B, xi) & km;
    const uint64_t vZeta = ballot_par<NR>(s.G, zeta) & km;
    const uint64_t xiP = xor_rows<NR>(s.G, vXi);
    int quad = 0;
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        if (x < k && getbit(vXi, x)) quad += __popcll(s.J[sl] & vXi & ~lowmask(x + 1));
    }
    quad = warp_sum(quad);
    int w = 2 * m + 4 * (__popcll(zeta & s.h) % 2) + 2 * __popcll(s.D1 & vXi) + 4 * __popcll(s.D2 & vXi) + 4 * quad;
    w = w % 8;
    const uint64_t eta = ballot_par<NR>(s.J, vXi) ^ vZeta;
    if (xi == xiP) {
        if (w == 0 || w == 4) {
            const uint64_t gam = xor_rows<NR>(s.B, eta & km);
            const int alpha = (w / 4 + __popcll(gam & s.h)) % 2;
            return shrink<NR, false, true>(s, gam, alpha);  // 0 EMPTY, 1 SAME, 2 SUCCESS == result codes
        }
        if (w == 2 || w == 6) {
            const int sigma = 2 - w / 2;
            s.Q = (s.Q + sigma) % 8;
            while (s.Q < 0) s.Q += 8;
            const uint64_t u = eta & km;  // D[a] -= 2 sigma eta_a  (mod 8, halves mod 4)
            if (sigma == 1) {
                const uint64_t borrow = ~s.D1 & u;
                s.D1 ^= u;
                s.D2 ^= borrow;
            } else {
                const uint64_t carry = s.D1 & u;
                s.D1 ^= u;
                s.D2 ^= carry;
            }
#pragma unroll
            for (int sl = 0; sl < NR; sl++)
                if (getbit(eta, row_of<NR>(sl))) s.J[sl] ^= eta;
            return 2;
        }
    }
    extend<NR>(s, xi);
    const int newD = 2 * m + 4 * (__popcll(zeta & xi) % 2) + 4 * (__popcll(zeta & s.h) % 2);
    const int kk = s.k - 1;
    if (kk < 0) return -1;  // the reference would fail an assert in setD here
    setD<NR>(s, kk, newD);
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        s.J[sl] = (s.J[sl] & ~bit1(kk)) | ((uint64_t)getbit(vZeta, x) << kk);
    }
    uint64_t rowk = vZeta;
    if (m & 1) rowk |= bit1(kk);
    else rowk &= ~bit1(kk);
    row_set<NR>(s.J, kk, rowk);
    return 2;
}

// ------------------------------------------------------------------ global memory I/O
// csim_state layout (include/csim.h): n k Q r | h D1 D2 r | G[64] | Gbar[64] | J[64]
struct alignas(16) GState {
    int32_t n, k, Q, r0;
    uint64_t h, D1, D2, r1;
    uint64_t G[64], B[64], J[64];
};
static_assert(sizeof(GState) == 1584, "csim_state layout");

template <int NR>
__device__ __forceinline__ void load_state(const GState* g, WS<NR>& s) {
    const int l = lane_id();
    s.n = g->n;
    s.k = g->k;
    s.Q = g->Q;
    s.h = g->h;
    s.D1 = g->D1;
    s.D2 = g->D2;
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = l + 32 * sl;
        const bool in = x < s.n;
        s.G[sl] = in ? g->G[x] : 0ull;
        s.B[sl] = in ? g->B[x] : 0ull;
        s.J[sl] = in ? g->J[x] : 0ull;
    }
}

template <int NR>
__device__ __forceinline__ void store_state(GState* g, const WS<NR>& s) {
    const int l = lane_id();
    if (l == 0) {
        g->n = s.n;
        g->k = s.k;
        g->Q = s.Q;
        g->r0 = 0;
        g->h = s.h;
        g->D1 = s.D1;
        g->D2 = s.D2;
        g->r1 = 0ull;
    }
#pragma unroll
    for (int sl = 0; sl < 2; sl++) {
        const int x = l + 32 * sl;
        uint64_t gv = 0ull, bv = 0ull, jv = 0ull;
        if (sl < NR) {
            gv = s.G[sl < NR ? sl : 0];
            bv = s.B[sl < NR ? sl : 0];
            jv = s.J[sl < NR ? sl : 0];
        }
        g->G[x] = gv;
        g->B[x] = bv;
        g->J[x] = jv;
    }
}

template <int NR>
__device__ __forceinline__ void init_identity(WS<NR>& s, int n) {
    s.n = n;
    s.k = n;
    s.Q = 0;
    s.h = s.D1 = s.D2 = 0ull;
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        s.G[sl] = x < n ? bit1(x) : 0ull;
        s.B[sl] = s.G[sl];
        s.J[sl] = 0ull;
    }
}

}  // namespace csim
