// csim_rng.cuh — random words for randomStabilizerState on the device.
//
// The reference draws every random bit through the C library's rand()
// (libcirc/stabilizer/stabilizer.c:669-756, libcirc/utils/matrix.c:85-92).
// A state's draws are addressed here by their position c in that state's own
// sequence, from one of two sources:
//   * Philox-4x32-10 (Salmon et al., SC'11), counter (c/4, id, id_hi, c>>34),
//     key = seed: an independent stream per state, 31-bit outputs like rand();
//   * replay: words[base + c], the exact values rand() returned to the
//     reference, recorded or regenerated on the host.
#pragma once

#include <cstdint>

#include "csim_warp.cuh"

namespace csim {

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

struct DevRng {
    int mode;                // 0 = Philox, 1 = replay
    uint32_t k0, k1;         // Philox key
    uint32_t id0, id1;       // Philox stream (state index)
    const uint32_t* words;   // replay words
    int64_t base, end;       // replay segment [base, end)
    int64_t cur;             // next draw position

    __device__ __forceinline__ uint32_t at(int64_t c, int& err) const {
        if (mode == 1) {
            const int64_t q = base + c;
            if (q >= end) {
                err |= kErrReplay;
                return 0u;
            }
            return words[q];
        }
        const uint4 r = philox4x32_10(make_uint4((uint32_t)(c >> 2), id0, id1, (uint32_t)(c >> 34)), k0, k1);
        const int j = (int)(c & 3);
        const uint32_t w = j == 0 ? r.x : (j == 1 ? r.y : (j == 2 ? r.z : r.w));
        return w >> 1;
    }

    __device__ __forceinline__ uint32_t next(int& err) { return at(cur++, err); }

    // ceil(n/8) bytes rand() % 256, bit j of byte b (MSB first) -> bit 8b+j
    __device__ __forceinline__ uint64_t bits(int n, int& err) {
        uint64_t w = 0ull;
        const int bytes = (n + 7) / 8;
        for (int b = 0; b < bytes; b++) {
            const uint32_t byte = next(err) % 256u;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int loc = 8 * b + j;
                if (loc < n && (byte & (0x80u >> j))) w |= bit1(loc);
            }
        }
        return w;
    }
};

// randomStabilizerState (stabilizer.c:689-756).  cum[0..n] is the
// normalized cumulative distribution of eq. 79 computed on the host with the
// reference's own libm expressions (logeta, stabilizer.c:677-687).
template <int NR>
__device__ void random_state(WS<NR>& s, int n, DevRng& rng, const double* cum, int& err) {
    double sample = 0.0;
    for (int guard = 0; guard < 64; guard++) {  // rand() == 0 has probability 2^-31 per draw
        sample = 0.0 + (double)rng.next(err) / 2147483647.0;
        if (sample != 0.0 || (err & kErrReplay)) break;
    }
    int d = 0;
    for (; d <= n; d++)
        if (sample <= cum[d]) break;
    if (d > n) d = n;
    const int kt = n - d;
    init_identity<NR>(s, n);
    for (int guard = 0; s.k > kt; guard++) {
        if (guard > 4096 || (err & kErrReplay)) {
            err |= (err & kErrReplay) ? 0 : kErrArg;
            break;
        }
        const uint64_t xi = rng.bits(n, err);
        shrink<NR, true, true>(s, xi, 0);
    }
    s.h = rng.bits(n, err);
    s.D1 = rng.bits(n, err);
    s.D2 = rng.bits(n, err);
    const int k = s.k;
    const int64_t base = rng.cur;
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        uint64_t row = 0ull;
        if (x < k) {
            row = (uint64_t)getbit(s.D1, x) << x;  // J[x][x] = ((2 D[x]) mod 8) / 4
            for (int c = 0; c < k; c++) {
                if (c == x) continue;
                const int64_t idx = x > c ? base + (int64_t)x * (x - 1) / 2 + c : base + (int64_t)c * (c - 1) / 2 + x;
                row |= (uint64_t)(rng.at(idx, err) & 1u) << c;
            }
        }
        s.J[sl] = row;
    }
    rng.cur = base + (int64_t)k * (k - 1) / 2;
    // every lane may have seen a different replay overrun
    if (__any_sync(kFull, (err & kErrReplay) != 0)) err |= kErrReplay;
}

}  // namespace csim
