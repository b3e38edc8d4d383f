// csim_block_prefix.cuh — the block-level step of the thread-per-pair kernels
// (csim_terms_tp.cu, csim_batch_kernels.cu).
//
// A pair's shrinks run over its codeword's zero bits from the top down, so all
// pairs whose codewords agree on some top bits pass through one state: the
// state after the shrinks by the zeros among those bits.  A block splits its
// codewords in two halves at the highest bit in which they differ, and each
// half again at its own highest differing bit: up to four groups, each
// agreeing on every bit above its split bits and on the bits it holds in
// common below them.  One lane per group runs that group's shared shrinks once
// (prefix_shrink), and each pair continues from its group's state.
#pragma once

#include <cstdint>

#include "csim_pair_core.cuh"

namespace csim {
namespace pc {

constexpr int kGroups = 4;

// The scalar part of a group's starting state; its J rows and G columns live
// in the block's state arrays (block_state_rows)
struct BlockScalars {
    uint64_t h, D1, D2;
    uint64_t done;  // top bits whose shrinks this state has been through
    int k, Q, dead, pad;
};

struct BlockPrefix {
    BlockScalars sc[kGroups];
    // AND / OR of the codewords: [0] all; [1 + h] half h; [3 + 2h + q] group 2h + q
    unsigned long long andm[7], orm[7];
    int split1;     // highest bit in which the codewords differ, or -1
    int split2[2];  // the same within each half
    int pad;
};

// Group g's J rows (nmax words) followed by its G columns (nmax words), in
// state arrays of kGroups * 2 * nmax words
CSIM_HD inline uint64_t* block_state_rows(uint64_t* sa, int nmax, int g) { return sa + (size_t)g * 2 * nmax; }
CSIM_HD inline size_t block_state_bytes(int nmax) { return (size_t)kGroups * 2 * nmax * 8; }

// The group of codeword x (splits as in BlockPrefix)
CSIM_HD inline int block_group(int split1, int split2a, int split2b, uint64_t x) {
    if (split1 < 0) return 0;
    const int h = (int)((x >> split1) & 1ull);
    const int s2 = h ? split2b : split2a;
    return 2 * h + (s2 >= 0 ? (int)((x >> s2) & 1ull) : 0);
}

// highest set bit of d, or -1
CSIM_HD inline int top_bit_or_none(uint64_t d) { return d ? 63 - hd_clz64(d) : -1; }

#if defined(__CUDACC__)
__device__ __forceinline__ uint64_t warp_and64(uint64_t v) {
    return ((uint64_t)__reduce_and_sync(0xffffffffu, (unsigned)(v >> 32)) << 32) |
           __reduce_and_sync(0xffffffffu, (unsigned)v);
}
__device__ __forceinline__ uint64_t warp_or64(uint64_t v) {
    return ((uint64_t)__reduce_or_sync(0xffffffffu, (unsigned)(v >> 32)) << 32) |
           __reduce_or_sync(0xffffffffu, (unsigned)v);
}

// AND / OR of the block's codewords by class into bp.andm / bp.orm [base + c]:
// class c = cls(x) in {0, 1}, or -1 to leave x out
template <int NT, class Cls>
__device__ __forceinline__ void block_and_or(BlockPrefix& bp, const uint64_t* cwb, int64_t count, int per_thread,
                                             int base, Cls cls) {
    uint64_t a0 = ~0ull, o0 = 0ull, a1 = ~0ull, o1 = 0ull;
    for (int r = 0; r < per_thread; r++) {
        const int64_t j = threadIdx.x + (int64_t)NT * r;
        if (j < count) {
            const uint64_t x = cwb[j];
            const int c = cls(x);
            if (c == 0) {
                a0 &= x;
                o0 |= x;
            } else if (c == 1) {
                a1 &= x;
                o1 |= x;
            }
        }
    }
    a0 = warp_and64(a0);
    o0 = warp_or64(o0);
    a1 = warp_and64(a1);
    o1 = warp_or64(o1);
    if ((threadIdx.x & 31) == 0) {
        atomicAnd(&bp.andm[base], (unsigned long long)a0);
        atomicOr(&bp.orm[base], (unsigned long long)o0);
        atomicAnd(&bp.andm[base + 1], (unsigned long long)a1);
        atomicOr(&bp.orm[base + 1], (unsigned long long)o1);
    }
}

// Call with group 0's state arrays and scalars holding theta (symmetric J),
// bp.andm[] = ~0 and bp.orm[] = 0, after a barrier; every thread of the
// NT-thread block calls it.  sa: the kGroups state arrays (block_state_rows).
// The block's codewords are cwb[0, count); thread t reads cwb[t + NT r] for
// r < per_thread.  `work`: 4 KB of shared scratch (the pair memory before the
// pairs use it).  On return, after the final barrier, the splits and every
// used group's state are set, each with its `done` bits and `dead` flag (a
// shrink found the projection empty).  Not inlined: it runs once per block
// item, and inlined it raised the kernels' register count (and so lowered
// their occupancy).
template <int NT>
__device__ __noinline__ void block_prefix(BlockPrefix& bp, uint64_t* sa, int nmax, const uint64_t* cwb, int64_t count,
                                          int per_thread, int n, unsigned char* work) {
    static_assert(NT == 64, "two groups per warp");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint64_t nm = lowmask(n);
    // [0] all codewords (class 0; class 1 stays empty)
    block_and_or<NT>(bp, cwb, count, per_thread, 0, [](uint64_t) { return 0; });
    __syncthreads();
    const int hb = top_bit_or_none((bp.andm[0] ^ bp.orm[0]) & nm);
    int hb2[2] = {-1, -1};
    if (hb >= 0) {
        block_and_or<NT>(bp, cwb, count, per_thread, 1, [hb](uint64_t x) { return (int)((x >> hb) & 1ull); });
        __syncthreads();
        hb2[0] = top_bit_or_none((bp.andm[1] ^ bp.orm[1]) & nm);
        hb2[1] = top_bit_or_none((bp.andm[2] ^ bp.orm[2]) & nm);
        for (int h = 0; h < 2; h++) {
            const int s2 = hb2[h];
            if (s2 >= 0)
                block_and_or<NT>(bp, cwb, count, per_thread, 3 + 2 * h, [hb, s2, h](uint64_t x) {
                    return (int)((x >> hb) & 1ull) == h ? (int)((x >> s2) & 1ull) : -1;
                });
        }
    }
    // the used groups and the AND / OR slot of each
    bool used[kGroups] = {true, false, false, false};
    int slot[kGroups] = {0, 0, 0, 0};
    if (hb >= 0) {
        for (int h = 0; h < 2; h++) {
            used[2 * h] = true;
            slot[2 * h] = hb2[h] < 0 ? 1 + h : 3 + 2 * h;
            if (hb2[h] >= 0) {
                used[2 * h + 1] = true;
                slot[2 * h + 1] = 4 + 2 * h;
            }
        }
    }
    // every other used group starts from its own copy of theta
    for (int g = 1; g < kGroups; g++) {
        if (!used[g]) continue;
        uint64_t* dst = block_state_rows(sa, nmax, g);
        const uint64_t* src = block_state_rows(sa, nmax, 0);
        for (int i = tid; i < 2 * nmax; i += NT) dst[i] = src[i];
        if (tid == 0) bp.sc[g] = bp.sc[0];
    }
    __syncthreads();  // the last AND / OR pass and the copies are complete
    // group g runs on lane g & 1 of warp g >> 1
    const int g = 2 * warp + (lane & 1);
    const bool mine = lane < 2 && used[g];
    const int gs = mine ? g : 2 * warp;  // a valid group for the lanes without one
    const uint64_t am = mine ? bp.andm[slot[g]] : 0ull, om = mine ? bp.orm[slot[g]] : 0ull;
    const uint64_t pm = agree_top(am ^ om, n);  // the group's codewords all equal am on pm
    const bool act = mine && hd_popc64(~am & pm & nm) > 0;
    BlockScalars& s = bp.sc[gs];
    uint64_t* rows = block_state_rows(sa, nmax, gs);
    int ok = 1;
    if (__any_sync(0xffffffffu, act)) {
        const PairMem M = pair_mem(work + 1024 * gs, nmax, 1, 0);
        ok = prefix_shrink(act, n, pm, am, s.k, s.Q, s.h, s.D1, s.D2, rows, rows + nmax, M);
    }
    if (mine) {
        s.done = pm;
        s.dead = !ok;
    }
    if (tid == 0) {
        bp.split1 = hb;
        bp.split2[0] = hb2[0];
        bp.split2[1] = hb2[1];
    }
    __syncthreads();
}
#endif

}  // namespace pc
}  // namespace csim
