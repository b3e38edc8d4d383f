// csim_block_prefix.cuh — the block-level step of the thread-per-pair kernels
// (csim_terms_tp.cu, csim_batch_kernels.cu).
//
// A pair's shrinks run over its codeword's zero bits from the top down, so all
// pairs whose codewords agree on some top bits pass through one state: the
// state after the shrinks by the zeros among those bits.  A block splits its
// codewords in two groups at the highest bit in which they differ; each group
// agrees on every bit above that one and on the bits it holds in common below
// it.  One lane per group runs that group's shared shrinks once
// (prefix_shrink), and each pair continues from its group's state.
#pragma once

#include <cstdint>

#include "csim_pair_core.cuh"

namespace csim {
namespace pc {

// Theta, or the state a group of a block's pairs starts from
struct BlockState {
    uint64_t pJ[64];   // J rows
    uint64_t pGT[64];  // G columns as row masks
    uint64_t h, D1, D2;
    uint64_t done;     // top bits whose shrinks this state has been through
    int k, Q, dead, pad;
};

struct BlockPrefix {
    BlockState st[2];                    // group 0 (bit `split` clear) and group 1
    unsigned long long andm[3], orm[3];  // AND / OR of the codewords: all, group 0, group 1
    int split;                           // highest bit in which the codewords differ, or -1
};

#if defined(__CUDACC__)
__device__ __forceinline__ uint64_t warp_and64(uint64_t v) {
    return ((uint64_t)__reduce_and_sync(0xffffffffu, (unsigned)(v >> 32)) << 32) |
           __reduce_and_sync(0xffffffffu, (unsigned)v);
}
__device__ __forceinline__ uint64_t warp_or64(uint64_t v) {
    return ((uint64_t)__reduce_or_sync(0xffffffffu, (unsigned)(v >> 32)) << 32) |
           __reduce_or_sync(0xffffffffu, (unsigned)v);
}

// Call with bp.st[0] holding theta (symmetric J), bp.andm[] = ~0 and bp.orm[]
// = 0, after a barrier; every thread of the NT-thread block calls it.  The
// block's codewords are cwb[0, count); thread t reads cwb[t + NT r] for
// r < per_thread.  `work`: 2 KB of shared scratch (the pair memory before the
// pairs use it).  On return, after the final barrier, bp.split and the group
// states (bp.st[0], and bp.st[1] if split >= 0) are set, each with its `done`
// bits and `dead` flag (a shrink found the projection empty).  Not inlined:
// it runs once per block item, and inlined it raised the kernels' register
// count (and so lowered their occupancy).
template <int NT>
__device__ __noinline__ void block_prefix(BlockPrefix& bp, const uint64_t* cwb, int64_t count, int per_thread,
                                          int n, int nmax, unsigned char* work) {
    static_assert(NT == 64, "one warp per group");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint64_t nm = lowmask(n);
    {
        uint64_t a = ~0ull, o = 0ull;
        for (int r = 0; r < per_thread; r++) {
            const int64_t j = tid + (int64_t)NT * r;
            if (j < count) {
                const uint64_t x = cwb[j];
                a &= x;
                o |= x;
            }
        }
        a = warp_and64(a);
        o = warp_or64(o);
        if (lane == 0) {
            atomicAnd(&bp.andm[0], (unsigned long long)a);
            atomicOr(&bp.orm[0], (unsigned long long)o);
        }
    }
    __syncthreads();
    const uint64_t dis = (bp.andm[0] ^ bp.orm[0]) & nm;
    const int hb = dis ? 63 - hd_clz64(dis) : -1;
    if (hb >= 0) {
        uint64_t a0 = ~0ull, o0 = 0ull, a1 = ~0ull, o1 = 0ull;
        for (int r = 0; r < per_thread; r++) {
            const int64_t j = tid + (int64_t)NT * r;
            if (j < count) {
                const uint64_t x = cwb[j];
                if ((x >> hb) & 1ull) {
                    a1 &= x;
                    o1 |= x;
                } else {
                    a0 &= x;
                    o0 |= x;
                }
            }
        }
        a0 = warp_and64(a0);
        o0 = warp_or64(o0);
        a1 = warp_and64(a1);
        o1 = warp_or64(o1);
        if (lane == 0) {
            atomicAnd(&bp.andm[1], (unsigned long long)a0);
            atomicOr(&bp.orm[1], (unsigned long long)o0);
            atomicAnd(&bp.andm[2], (unsigned long long)a1);
            atomicOr(&bp.orm[2], (unsigned long long)o1);
        }
        // group 1 starts from its own copy of theta
        bp.st[1].pJ[tid] = bp.st[0].pJ[tid];
        bp.st[1].pGT[tid] = bp.st[0].pGT[tid];
        if (tid == 0) {
            bp.st[1].h = bp.st[0].h;
            bp.st[1].D1 = bp.st[0].D1;
            bp.st[1].D2 = bp.st[0].D2;
            bp.st[1].k = bp.st[0].k;
            bp.st[1].Q = bp.st[0].Q;
        }
        __syncthreads();
    }
    // warp g runs group g's shared shrinks on its lane 0
    if (warp < (hb >= 0 ? 2 : 1)) {
        BlockState& s = bp.st[warp];
        const uint64_t am = hb >= 0 ? bp.andm[1 + warp] : bp.andm[0];
        const uint64_t om = hb >= 0 ? bp.orm[1 + warp] : bp.orm[0];
        const uint64_t pm = agree_top(am ^ om, n);  // the group's codewords all equal am on pm
        int ok = 1;
        if (hd_popc64(~am & pm & nm) > 0) {
            const PairMem M = pair_mem(work + 1024 * warp, nmax, 1, 0);
            ok = prefix_shrink(lane == 0, n, pm, am, s.k, s.Q, s.h, s.D1, s.D2, s.pJ, s.pGT, M);
        }
        if (lane == 0) {
            s.done = pm;
            s.dead = !ok;
        }
    }
    if (tid == 0) bp.split = hb;
    __syncthreads();
}
#endif

}  // namespace pc
}  // namespace csim
