// csim_batch_kernels.cu — kernels that run many probability queries at once
// (the batched executor, csim_run_queries).  They are the single-query kernels
// driven by descriptor tables, so states and (theta, term) pairs of queries
// with different t, codes and term counts share launches:
//   k_draw_project  one warp per state: draw it (Philox or replayed rand()
//                   words) or copy a term state, then project it onto its
//                   query's projector (innerprod.c:97-116 / :224-241)
//   k_items_tp      the thread-per-pair kernel over an item table of
//                   (state, range of |L> terms) work items
//   k_items_direct  the same items by direct restriction of each state's
//                   pivot form (launch_canon), one thread per pair
//   k_items_warp    the warp-per-pair kernel over (state, range of term states)
//   k_reduce_slots  per-slot sums of the items' partial sums
#include <cuda_runtime.h>

#include <cstdint>

#include "csim_batch.h"
#include "csim_internal.h"
#include "csim_block_prefix.cuh"
#include "csim_pair_core.cuh"
#include "csim_rng.cuh"
#include "csim_warp.cuh"

namespace csim {

namespace {

__device__ __forceinline__ int64_t wglobal() { return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ int64_t wcount() { return ((int64_t)gridDim.x * blockDim.x) >> 5; }

__device__ __forceinline__ void flush(int e, int* err) {
    e = (int)__reduce_or_sync(kFull, (unsigned)e);
    if (e && lane_id() == 0) atomicOr(err, e);
}

template <int NR>
__device__ void draw_project(const DrawDesc& d, GState* out, int* code, int& e) {
    WS<NR> st;
    if (d.mode == 2) {
        load_state<NR>(d.src, st);
    } else {
        DevRng rng;
        rng.mode = d.mode;
        rng.k0 = (uint32_t)d.seed;
        rng.k1 = (uint32_t)(d.seed >> 32);
        rng.id0 = (uint32_t)d.id;
        rng.id1 = (uint32_t)(d.id >> 32);
        rng.words = d.words;
        rng.base = d.wbegin;
        rng.end = d.wend;
        rng.cur = 0;
        random_state<NR>(st, d.n, rng, d.cum, e);
    }
    int c = 0;
    for (int r = 0; r < d.nstabs; r++) {
        const int res = measure_pauli<NR>(st, d.pm[r], d.pz[r], d.px[r]);
        if (res < 0) {
            e |= kErrRange;
            c = -1;
            break;
        }
        if (res == 0) {
            c = -1;
            break;
        }
        if (res == 2) c++;
    }
    store_state<NR>(out, st);
    if (lane_id() == 0) *code = c;
}

}  // namespace

__global__ void __launch_bounds__(256) k_draw_project(const DrawDesc* desc, int64_t count, GState* out, int* code,
                                                      int* err) {
    int e = 0;
    for (int64_t i = wglobal(); i < count; i += wcount()) {
        const DrawDesc d = desc[i];
        if (d.n <= 32) draw_project<1>(d, out + i, code + i, e);
        else draw_project<2>(d, out + i, code + i, e);
    }
    flush(e, err);
}

// ------------------------------------------------------------ thread-per-pair items
constexpr int kTPB = 64;

// Shared memory of a block: this struct, then the group states' J rows and G
// columns (pc::block_state_bytes(nmax)), then the pairs' working memory
struct ItemShared {
    pc::BlockPrefix bp;  // the item's state (group 0), then the states its codeword groups start from
    int n, live;
    long long next;      // the next item taken from the work queue
    __int128 red[kTPB / 32][8];
};

__device__ __forceinline__ __int128 shfl_xor_128(__int128 v, int m) {
    uint64_t lo = (uint64_t)v, hi = (uint64_t)((unsigned __int128)v >> 64);
    lo = ((uint64_t)__shfl_xor_sync(kFull, (uint32_t)(lo >> 32), m) << 32) | __shfl_xor_sync(kFull, (uint32_t)lo, m);
    hi = ((uint64_t)__shfl_xor_sync(kFull, (uint32_t)(hi >> 32), m) << 32) | __shfl_xor_sync(kFull, (uint32_t)hi, m);
    return (__int128)(((unsigned __int128)hi << 64) | lo);
}

// One block per item: up to kTPB * per_thread terms of one state.  part[4w..]:
// the item's sum; part_diag[4w..]: the term j == item.diag (exactProjector).
// Blocks take items in table order from the work queue `queue` (a zeroed
// counter; each block draws the next index when it finishes one), so a block
// that drew cheap items goes on to others while a costly one runs.
__global__ void __launch_bounds__(kTPB) k_items_tp(const PairItem* items, int64_t nitems, const GState* states,
                                                   const int* codes, int per_thread, int nmax, int gmax,
                                                   __int128* part, __int128* part_diag,
                                                   unsigned long long* queue, int only_live, const int* gate,
                                                   int* err) {
    if (gate && *gate == 0) return;  // no live state (block-uniform)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ItemShared& sh = *reinterpret_cast<ItemShared*>(smem_raw);
    uint64_t* const sa = reinterpret_cast<uint64_t*>(smem_raw + sizeof(ItemShared));
    unsigned char* const pair_base = smem_raw + sizeof(ItemShared) + pc::block_state_bytes(nmax);
    const int tid = threadIdx.x;
    int e = 0;
    if (tid == 0) sh.next = (long long)atomicAdd(queue, 1ull);
    __syncthreads();
    for (int64_t w = sh.next; w < nitems;) {
        const PairItem it = items[w];
        __syncthreads();
        const GState* g = states + it.theta;
        if (tid == 0) {
            sh.live = codes[it.theta] >= 0;
            sh.n = g->n;
            pc::BlockScalars& t0 = sh.bp.sc[0];
            t0.k = g->k;
            t0.Q = g->Q;
            t0.h = g->h;
            t0.D1 = g->D1;
            t0.D2 = g->D2;
            for (int q = 0; q < 7; q++) {
                sh.bp.andm[q] = ~0ull;
                sh.bp.orm[q] = 0ull;
            }
        }
        const int k0 = g->k;  // the state's own k, for p's correction
        const bool live0 = codes[it.theta] >= 0;  // sh.live, before the barrier that publishes it
        uint64_t* const r0 = pc::block_state_rows(sa, nmax, 0);
        if (live0 && tid < nmax) {
            r0[tid] = g->J[tid];
            const int n = g->n;
            uint64_t col = 0ull;
            if (tid < n)
                for (int r = 0; r < k0; r++) col |= ((g->G[r] >> tid) & 1ull) << r;
            r0[nmax + tid] = col;
        }
        __syncthreads();
        bool asym = false;
        if (sh.live && tid < k0 && k0 <= nmax)
            for (int r = 0; r < k0; r++) asym |= ((r0[tid] >> r) & 1ull) != ((r0[r] >> tid) & 1ull);
        asym = __syncthreads_or(asym) != 0;
        __int128 z[4] = {0, 0, 0, 0}, zd[4] = {0, 0, 0, 0};
        int deps = 0, dp = 0, dm = 0;  // the diagonal pair, summed apart after the loop
        const int n = sh.n;
        if (sh.live && (n > nmax || asym)) e |= kErrArg;
        if (sh.live && !asym && n >= 1 && n <= nmax) {
            // the shrinks that each of the item's codeword groups shares run once
            pc::block_prefix<kTPB>(sh.bp, sa, nmax, it.cw + it.j0, it.nj, per_thread, n, pair_base);
            const pc::PairMem mem = pc::pair_mem(pair_base, nmax, kTPB, tid);
            const int split1 = sh.bp.split1, split2a = sh.bp.split2[0], split2b = sh.bp.split2[1];
            const int P = 2 * n;
            for (int r = 0; r < per_thread; r++) {
                const int64_t j = it.j0 + tid + (int64_t)kTPB * r;
                const bool valid = j < it.j0 + it.nj;
                if (__all_sync(kFull, !valid)) break;
                const uint64_t x = valid ? it.cw[j] : 0ull;
                const int gr = pc::block_group(split1, split2a, split2b, x);
                const pc::BlockScalars& st = sh.bp.sc[gr];
                const uint64_t* rows = pc::block_state_rows(sa, nmax, gr);
                int eps = 0, pp = 0, mm = 0;
                pc::pair_l(valid && !st.dead, n, st.k, st.Q, st.h, st.D1, st.D2, rows, rows + nmax, x, mem, eps, pp,
                           mm, e, gmax, st.done, k0);
                if (!valid) continue;
                pc::zacc(z, eps, pp, mm, P, e);
                if (j == it.diag) {
                    deps = eps;
                    dp = pp;
                    dm = mm;
                }
            }
            pc::zacc(zd, deps, dp, dm, P, e);
            for (int q = 0; q < 4; q++) z[q] -= zd[q];
        }
        if (sh.live) {  // block-uniform
            for (int q = 0; q < 4; q++)
                for (int o = 16; o > 0; o >>= 1) {
                    z[q] += shfl_xor_128(z[q], o);
                    zd[q] += shfl_xor_128(zd[q], o);
                }
            if ((tid & 31) == 0)
                for (int q = 0; q < 4; q++) {
                    sh.red[tid >> 5][q] = z[q];
                    sh.red[tid >> 5][4 + q] = zd[q];
                }
        }
        __syncthreads();
        if (tid < 8 && (sh.live || !only_live)) {
            __int128 acc = 0;
            if (sh.live)
                for (int ww = 0; ww < kTPB / 32; ww++) acc += sh.red[ww][tid];
            if (tid < 4) part[4 * w + tid] = acc;
            else if (part_diag) part_diag[4 * w + tid - 4] = acc;
        }
        if (tid == 0) sh.next = (long long)atomicAdd(queue, 1ull);
        __syncthreads();
        w = sh.next;
    }
    e = (int)__reduce_or_sync(kFull, (unsigned)e);
    if (e && (tid & 31) == 0) atomicOr(err, e);
}

// ------------------------------------------------------------ direct-restriction items
// The direct kernel (pc::pair_direct) over the item table.  A block loads the
// item's state in pivot form into shared memory, then runs one thread per
// pair.  Items whose state launch_canon left to the block-prefix kernel
// (code_rest >= 0) are that kernel's to write; this one writes all others,
// zeros for dead states.
struct DirectItemShared {
    pc::Canon cs;
    int live, skip;
    long long next;  // the next item taken from the work queue
    __int128 red[kTPB / 32][8];
};
static_assert(kTPB == 64, "one thread per row of the 64-row pivot form");

__global__ void __launch_bounds__(kTPB) k_items_direct(const PairItem* items, int64_t nitems,
                                                       const pc::CanonG* canon, const int* code_direct,
                                                       const int* code_rest, int per_thread, int nmax, int rows,
                                                       int dslots, __int128* part, __int128* part_diag,
                                                       unsigned long long* queue, int* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DirectItemShared& sh = *reinterpret_cast<DirectItemShared*>(smem_raw);
    uint64_t* const sJ = reinterpret_cast<uint64_t*>(smem_raw + sizeof(DirectItemShared));  // 64 rows
    uint64_t* const sA = sJ + 64;                                                             // 64 masks
    unsigned char* const pair_base = smem_raw + sizeof(DirectItemShared) + 2 * 64 * 8;
    const int tid = threadIdx.x;
    int e = 0;
    const pc::PairMem mem = pc::pair_mem(pair_base, rows, kTPB, tid);
    if (tid == 0) sh.next = (long long)atomicAdd(queue, 1ull);
    __syncthreads();
    for (int64_t w = sh.next; w < nitems;) {
        const PairItem it = items[w];
        __syncthreads();  // the previous item's use of the shared state is over
        if (tid == 0) {
            sh.live = code_direct[it.theta] >= 0;
            sh.skip = code_rest[it.theta] >= 0;
            if (sh.live) sh.cs = canon[it.theta].cs;
        }
        __syncthreads();
        if (sh.live) {
            sJ[tid] = canon[it.theta].Jc[tid];
            sA[tid] = canon[it.theta].acol[tid];
        }
        __syncthreads();
        __int128 z[4] = {0, 0, 0, 0}, zd[4] = {0, 0, 0, 0};
        if (sh.live) {  // block-uniform
            const int n = sh.cs.n;
            if (n > nmax) e |= kErrArg;
            if (n >= 1 && n <= nmax) {
                const int P = 2 * n;
                int deps = 0, dp = 0, dm = 0;  // the diagonal pair, summed apart
                for (int r = 0; r < per_thread; r++) {
                    const int64_t j = it.j0 + tid + (int64_t)kTPB * r;
                    const bool valid = j < it.j0 + it.nj;
                    if (__all_sync(kFull, !valid)) break;  // warp-uniform exit
                    const uint64_t x = valid ? it.cw[j] : 0ull;
                    int eps = 0, pp = 0, mm = 0;
                    pc::pair_direct(valid, n, sh.cs, sJ, sA, x, mem, eps, pp, mm, e, dslots, sh.cs.k, rows);
                    if (!valid) continue;
                    pc::zacc(z, eps, pp, mm, P, e);
                    if (j == it.diag) {
                        deps = eps;
                        dp = pp;
                        dm = mm;
                    }
                }
                pc::zacc(zd, deps, dp, dm, P, e);
                for (int q = 0; q < 4; q++) z[q] -= zd[q];
            }
            for (int q = 0; q < 4; q++)
                for (int o = 16; o > 0; o >>= 1) {
                    z[q] += shfl_xor_128(z[q], o);
                    zd[q] += shfl_xor_128(zd[q], o);
                }
            if ((tid & 31) == 0)
                for (int q = 0; q < 4; q++) {
                    sh.red[tid >> 5][q] = z[q];
                    sh.red[tid >> 5][4 + q] = zd[q];
                }
        }
        __syncthreads();
        if (tid < 8 && !sh.skip) {
            __int128 acc = 0;
            if (sh.live)
                for (int ww = 0; ww < kTPB / 32; ww++) acc += sh.red[ww][tid];
            if (tid < 4) part[4 * w + tid] = acc;
            else if (part_diag) part_diag[4 * w + tid - 4] = acc;
        }
        if (tid == 0) sh.next = (long long)atomicAdd(queue, 1ull);
        __syncthreads();
        w = sh.next;
    }
    e = (int)__reduce_or_sync(kFull, (unsigned)e);
    if (e && (tid & 31) == 0) atomicOr(err, e);
}

// ------------------------------------------------------------ warp-per-pair items
__device__ __forceinline__ void zacc_w(__int128 (&z)[4], int eps, int p, int m, int P, int& err) {
    pc::zacc(z, eps, p, m, P, err);
}

template <int NR>
__device__ void item_warp(const PairItem& it, const GState* states, const int* codes, __int128* part,
                          __int128* part_diag, int64_t w, int& e) {
    __int128 z[4] = {0, 0, 0, 0}, zd[4] = {0, 0, 0, 0};
    if (codes[it.theta] >= 0) {
        WS<NR> base;
        load_state<NR>(states + it.theta, base);
        const int P = 2 * base.n;
        for (int64_t j = it.j0; j < it.j0 + it.nj; j++) {
            WS<NR> phi;
            load_state<NR>(it.phis + j, phi);
            int ee = 0, pp = 0, mm = 0;
            inner_product<NR>(base, phi, base.k, ee, pp, mm, e);
            if (j == it.diag) zacc_w(zd, ee, pp, mm, P, e);
            else zacc_w(z, ee, pp, mm, P, e);
        }
    }
    if (lane_id() == 0) {
        for (int q = 0; q < 4; q++) part[4 * w + q] = z[q];
        if (part_diag)
            for (int q = 0; q < 4; q++) part_diag[4 * w + q] = zd[q];
    }
}

__global__ void __launch_bounds__(256) k_items_warp(const PairItem* items, int64_t nitems, const GState* states,
                                                    const int* codes, __int128* part, __int128* part_diag, int* err) {
    int e = 0;
    for (int64_t w = wglobal(); w < nitems; w += wcount()) {
        const PairItem it = items[w];
        const int n = states[it.theta].n;
        if (n <= 32) item_warp<1>(it, states, codes, part, part_diag, w, e);
        else item_warp<2>(it, states, codes, part, part_diag, w, e);
    }
    flush(e, err);
}

// slot s sums the items [range[2s], range[2s+1]) and [range2[2s], range2[2s+1])
__global__ void k_reduce_slots(const __int128* part, const int64_t* range, const int64_t* range2, int64_t nslots,
                               __int128* out) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nslots * 4;
         w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = w / 4, q = w % 4;
        __int128 acc = 0;
        for (int64_t i = range[2 * s]; i < range[2 * s + 1]; i++) acc += part[4 * i + q];
        if (range2)
            for (int64_t i = range2[2 * s]; i < range2[2 * s + 1]; i++) acc += part[4 * i + q];
        out[w] = acc;
    }
}

// ------------------------------------------------------------ launchers
size_t items_tp_smem(int nmax, int gmax) {
    return sizeof(ItemShared) + pc::block_state_bytes(nmax) + pc::pair_mem_bytes(nmax, gmax, kTPB);
}

int launch_draw_project(const Launch& L, const DrawDesc* desc, int64_t count, GState* out, int* code) {
    if (count <= 0) return 0;
    int64_t blocks = (count + 7) / 8;
    if (blocks > (int64_t)L.num_sms * 8) blocks = (int64_t)L.num_sms * 8;
    k_draw_project<<<(int)blocks, 256, 0, L.stream>>>(desc, count, out, code, L.d_err);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int items_tp_occupancy(int nmax, int gmax) {
    if (nmax < 1 || nmax > 64 || gmax < 0 || gmax > nmax) return -1;
    if (cudaFuncSetAttribute(k_items_tp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)items_tp_smem(64, 64)) !=
        cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_items_tp, kTPB, items_tp_smem(nmax, gmax)) !=
        cudaSuccess)
        return -1;
    return per_sm;
}

int launch_items_tp(const Launch& L, const PairItem* items, int64_t nitems, const GState* states, const int* codes,
                    int per_thread, int nmax, int gmax, __int128* part, __int128* part_diag,
                    unsigned long long* queue, bool only_live, const int* gate) {
    if (nitems <= 0) return 0;
    if (nmax < 1 || nmax > 64 || gmax < 0 || gmax > nmax || !queue) return -1;
    if (cudaMemsetAsync(queue, 0, sizeof(unsigned long long), L.stream) != cudaSuccess) return -1;
    const size_t smem = items_tp_smem(nmax, gmax);
    if (cudaFuncSetAttribute(k_items_tp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)items_tp_smem(64, 64)) !=
        cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_items_tp, kTPB, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int64_t grid = (int64_t)L.num_sms * per_sm;
    if (grid > nitems) grid = nitems;
    k_items_tp<<<(int)grid, kTPB, smem, L.stream>>>(items, nitems, states, codes, per_thread, nmax, gmax, part,
                                                    part_diag, queue, only_live ? 1 : 0, gate, L.d_err);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

namespace {
size_t items_direct_smem(int nmax, int dslots) {
    return sizeof(DirectItemShared) + 2 * 64 * 8 + pc::pair_mem_bytes(nmax, dslots, kTPB);
}
}  // namespace

int launch_items_direct(const Launch& L, const PairItem* items, int64_t nitems, const void* canon,
                        const int* code_direct, const int* code_rest, int per_thread, int nmax, int rows, int dslots,
                        __int128* part, __int128* part_diag, unsigned long long* queue) {
    if (nitems <= 0) return 0;
    if (nmax < 1 || nmax > 64 || rows < 1 || rows > nmax || dslots < 0 || dslots > nmax || per_thread < 1 || !queue ||
        !canon)
        return -1;
    if (cudaMemsetAsync(queue, 0, sizeof(unsigned long long), L.stream) != cudaSuccess) return -1;
    if (cudaFuncSetAttribute(k_items_direct, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)items_direct_smem(64, 64)) != cudaSuccess)
        return -1;
    const size_t smem = items_direct_smem(rows, dslots);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_items_direct, kTPB, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int64_t grid = (int64_t)L.num_sms * per_sm;
    if (grid > nitems) grid = nitems;
    k_items_direct<<<(int)grid, kTPB, smem, L.stream>>>(items, nitems, (const pc::CanonG*)canon, code_direct,
                                                        code_rest, per_thread, nmax, rows, dslots, part, part_diag,
                                                        queue, L.d_err);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_items_warp(const Launch& L, const PairItem* items, int64_t nitems, const GState* states, const int* codes,
                      __int128* part, __int128* part_diag) {
    if (nitems <= 0) return 0;
    int64_t blocks = (nitems + 7) / 8;
    if (blocks > (int64_t)L.num_sms * 8) blocks = (int64_t)L.num_sms * 8;
    k_items_warp<<<(int)blocks, 256, 0, L.stream>>>(items, nitems, states, codes, part, part_diag, L.d_err);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_reduce_slots(const Launch& L, const __int128* part, const int64_t* range, const int64_t* range2,
                        int64_t nslots, __int128* out) {
    if (nslots <= 0) return 0;
    int64_t blocks = (nslots * 4 + 255) / 256;
    if (blocks > (int64_t)L.num_sms * 16) blocks = (int64_t)L.num_sms * 16;
    k_reduce_slots<<<(int)blocks, 256, 0, L.stream>>>(part, range, range2, nslots, out);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace csim
