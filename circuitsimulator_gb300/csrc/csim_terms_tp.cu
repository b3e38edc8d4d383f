// csim_terms_tp.cu — the (theta, prepL term) pair kernel, one thread per pair.
//
// For a term phi_x of |L> (a product of |0> and |+>, libcirc/stateprep.c:85-120)
// innerProductExact(theta, phi_x) (libcirc/stabilizer/stabilizer.c:589-659)
// reduces to shrinks of theta by e_q, alpha = 0, for the zero bits q of the
// codeword x in descending order, then exponentialSumExact: phi_x has
// Q = D = J = h = 0, so the R stage (stabilizer.c:611-652) changes nothing.
//
// Each thread keeps its pair's working state in shared memory with a
// [index][thread] layout (pc::PairMem):
//   rows 0..31 of J, low 32 bits, four per 16-byte unit
//   rows 32.. of J, 64 bits, two per 16-byte unit
//   the G columns of x's zero positions as row masks, in shrink order (the
//   only ones a later shrink or h-update of this pair reads)
// and D1, D2, h, Q, k in registers.  Every basis change is the elementary
// rank-one update of csim_warp.cuh applied row by row, with each row's
// column bits gathered in the same pass; the exponential sum folds each
// monomer/dimer factor into W0/W1 as soon as that row is final
// (stabilizer.c:372-418 never touches a finished row again).
//
// Before its pairs, a block runs the shrinks that each of its (up to four)
// codeword groups shares once, on one lane per group (csim_block_prefix.cuh);
// each pair starts from its group's state.
#include <cuda_runtime.h>

#include <cstdint>

#include "csim_internal.h"
#include "csim_block_prefix.cuh"
#include "csim_pair_core.cuh"
#include "csim_warp.cuh"

namespace csim {

constexpr int kTP = 64;  // threads per block

// Shared memory of a block: this struct, then the group states' J rows and G
// columns (pc::block_state_bytes(nmax)), then the pairs' working memory
struct TPShared {
    pc::BlockPrefix bp;  // theta (group 0), then the states the block's codeword groups start from
    int n, live;
    __int128 red[kTP / 32][4];
};

__device__ __forceinline__ __int128 shfl_xor_i128(__int128 v, int m) {
    uint64_t lo = (uint64_t)v, hi = (uint64_t)((unsigned __int128)v >> 64);
    lo = ((uint64_t)__shfl_xor_sync(kFull, (uint32_t)(lo >> 32), m) << 32) | __shfl_xor_sync(kFull, (uint32_t)lo, m);
    hi = ((uint64_t)__shfl_xor_sync(kFull, (uint32_t)(hi >> 32), m) << 32) | __shfl_xor_sync(kFull, (uint32_t)hi, m);
    return (__int128)(((unsigned __int128)hi << 64) | lo);
}

// Work item = (theta a, block cb of kTP * per_thread consecutive terms).  Thread t
// takes terms jb + t + kTP * r, r < per_thread.  Partial sums: 4 int128 per item,
// at part[4 * (a * part_stride + part_base + cb)].  gmax bounds the zeros of
// every codeword in [j0, j0 + nj) and sizes the G-column slots.
__global__ void __launch_bounds__(kTP) k_terms_tp(const uint64_t* codewords, const GState* theta, const int* code,
                                                  int64_t ntheta, int64_t j0, int64_t nj, int per_thread, int P,
                                                  int nmax, int gmax, __int128* part, int64_t part_stride,
                                                  int64_t part_base, int* eps_o, int* p_o, int* m_o,
                                                  const int* gate, int* err) {
    if (gate && *gate == 0) return;  // no live state (block-uniform)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TPShared& sh = *reinterpret_cast<TPShared*>(smem_raw);
    uint64_t* const sa = reinterpret_cast<uint64_t*>(smem_raw + sizeof(TPShared));
    unsigned char* const pair_base = smem_raw + sizeof(TPShared) + pc::block_state_bytes(nmax);
    const int tid = threadIdx.x;
    int e = 0;
    const int64_t span = (int64_t)kTP * per_thread;
    const int64_t nblk = (nj + span - 1) / span;
    const int64_t items = ntheta * nblk;
    for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
        const int64_t a = item / nblk, cb = item % nblk;
        __syncthreads();  // previous item's use of sh is over
        if (tid == 0) {
            sh.live = code ? (code[a] >= 0) : 1;
            sh.n = theta[a].n;
            pc::BlockScalars& t0 = sh.bp.sc[0];
            t0.k = theta[a].k;
            t0.Q = theta[a].Q;
            t0.h = theta[a].h;
            t0.D1 = theta[a].D1;
            t0.D2 = theta[a].D2;
            for (int q = 0; q < 7; q++) {
                sh.bp.andm[q] = ~0ull;
                sh.bp.orm[q] = 0ull;
            }
        }
        const GState* g = theta + a;
        const int k0 = g->k;  // theta's own k, for p's correction
        uint64_t* const r0 = pc::block_state_rows(sa, nmax, 0);
        if (tid < nmax) {
            r0[tid] = g->J[tid];
            // transpose G: column c as a mask over rows < k
            const int n = g->n;
            uint64_t col = 0ull;
            if (tid < n)
                for (int r = 0; r < k0; r++) col |= ((g->G[r] >> tid) & 1ull) << r;
            r0[nmax + tid] = col;
        }
        __syncthreads();
        // the pair routine relies on a symmetric J (true of every state drawn
        // and projected by this library); anything else is refused
        bool asym = false;
        if (tid < k0 && k0 <= nmax)
            for (int r = 0; r < k0; r++) asym |= ((r0[tid] >> r) & 1ull) != ((r0[r] >> tid) & 1ull);
        asym = __syncthreads_or(asym) != 0;
        __int128 z[4] = {0, 0, 0, 0};
        const int n = sh.n;
        if (n > nmax || asym) e |= kErrArg;
        if (sh.live && !asym && n >= 1 && n <= nmax) {
            const int64_t jb = j0 + cb * span;
            const int64_t cnt = j0 + nj - jb < span ? j0 + nj - jb : span;
            // the shrinks that each of the block's codeword groups shares run once
            pc::block_prefix<kTP>(sh.bp, sa, nmax, codewords + (jb - j0), cnt, per_thread, n, pair_base);
            const pc::PairMem mem = pc::pair_mem(pair_base, nmax, kTP, tid);
            const int split1 = sh.bp.split1, split2a = sh.bp.split2[0], split2b = sh.bp.split2[1];
            for (int r = 0; r < per_thread; r++) {
                const int64_t j = jb + tid + (int64_t)kTP * r;
                const bool valid = j < j0 + nj;
                if (__all_sync(kFull, !valid)) break;  // warp-uniform exit
                const uint64_t x = valid ? codewords[j - j0] : 0ull;
                const int gr = pc::block_group(split1, split2a, split2b, x);
                const pc::BlockScalars& st = sh.bp.sc[gr];
                const uint64_t* rows = pc::block_state_rows(sa, nmax, gr);
                int eps = 0, pp = 0, mm = 0;
                pc::pair_l(valid && !st.dead, n, st.k, st.Q, st.h, st.D1, st.D2, rows, rows + nmax, x, mem, eps, pp,
                           mm, e, gmax, st.done, k0);
                if (!valid) continue;
                pc::zacc(z, eps, pp, mm, P, e);
                if (eps_o) {
                    const int64_t w = a * nj + (j - j0);
                    eps_o[w] = eps;
                    p_o[w] = pp;
                    m_o[w] = mm;
                }
            }
        }
        if (part) {  // warp sums by shuffles, then the block's warps
            for (int q = 0; q < 4; q++)
                for (int o = 16; o > 0; o >>= 1) z[q] += shfl_xor_i128(z[q], o);
            if ((tid & 31) == 0)
                for (int q = 0; q < 4; q++) sh.red[tid >> 5][q] = z[q];
            __syncthreads();
            if (tid < 4 && sh.live) {  // a dead state's partials stay zero (another launch may own them)
                __int128 acc = 0;
                for (int w = 0; w < kTP / 32; w++) acc += sh.red[w][tid];
                part[4 * (a * part_stride + part_base + cb) + tid] = acc;
            }
        }
    }
    e = (int)__reduce_or_sync(kFull, (unsigned)e);
    if (e && (tid & 31) == 0) atomicOr(err, e);
}

// ---------------------------------------------------------------- direct restriction
// k_canon: one thread per state, theta in pivot coordinates (pc::canon_theta);
// states whose d = n - k exceeds `dslots` are left to the block-prefix kernel
// (code_direct < 0), the others to the direct kernel (code_rest < 0).
using pc::CanonG;

__global__ void __launch_bounds__(64) k_canon(const GState* theta, const int* code, int64_t ntheta, int dslots,
                                               CanonG* out, int* code_direct, int* code_rest, int* rest_count) {
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= ntheta) return;
    const GState* g = theta + a;
    const int c = code ? code[a] : 0;
    const int n = g->n, k = g->k;
    const bool direct = c >= 0 && n - k <= dslots && n >= 1 && n <= 64 && k >= 0 && k <= n;
    code_direct[a] = direct ? c : -1;
    code_rest[a] = direct ? -1 : c;
    if (rest_count && !direct && c >= 0) atomicAdd(rest_count, 1);
    if (!direct) return;
    uint64_t G[64], J[64];
    for (int r = 0; r < k; r++) {
        G[r] = g->G[r];
        J[r] = g->J[r];
    }
    pc::canon_theta(n, k, g->Q, g->h, g->D1, g->D2, G, J, out[a].Jc, out[a].acol, out[a].cs);
}

// The direct kernel: one thread per (theta, term) pair like k_terms_tp, each
// pair by pc::pair_direct from its state's pivot form, which a block loads
// into shared memory once per item.  The per-pair working memory needs no
// G slot per zero, only dslots constraint slots.
struct DirectShared {
    pc::Canon cs;
    int live, pad0, pad1, pad2;
    __int128 red[kTP / 32][4];
};

__global__ void __launch_bounds__(kTP) k_terms_direct(const uint64_t* codewords, const CanonG* canon, const int* code,
                                                      int64_t ntheta, int64_t j0, int64_t nj, int per_thread, int P,
                                                      int nmax, int rows, int dslots, __int128* part,
                                                      int64_t part_stride, int64_t part_base, int* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    DirectShared& sh = *reinterpret_cast<DirectShared*>(smem_raw);
    uint64_t* const sJ = reinterpret_cast<uint64_t*>(smem_raw + sizeof(DirectShared));  // 64 rows, then 64 masks
    uint64_t* const sA = sJ + 64;
    unsigned char* const pair_base = smem_raw + sizeof(DirectShared) + 2 * 64 * 8;
    const int tid = threadIdx.x;
    int e = 0;
    const pc::PairMem mem = pc::pair_mem(pair_base, rows, kTP, tid);
    const int64_t span = (int64_t)kTP * per_thread;
    const int64_t nblk = (nj + span - 1) / span;
    const int64_t items = ntheta * nblk;
    for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
        const int64_t a = item / nblk, cb = item % nblk;
        __syncthreads();  // previous item's use of the shared state is over
        if (tid == 0) {
            sh.live = code[a] >= 0;
            sh.cs = canon[a].cs;
        }
        sJ[tid] = canon[a].Jc[tid];
        sA[tid] = canon[a].acol[tid];
        __syncthreads();
        __int128 z[4] = {0, 0, 0, 0};
        const int n = sh.cs.n;
        if (sh.live && n > nmax) e |= kErrArg;
        if (sh.live && n >= 1 && n <= nmax) {
            const int64_t jb = j0 + cb * span;
            for (int r = 0; r < per_thread; r++) {
                const int64_t j = jb + tid + (int64_t)kTP * r;
                const bool valid = j < j0 + nj;
                if (__all_sync(kFull, !valid)) break;  // warp-uniform exit
                const uint64_t x = valid ? codewords[j - j0] : 0ull;
                int eps = 0, pp = 0, mm = 0;
                pc::pair_direct(valid, n, sh.cs, sJ, sA, x, mem, eps, pp, mm, e, dslots, sh.cs.k, rows);
                if (valid) pc::zacc(z, eps, pp, mm, P, e);
            }
        }
        if (part) {
            for (int q = 0; q < 4; q++)
                for (int o = 16; o > 0; o >>= 1) z[q] += shfl_xor_i128(z[q], o);
            if ((tid & 31) == 0)
                for (int q = 0; q < 4; q++) sh.red[tid >> 5][q] = z[q];
            __syncthreads();
            if (tid < 4 && sh.live) {
                __int128 acc = 0;
                for (int w = 0; w < kTP / 32; w++) acc += sh.red[w][tid];
                part[4 * (a * part_stride + part_base + cb) + tid] = acc;
            }
        }
    }
    e = (int)__reduce_or_sync(kFull, (unsigned)e);
    if (e && (tid & 31) == 0) atomicOr(err, e);
}

size_t canon_bytes() { return sizeof(CanonG); }

int launch_canon(const Launch& L, const GState* theta, const int* code, int64_t ntheta, int dslots, void* canon,
                 int* code_direct, int* code_rest, int* rest_count) {
    if (ntheta <= 0) return 0;
    const int64_t blocks = (ntheta + 63) / 64;
    k_canon<<<(int)blocks, 64, 0, L.stream>>>(theta, code, ntheta, dslots, (CanonG*)canon, code_direct, code_rest,
                                               rest_count);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

namespace {
size_t terms_direct_smem(int nmax, int dslots) {
    return sizeof(DirectShared) + 2 * 64 * 8 + pc::pair_mem_bytes(nmax, dslots, kTP);
}
}  // namespace

int launch_terms_direct(const Launch& L, int nmax, int rows, int dslots, const uint64_t* codewords,
                        const void* canon, const int* code, int64_t ntheta, int64_t j0, int64_t nj, int per_thread,
                        int P, __int128* part, int64_t part_stride, int64_t part_base) {
    if (ntheta <= 0 || nj <= 0) return 0;
    if (nmax < 1 || nmax > 64 || rows < 1 || rows > nmax || dslots < 0 || dslots > nmax || per_thread < 1 || !part ||
        !canon || !code)
        return -1;
    const int64_t span = (int64_t)kTP * per_thread;
    const int64_t nblk = (nj + span - 1) / span;
    if (part_stride < part_base + nblk) return -1;
    if (cudaFuncSetAttribute(k_terms_direct, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)terms_direct_smem(64, 64)) != cudaSuccess)
        return -1;
    const size_t smem = terms_direct_smem(rows, dslots);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_terms_direct, kTP, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int64_t grid = (int64_t)L.num_sms * per_sm;
    if (grid > ntheta * nblk) grid = ntheta * nblk;
    k_terms_direct<<<(int)grid, kTP, smem, L.stream>>>(codewords, (const CanonG*)canon, code, ntheta, j0, nj,
                                                        per_thread, P, nmax, rows, dslots, part, part_stride,
                                                        part_base, L.d_err);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// ---------------------------------------------------------------- per-thread runs
// The run kernel: codewords in runs of per_thread that agree on long top bits
// (run order, csim_host::run_ordered_codewords).  In a block's span of
// kTP * per_thread codewords, run r of thread t sits at positions t + kTP * i.
// Each thread shrinks theta once by its run's common zeros in the run's
// agreed top bits (pc::run_prefix, in its own region of the global scratch,
// [index][thread] like the shared-memory pair memory), then starts each of its
// pairs from that state (pc::pair_from_run).  No block-level prefix: a run of
// 32 codewords in numeric order agrees on about 11 top bits of a 16-row code
// at t = 40, against about 6 for a block of 2048.
struct RunShared {
    int n, live, k0, Q;
    uint64_t h, D1, D2;
    __int128 red[kTP / 32][4];
};

__global__ void __launch_bounds__(kTP) k_terms_runs(const uint64_t* codewords, const GState* theta, const int* code,
                                                    int64_t ntheta, int64_t j0, int64_t nj, int per_thread, int P,
                                                    int nmax, int gmax, __int128* part, int64_t part_stride,
                                                    int64_t part_base, unsigned char* scratch, int* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RunShared& sh = *reinterpret_cast<RunShared*>(smem_raw);
    uint64_t* const sJ = reinterpret_cast<uint64_t*>(smem_raw + sizeof(RunShared));  // theta's J rows, G columns
    uint64_t* const sGT = sJ + nmax;
    unsigned char* const pair_base = smem_raw + sizeof(RunShared) + (size_t)2 * nmax * 8;
    const int tid = threadIdx.x;
    int e = 0;
    const pc::PairMem mem = pc::pair_mem(pair_base, nmax, kTP, tid);
    const pc::PairMem rmem =
        pc::pair_mem(scratch + (size_t)blockIdx.x * pc::pair_mem_bytes(nmax, nmax, kTP), nmax, kTP, tid);
    const int64_t span = (int64_t)kTP * per_thread;
    const int64_t nblk = (nj + span - 1) / span;
    const int64_t items = ntheta * nblk;
    for (int64_t item = blockIdx.x; item < items; item += gridDim.x) {
        const int64_t a = item / nblk, cb = item % nblk;
        __syncthreads();  // previous item's use of the shared state is over
        const GState* g = theta + a;
        if (tid == 0) {
            sh.live = code ? (code[a] >= 0) : 1;
            sh.n = g->n;
            sh.k0 = g->k;
            sh.Q = g->Q;
            sh.h = g->h;
            sh.D1 = g->D1;
            sh.D2 = g->D2;
        }
        const int k0 = g->k;
        if (tid < nmax) {
            sJ[tid] = g->J[tid];
            const int n = g->n;
            uint64_t col = 0ull;
            if (tid < n)
                for (int r = 0; r < k0; r++) col |= ((g->G[r] >> tid) & 1ull) << r;
            sGT[tid] = col;
        }
        __syncthreads();
        bool asym = false;
        if (tid < k0 && k0 <= nmax)
            for (int r = 0; r < k0; r++) asym |= ((sJ[tid] >> r) & 1ull) != ((sJ[r] >> tid) & 1ull);
        asym = __syncthreads_or(asym) != 0;
        __int128 z[4] = {0, 0, 0, 0};
        const int n = sh.n;
        if (n > nmax || asym) e |= kErrArg;
        if (sh.live && !asym && n >= 1 && n <= nmax) {
            const int64_t jb = j0 + cb * span;
            // this thread's run: positions jb + tid + kTP * i
            uint64_t am = ~0ull, om = 0ull;
            bool any = false;
            for (int i = 0; i < per_thread; i++) {
                const int64_t j = jb + tid + (int64_t)kTP * i;
                if (j < j0 + nj) {
                    const uint64_t x = codewords[j - j0];
                    am &= x;
                    om |= x;
                    any = true;
                }
            }
            const uint64_t pm = pc::agree_top(am ^ om, n);
            pc::RunState rs;
            pc::run_prefix(any, n, pm, am, sh.k0, sh.Q, sh.h, sh.D1, sh.D2, sJ, sGT, rmem, rs);
            for (int i = 0; i < per_thread; i++) {
                const int64_t j = jb + tid + (int64_t)kTP * i;
                const bool valid = j < j0 + nj;
                if (__all_sync(kFull, !valid)) break;  // warp-uniform exit
                const uint64_t x = valid ? codewords[j - j0] : 0ull;
                int eps = 0, pp = 0, mm = 0;
                pc::pair_from_run(valid, n, rs, rmem, x, mem, eps, pp, mm, e, gmax, k0);
                if (valid) pc::zacc(z, eps, pp, mm, P, e);
            }
        }
        if (part) {
            for (int q = 0; q < 4; q++)
                for (int o = 16; o > 0; o >>= 1) z[q] += shfl_xor_i128(z[q], o);
            if ((tid & 31) == 0)
                for (int q = 0; q < 4; q++) sh.red[tid >> 5][q] = z[q];
            __syncthreads();
            if (tid < 4) {
                __int128 acc = 0;
                for (int w = 0; w < kTP / 32; w++) acc += sh.red[w][tid];
                part[4 * (a * part_stride + part_base + cb) + tid] = acc;
            }
        }
    }
    e = (int)__reduce_or_sync(kFull, (unsigned)e);
    if (e && (tid & 31) == 0) atomicOr(err, e);
}

namespace {
size_t terms_runs_smem(int nmax, int gmax) {
    return sizeof(RunShared) + (size_t)2 * nmax * 8 + pc::pair_mem_bytes(nmax, gmax, kTP);
}
int terms_runs_grid(const Launch& L, int nmax, int gmax, int64_t items) {
    if (cudaFuncSetAttribute(k_terms_runs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)terms_runs_smem(64, 64)) != cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_terms_runs, kTP, terms_runs_smem(nmax, gmax)) !=
            cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    int64_t grid = (int64_t)L.num_sms * per_sm;
    if (grid > items) grid = items;
    return (int)grid;
}
}  // namespace

size_t terms_runs_scratch_bytes(int num_sms, int nmax, int gmax) {
    Launch L{nullptr, nullptr, nullptr, num_sms};
    const int grid = terms_runs_grid(L, nmax, gmax, (int64_t)1 << 40);
    return grid < 1 ? 0 : (size_t)grid * pc::pair_mem_bytes(nmax, nmax, kTP);
}

int launch_terms_runs(const Launch& L, int nmax, int gmax, const uint64_t* codewords, const GState* theta,
                      const int* code, int64_t ntheta, int64_t j0, int64_t nj, int per_thread, int P, __int128* part,
                      int64_t part_stride, int64_t part_base, unsigned char* scratch, size_t scratch_bytes) {
    if (ntheta <= 0 || nj <= 0) return 0;
    if (nmax < 1 || nmax > 64 || gmax < 0 || gmax > nmax || per_thread < 1 || !scratch || !part) return -1;
    const int64_t span = (int64_t)kTP * per_thread;
    const int64_t nblk = (nj + span - 1) / span;
    if (part_stride < part_base + nblk) return -1;
    const int grid = terms_runs_grid(L, nmax, gmax, ntheta * nblk);
    if (grid < 1 || (size_t)grid * pc::pair_mem_bytes(nmax, nmax, kTP) > scratch_bytes) return -1;
    k_terms_runs<<<grid, kTP, terms_runs_smem(nmax, gmax), L.stream>>>(codewords, theta, code, ntheta, j0, nj,
                                                                       per_thread, P, nmax, gmax, part, part_stride,
                                                                       part_base, scratch, L.d_err);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t terms_tp_smem(int nmax, int gmax) {
    return sizeof(TPShared) + pc::block_state_bytes(nmax) + pc::pair_mem_bytes(nmax, gmax, kTP);
}

int launch_terms_tp(const Launch& L, int nmax, int gmax, const uint64_t* codewords, const GState* theta,
                    const int* code, int64_t ntheta, int64_t j0, int64_t nj, int per_thread, int P, __int128* part,
                    int64_t part_stride, int64_t part_base, int* eps_o, int* p_o, int* m_o, const int* gate) {
    if (ntheta <= 0 || nj <= 0) return 0;
    if (nmax < 1 || nmax > 64 || gmax < 0 || gmax > nmax) return -1;
    const int64_t span = (int64_t)kTP * per_thread;
    const int64_t nblk = (nj + span - 1) / span;
    if (part && part_stride < part_base + nblk) return -1;
    const size_t smem = terms_tp_smem(nmax, gmax);
    if (cudaFuncSetAttribute(k_terms_tp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)terms_tp_smem(64, 64)) !=
        cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_terms_tp, kTP, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int64_t items = ntheta * nblk;
    int64_t grid = (int64_t)L.num_sms * per_sm;
    if (grid > items) grid = items;
    k_terms_tp<<<(int)grid, kTP, smem, L.stream>>>(codewords, theta, code, ntheta, j0, nj, per_thread, P, nmax, gmax,
                                                    part, part_stride, part_base, eps_o, p_o, m_o, gate, L.d_err);
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int terms_tp_occupancy(int nmax, int gmax) {
    if (cudaFuncSetAttribute(k_terms_tp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)terms_tp_smem(64, 64)) !=
        cudaSuccess)
        return -1;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_terms_tp, kTP, terms_tp_smem(nmax, gmax)) !=
        cudaSuccess)
        return -1;
    return per_sm;
}

int64_t terms_tp_blocks(int64_t nj, int per_thread) {
    const int64_t span = (int64_t)kTP * per_thread;
    return (nj + span - 1) / span;
}

}  // namespace csim
