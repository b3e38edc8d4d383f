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
// k_canon: one warp per state, theta in pivot coordinates: pc::canon_theta's
// steps with lane l holding variables l and l + 32 (rows of G and J), the
// pivot step's row set B a ballot and its rank-two update done by every lane
// on its own rows; states whose d = n - k exceeds `dslots` are left to the
// block-prefix kernel (code_direct < 0), the others to the direct kernel
// (code_rest < 0).
using pc::CanonG;

namespace {
__device__ __forceinline__ uint64_t shfl_xor_u64(uint64_t v, int m) {
    const uint32_t lo = __shfl_xor_sync(kFull, (uint32_t)v, m), hi = __shfl_xor_sync(kFull, (uint32_t)(v >> 32), m);
    return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ uint64_t ballot64(bool lo, bool hi) {
    return (uint64_t)__ballot_sync(kFull, lo) | ((uint64_t)__ballot_sync(kFull, hi) << 32);
}
__device__ __forceinline__ uint64_t xor_reduce64(uint64_t v) {
    for (int o = 16; o > 0; o >>= 1) v ^= shfl_xor_u64(v, o);
    return v;
}
__device__ __forceinline__ uint64_t or_reduce64(uint64_t v) {
    for (int o = 16; o > 0; o >>= 1) v |= shfl_xor_u64(v, o);
    return v;
}
// coordinate-indexed mask of a variable-indexed one (variable a -> its pivot coordinate)
__device__ __forceinline__ uint64_t to_coords(uint64_t v, const unsigned char* piv) {
    uint64_t r = 0ull;
    while (v) {
        const int a = __ffsll((long long)v) - 1;
        v &= v - 1ull;
        r |= 1ull << piv[a];
    }
    return r;
}
}  // namespace

__global__ void __launch_bounds__(64) k_canon(const GState* theta, const int* code, int64_t ntheta, int dslots,
                                               CanonG* out, int* code_direct, int* code_rest, int* rest_count) {
    __shared__ unsigned char piv_s[2][64];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    unsigned char* const piv = piv_s[wib];
    const int64_t a0 = (int64_t)blockIdx.x * 2 + wib;  // this warp's state
    if (a0 >= ntheta) return;                          // warp-uniform
    const GState* g = theta + a0;
    const int c = code ? code[a0] : 0;
    const int n = g->n, k = g->k;
    const bool direct = c >= 0 && n - k <= dslots && n >= 1 && n <= 64 && k >= 0 && k <= n;
    if (lane == 0) {
        code_direct[a0] = direct ? c : -1;
        code_rest[a0] = direct ? -1 : c;
        if (rest_count && !direct && c >= 0) atomicAdd(rest_count, 1);
    }
    if (!direct) return;  // warp-uniform
    CanonG& o = out[a0];
    const uint64_t nm = pc::lowmask(n), km = pc::lowmask(k);
    const int r0 = lane, r1 = lane + 32;  // this lane's variables
    uint64_t g0 = r0 < k ? g->G[r0] & nm : 0ull, g1 = r1 < k ? g->G[r1] & nm : 0ull;
    uint64_t j0 = r0 < k ? g->J[r0] & km : 0ull, j1 = r1 < k ? g->J[r1] & km : 0ull;
    uint64_t D1 = g->D1 & km, D2 = g->D2 & km;
    int p0 = 0, p1 = 0;
    // Gauss-Jordan on the rows of G: rows b of B += row a (u_a = u'_a + u'_b), J <- R J R^T with
    // rows in B getting J_a and rows in C getting B, D_b += D_a + 4 J_ab (pc::canon_theta)
    for (int a = 0; a < k; a++) {
        const int src = a & 31;
        const bool up = a >= 32;
        const uint64_t ga = shfl64(up ? g1 : g0, src);
        const int pcol = ga ? __ffsll((long long)ga) - 1 : 0;
        if (lane == src) {
            if (up) p1 = pcol;
            else p0 = pcol;
        }
        const bool in0 = r0 < k && r0 != a && ((g0 >> pcol) & 1ull), in1 = r1 < k && r1 != a && ((g1 >> pcol) & 1ull);
        const uint64_t B = ballot64(in0, in1);
        if (!B) continue;  // warp-uniform
        if (in0) g0 ^= ga;
        if (in1) g1 ^= ga;
        const uint64_t Ja = shfl64(up ? j1 : j0, src);
        const uint64_t C = Ja ^ (((Ja >> a) & 1ull) ? B : 0ull);
        j0 ^= (((B >> r0) & 1ull) ? Ja : 0ull) ^ (((C >> r0) & 1ull) ? B : 0ull);
        j1 ^= (((B >> r1) & 1ull) ? Ja : 0ull) ^ (((C >> r1) & 1ull) ? B : 0ull);
        pc::add_D64(D1, D2, B, (int)((D1 >> a) & 1ull), (int)((D2 >> a) & 1ull));
        D2 ^= B & Ja;
    }
    // shift v = u + w, w_a = h at a's pivot: in order of a, Q += D_a and D_a -> -D_a, D_b += 4 J_ab;
    // D_a as read at step a carries the earlier steps' flips J_{a'a}, a' < a in w
    const bool w0 = r0 < k && ((g->h >> p0) & 1ull), w1 = r1 < k && ((g->h >> p1) & 1ull);
    const uint64_t wv = ballot64(w0, w1);
    int dq = 0;
    if (w0) dq += 2 * (2 * (int)(((D2 >> r0) ^ (uint64_t)__popcll(j0 & wv & pc::lowmask(r0))) & 1ull) +
                       (int)((D1 >> r0) & 1ull));
    if (w1) dq += 2 * (2 * (int)(((D2 >> r1) ^ (uint64_t)__popcll(j1 & wv & pc::lowmask(r1))) & 1ull) +
                       (int)((D1 >> r1) & 1ull));
    dq = (int)__reduce_add_sync(kFull, (unsigned)dq);
    const uint64_t flips = xor_reduce64((w0 ? j0 & ~(1ull << r0) : 0ull) ^ (w1 ? j1 & ~(1ull << r1) : 0ull));
    D2 ^= (D1 & wv) ^ (flips & km);
    // to coordinate indexing
    piv[r0] = (unsigned char)(r0 < k ? p0 : 0);
    piv[r1] = (unsigned char)(r1 < k ? p1 : 0);
    __syncwarp();
    const uint64_t P = or_reduce64((r0 < k ? 1ull << p0 : 0ull) | (r1 < k ? 1ull << p1 : 0ull));
    o.Jc[r0] = 0ull;
    o.Jc[r1] = 0ull;
    o.acol[r0] = 0ull;
    o.acol[r1] = 0ull;
    __syncwarp();
    if (r0 < k) o.Jc[p0] = to_coords(j0, piv);
    if (r1 < k) o.Jc[p1] = to_coords(j1, piv);
    // each non-pivot coordinate: the variables its coordinate depends on, and the constraint's bit
    uint64_t bm = 0ull;
    for (uint64_t np = ~P & nm; np;) {
        const int cc = __ffsll((long long)np) - 1;
        np &= np - 1ull;
        const uint64_t av = ballot64(r0 < k && ((g0 >> cc) & 1ull), r1 < k && ((g1 >> cc) & 1ull));
        if (lane == (cc & 31)) o.acol[cc] = to_coords(av, piv);
        if ((((g->h >> cc) & 1ull) ^ (uint64_t)(__popcll(wv & av) & 1)) != 0ull) bm |= 1ull << cc;
    }
    if (lane == 0) {
        pc::Canon cs;
        cs.P = P;
        cs.D1 = to_coords(D1, piv);
        cs.D2 = to_coords(D2, piv);
        cs.bm = bm;
        cs.Q = (g->Q + dq) & 7;
        cs.k = k;
        cs.n = n;
        cs.pad = 0;
        o.cs = cs;
    }
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
    const int64_t blocks = (ntheta + 1) / 2;  // a warp per state
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
