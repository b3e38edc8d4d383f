// csim_kernels.cu — sm_103a kernels of the stabilizer-rank estimator and
// their launchers.  Every kernel is warp-per-item (one stabilizer state or one
// (theta, term) pair per warp, csim_warp.cuh) with a grid-stride loop over
// items sized to the SM count.
#include <cuda_runtime.h>

#include <cstdint>

#include "csim_internal.h"
#include "csim_rng.cuh"
#include "csim_warp.cuh"

namespace csim {

__device__ __forceinline__ int64_t warp_global() {
    return ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ int64_t warp_count() { return ((int64_t)gridDim.x * blockDim.x) >> 5; }

__device__ __forceinline__ void flush_err(int e, int* err) {
    e = __reduce_or_sync(kFull, (unsigned)e);
    if (e && lane_id() == 0) atomicOr(err, e);
}

__device__ __forceinline__ bool n_ok(int n, int nr) { return n >= 1 && n <= 32 * nr; }

// ------------------------------------------------------------ batched primitives
template <int NR>
__global__ void __launch_bounds__(256) k_inner_product(const GState* a, const GState* b, int64_t count, int* eps,
                                                       int* p, int* m, int* err) {
    int e = 0;
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        WS<NR> s1, s2;
        load_state<NR>(a + i, s1);
        load_state<NR>(b + i, s2);
        int ee = 0, pp = 0, mm = 0;
        if (s1.n != s2.n || !n_ok(s1.n, NR)) e |= kErrArg;
        else inner_product<NR>(s1, s2, s1.k, ee, pp, mm, e);
        if (lane_id() == 0) {
            eps[i] = ee;
            p[i] = pp;
            m[i] = mm;
        }
    }
    flush_err(e, err);
}

template <int NR>
__global__ void __launch_bounds__(256) k_exp_sum(GState* s, int64_t count, int* eps, int* p, int* m, int* err) {
    int e = 0;
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        WS<NR> st;
        load_state<NR>(s + i, st);
        int ee = 0, pp = 0, mm = 0;
        if (!n_ok(st.n, NR)) e |= kErrArg;
        else exp_sum<NR>(st, ee, pp, mm, e);
        store_state<NR>(s + i, st);
        if (lane_id() == 0) {
            eps[i] = ee;
            p[i] = pp;
            m[i] = mm;
        }
    }
    flush_err(e, err);
}

template <int NR>
__global__ void __launch_bounds__(256) k_shrink(GState* s, const uint64_t* xi, const int* alpha, int lazy,
                                                int64_t count, int* status, int* err) {
    int e = 0;
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        WS<NR> st;
        load_state<NR>(s + i, st);
        int r = 0;
        if (!n_ok(st.n, NR)) e |= kErrArg;
        else if (lazy == 1) r = shrink<NR, true, true>(st, xi[i], alpha[i]);
        else r = shrink<NR, false, true>(st, xi[i], alpha[i]);
        store_state<NR>(s + i, st);
        if (lane_id() == 0) status[i] = r;
    }
    flush_err(e, err);
}

template <int NR>
__global__ void __launch_bounds__(256) k_measure(GState* s, const int* mm, const uint64_t* zeta, const uint64_t* xi,
                                                 int64_t count, int* code, int* err) {
    int e = 0;
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        WS<NR> st;
        load_state<NR>(s + i, st);
        int r = 0;
        if (!n_ok(st.n, NR)) e |= kErrArg;
        else {
            r = measure_pauli<NR>(st, mm[i], zeta[i], xi[i]);
            if (r < 0) e |= kErrRange;
        }
        store_state<NR>(s + i, st);
        if (lane_id() == 0) code[i] = r;
    }
    flush_err(e, err);
}

template <int NR>
__global__ void __launch_bounds__(256) k_extend(GState* s, const uint64_t* xi, int64_t count, int* err) {
    int e = 0;
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        WS<NR> st;
        load_state<NR>(s + i, st);
        if (!n_ok(st.n, NR)) e |= kErrArg;
        else extend<NR>(st, xi[i]);
        store_state<NR>(s + i, st);
    }
    flush_err(e, err);
}

// ------------------------------------------------------------ theta generation
template <int NR>
__global__ void __launch_bounds__(256) k_random_states(int n, int64_t count, int mode, uint64_t seed, uint64_t first,
                                                       const uint32_t* words, const int64_t* offsets,
                                                       const double* cum, GState* out, int64_t* consumed, int* err) {
    int e = 0;
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        DevRng rng;
        rng.mode = mode;
        rng.k0 = (uint32_t)seed;
        rng.k1 = (uint32_t)(seed >> 32);
        rng.id0 = (uint32_t)(first + i);
        rng.id1 = (uint32_t)((first + i) >> 32);
        rng.words = words;
        rng.base = mode == 1 ? offsets[i] : 0;
        rng.end = mode == 1 ? offsets[i + 1] : 0;
        rng.cur = 0;
        WS<NR> st;
        random_state<NR>(st, n, rng, cum, e);
        store_state<NR>(out + i, st);
        if (consumed && lane_id() == 0) consumed[i] = rng.cur;
    }
    flush_err(e, err);
}

// project each state onto P (innerprod.c:97-116); code = number of 2^{-1/2}
// factors, or -1 when a measurement annihilates the state
template <int NR>
__global__ void __launch_bounds__(256) k_project(GState* s, int64_t count, int nstabs, const int* mm,
                                                 const uint64_t* zeta, const uint64_t* xi, int* code, int* err) {
    int e = 0;
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        WS<NR> st;
        load_state<NR>(s + i, st);
        int c = 0;
        for (int r = 0; r < nstabs; r++) {
            const int res = measure_pauli<NR>(st, mm[r], zeta[r], xi[r]);
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
        store_state<NR>(s + i, st);
        if (lane_id() == 0) code[i] = c;
    }
    flush_err(e, err);
}

// ------------------------------------------------------------ decomposition terms
// prepH (stateprep.c:36-81): bit j of the ceil(t/2)-bit index, MSB first
template <int NR>
__device__ void prep_h(WS<NR>& s, int t, int64_t idx) {
    const int size = (t + 1) / 2;
    init_identity<NR>(s, t);
#pragma unroll
    for (int sl = 0; sl < NR; sl++) {
        const int x = row_of<NR>(sl);
        if (x < t) {
            const int j = x / 2;
            const int bit = (int)((idx >> (size - 1 - j)) & 1);
            if (bit == 0 && !((t % 2) && j == size - 1)) s.J[sl] |= bit1(x ^ 1);
        }
    }
    for (int j = 0; j < size; j++) {
        const int bit = (int)((idx >> (size - 1 - j)) & 1);
        if ((t % 2) && j == size - 1) {
            if (bit == 1) shrink<NR, false, true>(s, bit1(t - 1), 0);
            continue;
        }
        if (bit == 1) shrink<NR, false, true>(s, bit1(2 * j + 1) | bit1(2 * j), 0);
    }
}

// prepL (stateprep.c:85-120) from the codeword x of the term
template <int NR>
__device__ void prep_l(WS<NR>& s, int t, uint64_t x) {
    init_identity<NR>(s, t);
    for (int idx = 0; idx < t; idx++)
        if (!getbit(x, idx)) shrink_unit<NR, true>(s, idx);
}

// codeword of term j: rows r of L with bit (k-1-r) of j set (binrep, stateprep.c:5-32)
__global__ void k_codewords(const uint64_t* L, int k, int64_t j0, int64_t count, uint64_t* out) {
    __shared__ uint64_t sL[64];
    if (threadIdx.x < 64) sL[threadIdx.x] = threadIdx.x < (unsigned)k ? L[threadIdx.x] : 0ull;
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = j0 + i;
        uint64_t x = 0ull;
        for (int r = 0; r < k; r++)
            if ((j >> (k - 1 - r)) & 1) x ^= sL[r];
        out[i] = x;
    }
}

template <int NR>
__global__ void __launch_bounds__(256) k_prep(int t, int exact, const uint64_t* codewords, const int64_t* idx,
                                              int64_t count, GState* out) {
    for (int64_t i = warp_global(); i < count; i += warp_count()) {
        WS<NR> st;
        if (exact) prep_h<NR>(st, t, idx[i]);
        else prep_l<NR>(st, t, codewords[i]);
        store_state<NR>(out + i, st);
    }
}

// decompose()'s fidelity sum (probability.c:391-398): Z(L) = sum over the 2^k
// codewords x of 2^(-|x|/2), |x|/2 in integer division.  Terms are powers of
// two, so the sum is taken exactly as the integer sum of 2^(S - |x|/2),
// S = floor(t/2), in 128 bits; the order of the codewords does not matter.
// Each thread walks a contiguous range of Gray-code indices, so consecutive
// codewords differ by one row of L.  One 128-bit partial per block.
__global__ void __launch_bounds__(256) k_fidelity_sum(const uint64_t* L, int k, int S, int64_t per_thread,
                                                      unsigned __int128* part) {
    __shared__ uint64_t sL[64];
    __shared__ unsigned __int128 red[8];
    if (threadIdx.x < 64) sL[threadIdx.x] = threadIdx.x < (unsigned)k ? L[threadIdx.x] : 0ull;
    __syncthreads();
    const int64_t total = (int64_t)1 << k;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t i0 = tid * per_thread;
    unsigned __int128 acc = 0;
    if (i0 < total) {
        const int64_t i1 = i0 + per_thread < total ? i0 + per_thread : total;
        // codeword of Gray index g = i0 ^ (i0 >> 1): bit b of g selects row k-1-b
        const uint64_t g = (uint64_t)(i0 ^ (i0 >> 1));
        uint64_t x = 0;
        for (int b = 0; b < k; b++)
            if ((g >> b) & 1) x ^= sL[k - 1 - b];
        for (int64_t i = i0; i < i1; i++) {
            acc += (unsigned __int128)1 << (S - __popcll(x) / 2);
            const int b = __ffsll((long long)(i + 1)) - 1;  // Gray code i -> i+1 flips bit ctz(i+1)
            if (b < k) x ^= sL[k - 1 - b];
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t lo = (uint64_t)acc, hi = (uint64_t)(acc >> 64);
        acc += ((unsigned __int128)__shfl_xor_sync(kFull, hi, o) << 64) | __shfl_xor_sync(kFull, lo, o);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned __int128 s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
        part[blockIdx.x] = s;
    }
}

// ------------------------------------------------------------ the hot loop
// Adds eps 2^{p/2} w^m, scaled by 2^{P/2}, to z = z0 + z1 w + z2 w^2 + z3 w^3
// (w = e^{i pi/4}); sqrt 2 = w - w^3.  The reference's p lies in [-2n, n]
// (p = p_expsum - k1 - k2 with 0 <= p_expsum <= 2 k' and k' <= k1), so with
// P = 2n every term is an integer below 2^{3n/2} <= 2^96 and a sum of up
// to 2^30 terms is exact in 128 bits.
__device__ __forceinline__ void zacc(__int128 (&z)[4], int eps, int p, int m, int P, int& err) {
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

// One (theta, prepL term) pair.  For terms of |L> the second state of
// innerProductExact is a product of |0> and |+>: its Gbar rows k2..n-1 are
// e_q for the zero bits q of the codeword in descending order, its h, Q, D
// and J are zero, so the R stage of stabilizer.c:611-652 changes nothing and
// the pair reduces to shrinks by e_q (alpha = 0) and one exponential sum.
template <int NR>
__device__ __forceinline__ void pair_l(WS<NR> st, uint64_t x, int& eps, int& p, int& m, int& err) {
    const int k1 = st.k, k2 = __popcll(x);
    uint64_t zeros = ~x & lowmask(st.n);
    while (zeros) {
        const int q = 63 - __clzll((long long)zeros);
        zeros &= ~bit1(q);
        eps = shrink_unit<NR, false>(st, q);
        if (eps == 0) {
            p = 0;
            m = 0;
            return;
        }
    }
    exp_sum<NR>(st, eps, p, m, err);
    p -= k1 + k2;
}

// Pairs <theta_a | phi_j>, a < ntheta, j in [j0, j0+nj).
// MODE 0: phi_j = prepL term from codewords[j - j0] (fast path);
// MODE 1: phi_j = phis[j - j0] (any state, full innerProductExact);
// MODE 2: exactProjector rows: theta_a = projected phi_a, j >= a only,
//         the j == a term goes to part_diag, the rest to part.
// Work item = (theta a, chunk c of `chunk` consecutive terms); the partial sums
// part[4 * item .. +4) must be zeroed before the launch (skipped items leave 0).
template <int NR, int MODE>
__global__ void __launch_bounds__(256) k_terms(const uint64_t* codewords, const GState* phis, const GState* theta,
                                               const int* code, int64_t ntheta, int64_t j0, int64_t nj, int chunk,
                                               int P, __int128* part, __int128* part_diag, int* eps_o, int* p_o,
                                               int* m_o, int* err) {
    int e = 0;
    const int64_t nchunks = (nj + chunk - 1) / chunk;
    const int64_t items = ntheta * nchunks;
    for (int64_t item = warp_global(); item < items; item += warp_count()) {
        const int64_t a = item / nchunks, c = item % nchunks;
        int64_t jb = j0 + c * chunk;
        const int64_t je = jb + chunk < j0 + nj ? jb + chunk : j0 + nj;
        if (MODE == 2 && jb < a) jb = a;
        if (jb >= je) continue;
        if (code && code[a] < 0) continue;
        WS<NR> base;
        load_state<NR>(theta + a, base);
        if (!n_ok(base.n, NR)) {
            e |= kErrArg;
            continue;
        }
        __int128 z[4] = {0, 0, 0, 0}, zd[4] = {0, 0, 0, 0};
        for (int64_t j = jb; j < je; j++) {
            int ee = 0, pp = 0, mm = 0;
            if (MODE == 0) {
                pair_l<NR>(base, codewords[j - j0], ee, pp, mm, e);
            } else {
                WS<NR> phi;
                load_state<NR>(phis + (j - j0), phi);
                inner_product<NR>(base, phi, base.k, ee, pp, mm, e);
            }
            if (MODE == 2 && j == a) zacc(zd, ee, pp, mm, P, e);
            else zacc(z, ee, pp, mm, P, e);
            if (eps_o && lane_id() == 0) {
                const int64_t w = a * nj + (j - j0);
                eps_o[w] = ee;
                p_o[w] = pp;
                m_o[w] = mm;
            }
        }
        // one partial sum per work item; k_reduce_parts adds them per theta (no atomics, deterministic)
        if (lane_id() == 0) {
            if (part)
                for (int q = 0; q < 4; q++) part[4 * item + q] = z[q];
            if (MODE == 2 && part_diag)
                for (int q = 0; q < 4; q++) part_diag[4 * item + q] = zd[q];
        }
    }
    flush_err(e, err);
}

// per-theta sums of the per-item partials: acc[4a+q] = sum_c part[4(a*nchunks+c)+q]
__global__ void k_reduce_parts(const __int128* part, int64_t ntheta, int64_t nchunks, __int128* acc) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < ntheta * 4;
         w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = w / 4, q = w % 4;
        __int128 s = 0;
        for (int64_t c = 0; c < nchunks; c++) s += part[4 * (a * nchunks + c) + q];
        acc[w] = s;
    }
}

// ------------------------------------------------------------ launchers
namespace {

int grid_for(const Launch& L, int64_t warps_needed) {
    const int64_t blocks = (warps_needed + 7) / 8;
    const int64_t cap = (int64_t)L.num_sms * 8;
    int64_t g = blocks < cap ? blocks : cap;
    return (int)(g < 1 ? 1 : g);
}

int post(const Launch& L) {
    (*L.launches)++;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

#define CSIM_DISPATCH(nr, call) ((nr) == 1 ? (call<1>) : (call<2>))

int launch_inner_product(const Launch& L, int nr, const GState* a, const GState* b, int64_t count, int* eps, int* p,
                         int* m) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (nr == 1) k_inner_product<1><<<g, 256, 0, L.stream>>>(a, b, count, eps, p, m, L.d_err);
    else k_inner_product<2><<<g, 256, 0, L.stream>>>(a, b, count, eps, p, m, L.d_err);
    return post(L);
}

int launch_exp_sum(const Launch& L, int nr, GState* s, int64_t count, int* eps, int* p, int* m) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (nr == 1) k_exp_sum<1><<<g, 256, 0, L.stream>>>(s, count, eps, p, m, L.d_err);
    else k_exp_sum<2><<<g, 256, 0, L.stream>>>(s, count, eps, p, m, L.d_err);
    return post(L);
}

int launch_shrink(const Launch& L, int nr, GState* s, const uint64_t* xi, const int* alpha, int lazy, int64_t count,
                  int* status) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (nr == 1) k_shrink<1><<<g, 256, 0, L.stream>>>(s, xi, alpha, lazy, count, status, L.d_err);
    else k_shrink<2><<<g, 256, 0, L.stream>>>(s, xi, alpha, lazy, count, status, L.d_err);
    return post(L);
}

int launch_measure(const Launch& L, int nr, GState* s, const int* m, const uint64_t* zeta, const uint64_t* xi,
                   int64_t count, int* code) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (nr == 1) k_measure<1><<<g, 256, 0, L.stream>>>(s, m, zeta, xi, count, code, L.d_err);
    else k_measure<2><<<g, 256, 0, L.stream>>>(s, m, zeta, xi, count, code, L.d_err);
    return post(L);
}

int launch_extend(const Launch& L, int nr, GState* s, const uint64_t* xi, int64_t count) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (nr == 1) k_extend<1><<<g, 256, 0, L.stream>>>(s, xi, count, L.d_err);
    else k_extend<2><<<g, 256, 0, L.stream>>>(s, xi, count, L.d_err);
    return post(L);
}

int launch_random_states(const Launch& L, int n, int64_t count, int mode, uint64_t seed, uint64_t first,
                         const uint32_t* words, const int64_t* offsets, const double* cum, GState* out,
                         int64_t* consumed) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (n <= 32)
        k_random_states<1><<<g, 256, 0, L.stream>>>(n, count, mode, seed, first, words, offsets, cum, out, consumed,
                                                     L.d_err);
    else
        k_random_states<2><<<g, 256, 0, L.stream>>>(n, count, mode, seed, first, words, offsets, cum, out, consumed,
                                                     L.d_err);
    return post(L);
}

int launch_project(const Launch& L, int nr, GState* s, int64_t count, int nstabs, const int* m, const uint64_t* zeta,
                   const uint64_t* xi, int* code) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (nr == 1) k_project<1><<<g, 256, 0, L.stream>>>(s, count, nstabs, m, zeta, xi, code, L.d_err);
    else k_project<2><<<g, 256, 0, L.stream>>>(s, count, nstabs, m, zeta, xi, code, L.d_err);
    return post(L);
}

int launch_codewords(const Launch& L, const uint64_t* Ld, int k, int64_t j0, int64_t count, uint64_t* out) {
    if (count <= 0) return 0;
    int64_t blocks = (count + 255) / 256;
    if (blocks > (int64_t)L.num_sms * 16) blocks = (int64_t)L.num_sms * 16;
    k_codewords<<<(int)blocks, 256, 0, L.stream>>>(Ld, k, j0, count, out);
    return post(L);
}

int launch_prep(const Launch& L, int t, int exact, const uint64_t* codewords, const int64_t* idx, int64_t count,
                GState* out) {
    if (count <= 0) return 0;
    const int g = grid_for(L, count);
    if (t <= 32) k_prep<1><<<g, 256, 0, L.stream>>>(t, exact, codewords, idx, count, out);
    else k_prep<2><<<g, 256, 0, L.stream>>>(t, exact, codewords, idx, count, out);
    return post(L);
}

int launch_fidelity_sum(const Launch& L, const uint64_t* Ld, int k, int S, unsigned __int128* part, int* nblocks) {
    if (k < 0 || k > 40 || S < 0 || S > 32) return -1;
    const int64_t total = (int64_t)1 << k;
    const int64_t threads = (int64_t)L.num_sms * 2048;
    int64_t per_thread = (total + threads - 1) / threads;
    if (per_thread < 1) per_thread = 1;
    const int64_t nthreads = (total + per_thread - 1) / per_thread;
    const int64_t blocks = (nthreads + 255) / 256;
    *nblocks = (int)blocks;
    k_fidelity_sum<<<(int)blocks, 256, 0, L.stream>>>(Ld, k, S, per_thread, part);
    return post(L);
}

int launch_terms(const Launch& L, int nr, int mode, const uint64_t* codewords, const GState* phis,
                 const GState* theta, const int* code, int64_t ntheta, int64_t j0, int64_t nj, int chunk, int P,
                 __int128* part, __int128* part_diag, int* eps_o, int* p_o, int* m_o) {
    if (ntheta <= 0 || nj <= 0) return 0;
    const int64_t items = ntheta * ((nj + chunk - 1) / chunk);
    const int g = grid_for(L, items);
#define CSIM_TERMS(NRV, MV)                                                                                   \
    k_terms<NRV, MV><<<g, 256, 0, L.stream>>>(codewords, phis, theta, code, ntheta, j0, nj, chunk, P, part, \
                                              part_diag, eps_o, p_o, m_o, L.d_err)
    if (nr == 1) {
        if (mode == 0) CSIM_TERMS(1, 0);
        else if (mode == 1) CSIM_TERMS(1, 1);
        else CSIM_TERMS(1, 2);
    } else {
        if (mode == 0) CSIM_TERMS(2, 0);
        else if (mode == 1) CSIM_TERMS(2, 1);
        else CSIM_TERMS(2, 2);
    }
#undef CSIM_TERMS
    return post(L);
}

int launch_reduce_parts(const Launch& L, const __int128* part, int64_t ntheta, int64_t nchunks, __int128* acc) {
    if (ntheta <= 0) return 0;
    int64_t blocks = (ntheta * 4 + 255) / 256;
    if (blocks > (int64_t)L.num_sms * 16) blocks = (int64_t)L.num_sms * 16;
    k_reduce_parts<<<(int)blocks, 256, 0, L.stream>>>(part, ntheta, nchunks, acc);
    return post(L);
}

}  // namespace csim
