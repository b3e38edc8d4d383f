// csim_internal.h — launch interface between the host code (csim_host.cpp,
// csim_engine.cpp, csim_static.cu) and the kernels (csim_kernels.cu,
// csim_terms_tp.cu).  Not installed.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace csim {

struct GState;  // device image of csim_state (csim_warp.cuh)

struct Launch {
    cudaStream_t stream;
    int* d_err;         // device error word, OR of csim::kErr* flags
    int64_t* launches;  // host counter of kernel launches
    int num_sms;
};

int launch_inner_product(const Launch& L, int nr, const GState* a, const GState* b, int64_t count, int* eps, int* p,
                         int* m);
int launch_exp_sum(const Launch& L, int nr, GState* s, int64_t count, int* eps, int* p, int* m);
int launch_shrink(const Launch& L, int nr, GState* s, const uint64_t* xi, const int* alpha, int lazy, int64_t count,
                  int* status);
int launch_measure(const Launch& L, int nr, GState* s, const int* m, const uint64_t* zeta, const uint64_t* xi,
                   int64_t count, int* code);
int launch_extend(const Launch& L, int nr, GState* s, const uint64_t* xi, int64_t count);
int launch_random_states(const Launch& L, int n, int64_t count, int mode, uint64_t seed, uint64_t first,
                         const uint32_t* words, const int64_t* offsets, const double* cum, GState* out,
                         int64_t* consumed);
int launch_project(const Launch& L, int nr, GState* s, int64_t count, int nstabs, const int* m, const uint64_t* zeta,
                   const uint64_t* xi, int* code);
int launch_codewords(const Launch& L, const uint64_t* Ld, int k, int64_t j0, int64_t count, uint64_t* out);
// decompose()'s fidelity sum as the integer sum of 2^(S - |x|/2) over the 2^k
// codewords: one partial per block (*nblocks of them, at most SMs * 8)
int launch_fidelity_sum(const Launch& L, const uint64_t* Ld, int k, int S, unsigned __int128* part, int* nblocks);
int launch_prep(const Launch& L, int t, int exact, const uint64_t* codewords, const int64_t* idx, int64_t count,
                GState* out);
// part / part_diag: 4 int128 per work item (ntheta * ceil(nj/chunk) items), zeroed by the caller
int launch_terms(const Launch& L, int nr, int mode, const uint64_t* codewords, const GState* phis,
                 const GState* theta, const int* code, int64_t ntheta, int64_t j0, int64_t nj, int chunk, int P,
                 __int128* part, __int128* part_diag, int* eps_o, int* p_o, int* m_o);
int launch_reduce_parts(const Launch& L, const __int128* part, int64_t ntheta, int64_t nchunks, __int128* acc);

// thread-per-pair kernel for terms of |L> (csim_terms_tp.cu); nmax >= every theta's n,
// gmax >= the zeros of every codeword in [j0, j0 + nj) (gmax = nmax always holds).
// codewords[0] is term j0's codeword.
// Work item = (theta a, block cb of 64 * per_thread terms): 4 int128 partial sums at
// part[4 * (a * part_stride + part_base + cb)].  gate (optional, device): when *gate is 0
// the launch has no live state and its blocks return at once (the direct kernel's fallback).
int launch_terms_tp(const Launch& L, int nmax, int gmax, const uint64_t* codewords, const GState* theta,
                    const int* code, int64_t ntheta, int64_t j0, int64_t nj, int per_thread, int P, __int128* part,
                    int64_t part_stride, int64_t part_base, int* eps_o, int* p_o, int* m_o,
                    const int* gate = nullptr);
int64_t terms_tp_blocks(int64_t nj, int per_thread);
// resident blocks per SM of the thread-per-pair kernel for states of up to nmax
// qubits and codewords of up to gmax zeros (-1 if the query fails)
int terms_tp_occupancy(int nmax, int gmax);

// the direct kernel (csim_terms_tp.cu).  launch_canon: each live state in
// pivot coordinates (canon_bytes() per state in `canon`); states with n - k >
// dslots get code_direct = -1 and keep their code in code_rest (for the
// block-prefix kernel), the others the reverse.  launch_terms_direct: all pairs
// of the states with code >= 0 against codewords [j0, j0 + nj), partial sums as
// launch_terms_tp's (only live states write theirs); `rows` (<= nmax) bounds the
// ones of every codeword in the range, which sizes the per-pair rows (a pair
// with more live variables sets the range error).
size_t canon_bytes();
// rest_count (optional): the number of live states left to the block-prefix
// kernel is added to *rest_count (zero it before the first launch)
int launch_canon(const Launch& L, const GState* theta, const int* code, int64_t ntheta, int dslots, void* canon,
                 int* code_direct, int* code_rest, int* rest_count = nullptr);
int launch_terms_direct(const Launch& L, int nmax, int rows, int dslots, const uint64_t* codewords,
                        const void* canon, const int* code, int64_t ntheta, int64_t j0, int64_t nj, int per_thread,
                        int P, __int128* part, int64_t part_stride, int64_t part_base);

// the run kernel (csim_terms_tp.cu): codewords [j0, j0 + nj) in run order
// (csim_host::run_ordered_codewords), runs of per_thread codewords, partial
// sums as launch_terms_tp's; gmax bounds the zeros of every codeword below its
// run's agreed top bits.  scratch: global run memory of at least
// terms_runs_scratch_bytes(num_sms, nmax, gmax) bytes (the grid of a launch with
// that gmax times one block's run memory; a larger gmax gives a smaller grid).
size_t terms_runs_scratch_bytes(int num_sms, int nmax, int gmax);
int launch_terms_runs(const Launch& L, int nmax, int gmax, const uint64_t* codewords, const GState* theta,
                      const int* code, int64_t ntheta, int64_t j0, int64_t nj, int per_thread, int P, __int128* part,
                      int64_t part_stride, int64_t part_base, unsigned char* scratch, size_t scratch_bytes);

}  // namespace csim
