// csim_batch.h — descriptor tables of the query engine (csim_engine.cpp),
// shared with its kernels (csim_batch_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "csim_internal.h"

namespace csim {

struct GState;

// one state to prepare: draw it (mode 0 Philox, 1 replayed rand() words) or copy
// `src` (mode 2, a term state of the exact projector), then project it onto the
// query's projector (nstabs rows pm/pz/px)
struct DrawDesc {
    int32_t n, mode, nstabs, pad;
    uint64_t seed, id;
    int64_t wbegin, wend;
    const uint32_t* words;
    const double* cum;
    const GState* src;
    const int32_t* pm;
    const uint64_t* pz;
    const uint64_t* px;
};

// one work item of the pair kernels: state `theta` against terms [j0, j0+nj) of
// either a codeword table (cw, |L> terms) or a term-state array (phis); the term
// j == diag (if >= 0) is summed apart (exactProjector's diagonal)
struct PairItem {
    int64_t theta, j0, nj, diag;
    const uint64_t* cw;
    const GState* phis;
};

int launch_draw_project(const Launch& L, const DrawDesc* desc, int64_t count, GState* out, int* code);
// resident blocks per SM of k_items_tp launched for states of up to nmax qubits
// and codewords of up to gmax zeros
int items_tp_occupancy(int nmax, int gmax);
// queue: one device counter, zeroed by the launch (stream-ordered) and drawn from by the blocks.
// only_live: write the partial sums of live states' items only (the other items are another launch's).
// gate (optional, device): when *gate is 0 no item has a live state and the blocks return at once.
int launch_items_tp(const Launch& L, const PairItem* items, int64_t nitems, const GState* states, const int* codes,
                    int per_thread, int nmax, int gmax, __int128* part, __int128* part_diag,
                    unsigned long long* queue, bool only_live = false, const int* gate = nullptr);
// the direct kernel over the items; canon, code_direct, code_rest as launch_canon
// wrote them for the items' states.  Writes every item's partial sums except
// those of states with code_rest >= 0 (launch_items_tp with code_rest, only_live).
// `rows` (<= nmax) bounds the ones of every item's codewords.
int launch_items_direct(const Launch& L, const PairItem* items, int64_t nitems, const void* canon,
                        const int* code_direct, const int* code_rest, int per_thread, int nmax, int rows, int dslots,
                        __int128* part, __int128* part_diag, unsigned long long* queue);
int launch_items_warp(const Launch& L, const PairItem* items, int64_t nitems, const GState* states, const int* codes,
                      __int128* part, __int128* part_diag);
// per-slot sums of item partials; slot s owns items [range[2s], range[2s+1]) and,
// if range2 is not null, [range2[2s], range2[2s+1])
int launch_reduce_slots(const Launch& L, const __int128* part, const int64_t* range, const int64_t* range2,
                        int64_t nslots, __int128* out);

}  // namespace csim
