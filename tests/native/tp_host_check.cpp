// Host build of the thread-per-pair kernel's pair routine
// (circuitsimulator_gb300/csrc/csim_pair_core.cuh), for CPU tests only: the
// same source the kernel runs, checked against the oracle without a GPU.
#include <cstdint>
#include <cstring>

// rows the direct path touches (the pair core's CSIM_COUNT_ROWS hook)
static int64_t g_direct_rows = 0;
#define CSIM_COUNT_ROWS(r) (g_direct_rows += (int64_t)(r))

#include "../../circuitsimulator_gb300/csrc/csim_block_prefix.cuh"
#include "../../circuitsimulator_gb300/csrc/csim_pair_core.cuh"
#include "../../include/csim.h"

extern "C" int tp_host_pairs(const csim_state* theta, int ntheta, const uint64_t* xs, int nx, int* eps, int* p,
                             int* m) {
    int err = 0;
    uint64_t pGT[64];
    alignas(16) uint32_t wJ32[32];
    alignas(16) uint64_t wJ64[34];
    alignas(16) uint64_t wG[64];
    const csim::pc::PairMem mem{wJ32, wJ64, wG, 1};
    for (int a = 0; a < ntheta; a++) {
        const csim_state& th = theta[a];
        for (int c = 0; c < 64; c++) {
            uint64_t col = 0;
            if (c < th.n)
                for (int r = 0; r < th.k; r++) col |= ((th.G[r] >> c) & 1ull) << r;
            pGT[c] = col;
        }
        for (int j = 0; j < nx; j++) {
            const int w = a * nx + j;
            csim::pc::pair_l(true, th.n, th.k, th.Q, th.h, th.D1, th.D2, th.J, pGT, xs[j], mem, eps[w], p[w], m[w],
                             err);
        }
    }
    return err;
}

// The kernels' block path (csim_block_prefix.cuh): the codewords split in two
// halves at the highest bit in which they differ, each half again at its own
// highest differing bit; each group's shared top-bit shrinks run once per
// theta (prefix_shrink), then every pair continues from its group's state
// (pair_l with done = that group's agreed top bits).
extern "C" int tp_host_block(const csim_state* theta, int ntheta, const uint64_t* xs, int nx, int* eps, int* p,
                             int* m) {
    using namespace csim::pc;
    int err = 0;
    alignas(16) uint32_t wJ32[32];
    alignas(16) uint64_t wJ64[34];
    alignas(16) uint64_t wG[64];
    const PairMem mem{wJ32, wJ64, wG, 1};
    for (int a = 0; a < ntheta; a++) {
        const csim_state& th = theta[a];
        const uint64_t nm = lowmask(th.n);
        // AND / OR: [0] all, [1 + h] half h, [3 + 2h + q] group 2h + q
        uint64_t andm[7], orm[7];
        for (int q = 0; q < 7; q++) {
            andm[q] = ~0ull;
            orm[q] = 0;
        }
        for (int j = 0; j < nx; j++) {
            andm[0] &= xs[j];
            orm[0] |= xs[j];
        }
        const int hb = top_bit_or_none((andm[0] ^ orm[0]) & nm);
        int hb2[2] = {-1, -1};
        if (hb >= 0) {
            for (int j = 0; j < nx; j++) {
                const int h = (int)((xs[j] >> hb) & 1ull);
                andm[1 + h] &= xs[j];
                orm[1 + h] |= xs[j];
            }
            for (int h = 0; h < 2; h++) hb2[h] = top_bit_or_none((andm[1 + h] ^ orm[1 + h]) & nm);
            for (int j = 0; j < nx; j++) {
                const int h = (int)((xs[j] >> hb) & 1ull);
                if (hb2[h] < 0) continue;
                const int q = (int)((xs[j] >> hb2[h]) & 1ull);
                andm[3 + 2 * h + q] &= xs[j];
                orm[3 + 2 * h + q] |= xs[j];
            }
        }
        struct {
            uint64_t pJ[64], pGT[64], h, D1, D2, done;
            int k, Q, ok, used;
        } st[kGroups];
        for (int g = 0; g < kGroups; g++) {
            int slot = -1;
            if (hb < 0) slot = g == 0 ? 0 : -1;
            else if (hb2[g / 2] < 0) slot = (g & 1) ? -1 : 1 + g / 2;
            else slot = 3 + g;
            st[g].used = slot >= 0;
            if (slot < 0) continue;
            for (int c = 0; c < 64; c++) {
                uint64_t col = 0;
                if (c < th.n)
                    for (int r = 0; r < th.k; r++) col |= ((th.G[r] >> c) & 1ull) << r;
                st[g].pGT[c] = col;
                st[g].pJ[c] = th.J[c];
            }
            st[g].k = th.k;
            st[g].Q = th.Q;
            st[g].h = th.h;
            st[g].D1 = th.D1;
            st[g].D2 = th.D2;
            const uint64_t pm = agree_top(andm[slot] ^ orm[slot], th.n);
            st[g].done = pm;
            st[g].ok = 1;
            if (hd_popc64(~andm[slot] & pm & nm) > 0)
                st[g].ok = prefix_shrink(true, th.n, pm, andm[slot], st[g].k, st[g].Q, st[g].h, st[g].D1, st[g].D2,
                                         st[g].pJ, st[g].pGT, mem);
        }
        for (int j = 0; j < nx; j++) {
            const int w = a * nx + j;
            const auto& s = st[block_group(hb, hb2[0], hb2[1], xs[j])];
            if (!s.used) return -1;
            eps[w] = p[w] = m[w] = 0;
            if (s.ok)
                pair_l(true, th.n, s.k, s.Q, s.h, s.D1, s.D2, s.pJ, s.pGT, xs[j], mem, eps[w], p[w], m[w], err, 64,
                       s.done, th.k);
        }
    }
    return err;
}

// The per-thread run path of the run kernel (run_prefix, pair_from_run):
// xs in runs of run_len consecutive codewords; each run's common zeros in its
// agreed top bits are shrunk once per theta, and each pair continues from that
// state, as one kernel thread does for its run.
extern "C" int tp_host_runs(const csim_state* theta, int ntheta, const uint64_t* xs, int nx, int run_len, int* eps,
                            int* p, int* m) {
    using namespace csim::pc;
    int err = 0;
    alignas(16) uint32_t wJ32[32], rJ32[32];
    alignas(16) uint64_t wJ64[34], rJ64[34];
    alignas(16) uint64_t wG[64], rG[64];
    const PairMem mem{wJ32, wJ64, wG, 1};
    const PairMem rmem{rJ32, rJ64, rG, 1};
    uint64_t pGT[64];
    for (int a = 0; a < ntheta; a++) {
        const csim_state& th = theta[a];
        for (int c = 0; c < 64; c++) {
            uint64_t col = 0;
            if (c < th.n)
                for (int r = 0; r < th.k; r++) col |= ((th.G[r] >> c) & 1ull) << r;
            pGT[c] = col;
        }
        for (int r0 = 0; r0 < nx; r0 += run_len) {
            const int r1 = r0 + run_len < nx ? r0 + run_len : nx;
            uint64_t am = ~0ull, om = 0ull;
            for (int j = r0; j < r1; j++) {
                am &= xs[j];
                om |= xs[j];
            }
            const uint64_t pm = agree_top(am ^ om, th.n);
            RunState rs;
            run_prefix(true, th.n, pm, am, th.k, th.Q, th.h, th.D1, th.D2, th.J, pGT, rmem, rs);
            for (int j = r0; j < r1; j++) {
                const int w = a * nx + j;
                pair_from_run(true, th.n, rs, rmem, xs[j], mem, eps[w], p[w], m[w], err, 64, th.k);
            }
        }
    }
    return err;
}

// The direct-restriction path (canon_theta once per theta, pair_direct per
// pair): eps, p and m mod 8 of every pair, for comparison with the oracle.
extern "C" int tp_host_direct(const csim_state* theta, int ntheta, const uint64_t* xs, int nx, int* eps, int* p,
                              int* m) {
    using namespace csim::pc;
    int err = 0;
    alignas(16) uint32_t wJ32[32];
    alignas(16) uint64_t wJ64[34];
    alignas(16) uint64_t wG[64];
    const PairMem mem{wJ32, wJ64, wG, 1};
    uint64_t Jc[64], acol[64];
    for (int a = 0; a < ntheta; a++) {
        const csim_state& th = theta[a];
        Canon cs;
        canon_theta(th.n, th.k, th.Q, th.h, th.D1, th.D2, th.G, th.J, Jc, acol, cs);
        for (int j = 0; j < nx; j++) {
            const int w = a * nx + j;
            pair_direct(true, th.n, cs, Jc, acol, xs[j], mem, eps[w], p[w], m[w], err, 64, th.k, 64);
        }
    }
    return err;
}

// Rows the direct path touched since the last call (CSIM_COUNT_ROWS), then 0.
extern "C" int64_t tp_host_rows_take() {
    const int64_t r = g_direct_rows;
    g_direct_rows = 0;
    return r;
}
