// Host build of the thread-per-pair kernel's pair routine
// (circuitsimulator_gb300/csrc/csim_pair_core.cuh), for CPU tests only: the
// same source the kernel runs, checked against the oracle without a GPU.
#include <cstring>

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

// The kernels' block path: the shrinks by the zeros of the codewords' common
// top bits run once per theta (prefix_shrink), then every pair continues from
// that state (pair_l with done = those bits).
extern "C" int tp_host_block(const csim_state* theta, int ntheta, const uint64_t* xs, int nx, int* eps, int* p,
                             int* m) {
    int err = 0;
    uint64_t pJ[64], pGT[64];
    alignas(16) uint32_t wJ32[32];
    alignas(16) uint64_t wJ64[34];
    alignas(16) uint64_t wG[64];
    const csim::pc::PairMem mem{wJ32, wJ64, wG, 1};
    uint64_t dis = 0;
    for (int j = 0; j < nx; j++) dis |= xs[j] ^ xs[0];
    for (int a = 0; a < ntheta; a++) {
        const csim_state& th = theta[a];
        for (int c = 0; c < 64; c++) {
            uint64_t col = 0;
            if (c < th.n)
                for (int r = 0; r < th.k; r++) col |= ((th.G[r] >> c) & 1ull) << r;
            pGT[c] = col;
            pJ[c] = th.J[c];
        }
        int k = th.k, Q = th.Q;
        uint64_t h = th.h, D1 = th.D1, D2 = th.D2;
        const uint64_t pm = nx > 0 ? csim::pc::agree_top(dis, th.n) : 0ull;
        int ok = 1;
        if (nx > 0 && csim::pc::hd_popc64(~xs[0] & pm & csim::pc::lowmask(th.n)) > 0)
            ok = csim::pc::prefix_shrink(true, th.n, pm, xs[0], k, Q, h, D1, D2, pJ, pGT, mem);
        for (int j = 0; j < nx; j++) {
            const int w = a * nx + j;
            eps[w] = p[w] = m[w] = 0;
            if (ok)
                csim::pc::pair_l(true, th.n, k, Q, h, D1, D2, pJ, pGT, xs[j], mem, eps[w], p[w], m[w], err, 64, pm,
                                 th.k);
        }
    }
    return err;
}
