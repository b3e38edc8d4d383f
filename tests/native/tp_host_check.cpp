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
