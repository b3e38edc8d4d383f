// Host build of the sampled estimators' codeword order
// (circuitsimulator_gb300/csrc/csim_host_common.h: ordered_codewords,
// light_split), for CPU tests only.
#include "../../circuitsimulator_gb300/csrc/csim_host_common.h"

extern "C" int64_t order_codewords(const uint64_t* L, int k, int t, uint64_t* out) {
    std::vector<uint64_t> cw;
    csim_host::ordered_codewords(L, k, t, cw);
    std::copy(cw.begin(), cw.end(), out);
    return csim_host::light_split(cw, t);
}

extern "C" int order_prefix_bits(int k, int t) { return csim_host::ordered_prefix_bits(k, t); }
extern "C" int order_light_zeros(int t) { return csim_host::light_zeros(t); }
extern "C" int order_per_thread(int fixed, int t) { return csim_host::tp_per_thread(fixed, t); }
