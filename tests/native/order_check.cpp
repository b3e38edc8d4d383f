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

// The run kernel's order (run_ordered_codewords); returns the light launch's first position.
extern "C" int64_t order_runs(const uint64_t* L, int k, int t, int pt, int gl, uint64_t* out) {
    std::vector<uint64_t> cw;
    const int64_t split = csim_host::run_ordered_codewords(L, k, t, pt, gl, cw);
    std::copy(cw.begin(), cw.end(), out);
    return split;
}

// Zero-class order (ordered_codewords_classes); starts has nbounds + 1 entries.
extern "C" void order_classes(const uint64_t* L, int k, int t, const int* bounds, int nbounds, uint64_t* out,
                              int64_t* starts) {
    std::vector<uint64_t> cw;
    std::vector<int64_t> st;
    csim_host::ordered_codewords_classes(L, k, t, std::vector<int>(bounds, bounds + nbounds), cw, st);
    std::copy(cw.begin(), cw.end(), out);
    std::copy(st.begin(), st.end(), starts);
}
