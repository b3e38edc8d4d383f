// csim_static.cu — csim_single_projector_samples_static: the sampler for
// terms of |L> with no device allocation at all.
//
// Who needs it: code that owns the GPU's memory itself and must not call
// cudaMalloc — a host framework with its own pool allocator, a process that
// pre-plans every byte of device memory, or a caller that has handed all free
// memory to another component.  Such callers still get the full path
// (random states -> projection -> all terms -> exact per-state sums).
//
// Every byte of device scratch lives in g_scratch below: one file-scope
// array of kScratchBytes, held by every GPU that loads the library until the
// process exits.  Inputs and outputs stay in the caller's host buffers;
// copies to and from the scratch use the legacy default stream.  Nothing
// here calls cudaMalloc, cudaFree or an allocating library routine.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/csim.h"
#include "csim_host_common.h"
#include "csim_internal.h"

namespace {

constexpr size_t kScratchBytes = (size_t)5 << 19;  // 2.5 MiB per GPU

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// regions of g_scratch (byte offsets, each 256-aligned)
constexpr size_t kOffErr = 0;
constexpr size_t kOffPm = 256;                       // int32 m[64]
constexpr size_t kOffPz = kOffPm + 256;              // uint64 zeta[64]
constexpr size_t kOffPx = kOffPz + 512;              // uint64 xi[64]
constexpr size_t kOffCum = kOffPx + 512;             // double cum[65]
constexpr size_t kOffL = kOffCum + 768;              // uint64 L[64]
constexpr size_t kOffCw = kOffL + 512;               // uint64 codewords[2^16]
constexpr size_t kOffStates = kOffCw + ((size_t)8 << 16);  // csim_state[256]
constexpr size_t kOffCode = kOffStates + (size_t)CSIM_STATIC_MAX_STATES * sizeof(csim_state);  // int32[256]
constexpr size_t kOffPart = kOffCode + 1024;         // int128[256 * 64 * 4]
constexpr int kPerThread = 16;                       // terms per thread per work item (64 * 16 per item)
constexpr int64_t kMaxItems = (int64_t)CSIM_STATIC_MAX_STATES * ((1 << CSIM_STATIC_MAX_K) / (64 * kPerThread));
constexpr size_t kOffAcc = kOffPart + (size_t)kMaxItems * 4 * 16;  // int128[256 * 4]
constexpr size_t kEnd = kOffAcc + (size_t)CSIM_STATIC_MAX_STATES * 4 * 16;
static_assert(kEnd <= kScratchBytes, "scratch regions exceed the static array");

// Device address of g_scratch, looked up once per device with that device
// current.  In host code g_scratch names a host-side stand-in, never usable
// as a device pointer, hence the lookup.
std::mutex g_mu;
unsigned char* g_ptr[64] = {};

int scratch_for(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (device < 0 || device >= 64) return CSIM_ERR_ARG;
    if (!g_ptr[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return CSIM_ERR_CUDA;
        g_ptr[device] = (unsigned char*)p;
    }
    *out = g_ptr[device];
    return CSIM_OK;
}

// Puts the caller's current device back on every return path, so a host
// framework that binds its threads to devices sees no change.
struct DeviceRestore {
    int prev = -1;
    DeviceRestore() {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    }
    ~DeviceRestore() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int run_static(int32_t device, const csim_projector* P, const uint64_t* L, int32_t k, int64_t count, uint64_t seed,
               double* values);

}  // namespace

extern "C" int csim_single_projector_samples_static(int32_t device, const csim_projector* P, const uint64_t* L,
                                                    int32_t k, int64_t count, uint64_t seed, double* values) {
    DeviceRestore keep;
    return run_static(device, P, L, k, count, seed, values);
}

namespace {

int run_static(int32_t device, const csim_projector* P, const uint64_t* L, int32_t k, int64_t count, uint64_t seed,
               double* values) {
    if (!P || !values || (k > 0 && !L)) return CSIM_ERR_ARG;
    const int t = P->nqubits, nstabs = P->nstabs;
    if (count < 1 || count > CSIM_STATIC_MAX_STATES || t < 1 || t > CSIM_MAX_QUBITS || k < 0 ||
        k > CSIM_STATIC_MAX_K || nstabs < 1 || nstabs > 64 || !P->phase || !P->xs || !P->zs)
        return CSIM_ERR_ARG;
    const uint64_t tm = t >= 64 ? ~0ull : ((1ull << t) - 1);
    for (int r = 0; r < k; r++)
        if (L[r] & ~tm) return CSIM_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return CSIM_ERR_NODEVICE;
    int num_sms = 0;
    if (cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return CSIM_ERR_CUDA;
    unsigned char* base = nullptr;
    int rc = scratch_for(device, &base);
    if (rc != CSIM_OK) return rc;

    const cudaStream_t st = 0;
    int* d_err = (int*)(base + kOffErr);
    int64_t launches = 0;
    const csim::Launch Lh{st, d_err, &launches, num_sms};

    // small inputs: projector, cumulative d-distribution, code rows
    int32_t pm[64];
    for (int r = 0; r < nstabs; r++) pm[r] = csim_host::phase_m(P->phase[r]);
    double cum[CSIM_MAX_QUBITS + 1];
    csim_host::cum_table(t, cum);  // the allocating sampler's table
    uint64_t Lrows[64] = {0};
    for (int r = 0; r < k; r++) Lrows[r] = L[r];

    const int64_t chi = (int64_t)1 << k;
    const int64_t nblk = csim::terms_tp_blocks(chi, kPerThread);
    const size_t nparts = (size_t)count * nblk * 4 * 16;
    bool ok = cudaMemsetAsync(d_err, 0, sizeof(int), st) == cudaSuccess &&
              cudaMemcpyAsync(base + kOffPm, pm, sizeof(int32_t) * nstabs, cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemcpyAsync(base + kOffPz, P->zs, sizeof(uint64_t) * nstabs, cudaMemcpyHostToDevice, st) ==
                  cudaSuccess &&
              cudaMemcpyAsync(base + kOffPx, P->xs, sizeof(uint64_t) * nstabs, cudaMemcpyHostToDevice, st) ==
                  cudaSuccess &&
              cudaMemcpyAsync(base + kOffCum, cum, sizeof(double) * (t + 1), cudaMemcpyHostToDevice, st) ==
                  cudaSuccess &&
              cudaMemcpyAsync(base + kOffL, Lrows, sizeof(Lrows), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemsetAsync(base + kOffPart, 0, nparts, st) == cudaSuccess;  // partial sums start at zero
    if (!ok) return CSIM_ERR_CUDA;

    uint64_t* cw = (uint64_t*)(base + kOffCw);
    csim::GState* states = (csim::GState*)(base + kOffStates);
    int* code = (int*)(base + kOffCode);
    __int128* part = (__int128*)(base + kOffPart);
    __int128* acc = (__int128*)(base + kOffAcc);
    const int nr = t > 32 ? 2 : 1;
    if (csim::launch_codewords(Lh, (const uint64_t*)(base + kOffL), k, 0, chi, cw) ||
        csim::launch_random_states(Lh, t, count, 0, seed, 0, nullptr, nullptr, (const double*)(base + kOffCum),
                                   states, nullptr) ||
        csim::launch_project(Lh, nr, states, count, nstabs, (const int*)(base + kOffPm),
                             (const uint64_t*)(base + kOffPz), (const uint64_t*)(base + kOffPx), code) ||
        csim::launch_terms_tp(Lh, t, t, cw, states, code, count, 0, chi, kPerThread, 2 * t, part, nblk, 0, nullptr,
                              nullptr, nullptr) ||
        csim::launch_reduce_parts(Lh, part, count, nblk, acc))
        return CSIM_ERR_CUDA;

    int hcode[CSIM_STATIC_MAX_STATES];
    __int128 hacc[CSIM_STATIC_MAX_STATES * 4];
    int herr = 0;
    ok = cudaMemcpyAsync(hcode, code, sizeof(int) * count, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaMemcpyAsync(hacc, acc, sizeof(__int128) * 4 * count, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
         cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) return CSIM_ERR_CUDA;
    if (herr) return CSIM_ERR_DEVICE;

    // singleProjectorSample's value per state (innerprod.c:142): 2^t |projfactor * sum|^2,
    // with the allocating sampler's conversions
    const double scale = pow(2, t);
    for (int64_t i = 0; i < count; i++) {
        if (hcode[i] < 0) {
            values[i] = 0;
            continue;
        }
        double re, im;
        csim_host::zomega_to_complex(&hacc[4 * i], 2 * t, &re, &im);
        const double pf = csim_host::sqrt_half_power(hcode[i]);
        const double a = re * pf, b = im * pf;
        values[i] = scale * (a * a + b * b);
    }
    return CSIM_OK;
}

}  // namespace
