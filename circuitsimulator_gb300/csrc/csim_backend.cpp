// csim_backend.cpp — the backend process protocol of CircuitSimulator on the GPU.
//
// Reads what libcirc/probability.py:249-272 writes (13 scalars, then the
// projectors G' and H' in the encoding of libcirc/utils/comms.c:9-36) and
// prints what the reference master prints (libcirc/probability.c:44-221): echo
// lines, then numerator and denominator as %.17e on the last two lines.  The
// Python caller keeps only those two lines and prints the rest, so
// probability() and sampleQubits() run unchanged with cpath pointing here.
//
// Sampling draws come from the C library's rand() sequence, as in the
// reference, seeded with the process id (probability.c:182) unless CSIM_SEED is
// set; CSIM_RNG=philox switches to the counter-based generator.
#include <unistd.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/csim.h"

namespace {

struct Proj {
    int nstabs = 0, nqubits = 0;
    std::vector<int32_t> phase;
    std::vector<uint64_t> xs, zs;
    csim_projector view() const {
        csim_projector p;
        p.nstabs = nstabs;
        p.nqubits = nqubits;
        p.phase = phase.data();
        p.xs = xs.data();
        p.zs = zs.data();
        return p;
    }
};

// readProjector, libcirc/utils/comms.c:9-36
bool read_projector(FILE* in, Proj& P) {
    if (fscanf(in, "%d", &P.nstabs) != 1 || fscanf(in, "%d", &P.nqubits) != 1) return false;
    if (P.nstabs < 0 || P.nqubits < 0 || P.nqubits > CSIM_MAX_QUBITS) return false;
    if (P.nstabs == 0) return true;
    P.phase.assign(P.nstabs, 0);
    P.xs.assign(P.nstabs, 0);
    P.zs.assign(P.nstabs, 0);
    for (int i = 0; i < P.nstabs; i++) {
        int v;
        if (fscanf(in, "%d", &v) != 1) return false;
        P.phase[i] = v;
        for (int j = 0; j < P.nqubits; j++) {
            int x, z;
            if (fscanf(in, "%d", &x) != 1 || fscanf(in, "%d", &z) != 1) return false;
            if (x & 1) P.xs[i] |= 1ull << j;
            if (z & 1) P.zs[i] |= 1ull << j;
        }
    }
    return true;
}

}  // namespace

extern "C" int csim_backend_run(FILE* in, FILE* out, int device) {
    int quiet, verbose, noapprox, samples, bins, t, k, exact, fidelity, rank, forceL, forceSample;
    double fidbound;
    // libcirc/probability.c:73-128
    if (fscanf(in, "%d", &quiet) != 1) goto bad;
    fprintf(out, "quiet: %d\n", quiet);
    if (fscanf(in, "%d", &verbose) != 1) goto bad;
    fprintf(out, "verbose: %d\n", verbose);
    if (fscanf(in, "%d", &noapprox) != 1) goto bad;
    fprintf(out, "noapprox: %d\n", noapprox);
    if (fscanf(in, "%d", &samples) != 1) goto bad;
    fprintf(out, "samples: %d\n", samples);
    if (fscanf(in, "%d", &bins) != 1) goto bad;
    fprintf(out, "bins: %d\n", bins);
    if (fscanf(in, "%d", &t) != 1) goto bad;
    fprintf(out, "t: %d\n", t);
    if (fscanf(in, "%d", &k) != 1) goto bad;
    fprintf(out, "k: %d\n", k);
    if (fscanf(in, "%d", &exact) != 1) goto bad;
    fprintf(out, "exact: %d\n", exact);
    if (fscanf(in, "%lf", &fidbound) != 1) goto bad;
    fprintf(out, "fidbound: %f\n", fidbound);
    if (fscanf(in, "%d", &fidelity) != 1) goto bad;
    fprintf(out, "fidelity: %d\n", fidelity);
    if (fscanf(in, "%d", &rank) != 1) goto bad;
    fprintf(out, "rank: %d\n", rank);
    if (fscanf(in, "%d", &forceL) != 1) goto bad;
    fprintf(out, "forceL: %d\n", forceL);
    if (fscanf(in, "%d", &forceSample) != 1) goto bad;
    fprintf(out, "forceSample: %d\n", forceSample);
    {
        Proj G, H;
        if (!read_projector(in, G) || !read_projector(in, H)) goto bad;
        if (t < 0 || t > CSIM_MAX_QUBITS) {
            fprintf(out, "csim: t=%d outside 0..%d\n", t, CSIM_MAX_QUBITS);
            fflush(out);
            return CSIM_ERR_PROTOCOL;
        }
        fprintf(out, "Using GB300 (sm_103a) kernels for matrix operations.\n");

        // decompose() runs before the sampler is seeded, on rand()'s default stream
        std::vector<unsigned char> dstate((size_t)csim_libc_rand_size());
        csim_libc_rand_seed(dstate.data(), 1);
        double norm = 0;
        uint64_t L[CSIM_MAX_QUBITS] = {0};
        // the fidelity sum runs on the GPU; without one the lines up to the L
        // matrix still print, and the run stops below with the device error
        csim_ctx* ctx = nullptr;
        const int ctx_rc = csim_ctx_create(device, &ctx);
        const int rc = ctx ? csim_decompose_on(ctx, t, fidbound, rank, fidelity, forceL, verbose, quiet, &exact, &k,
                                               &norm, L, dstate.data(), out)
                           : csim_decompose(t, fidbound, rank, fidelity, forceL, verbose, quiet, &exact, &k, &norm,
                                            L, dstate.data(), out);
        if (rc != CSIM_OK) {
            fprintf(out, "csim: decompose failed (%d)\n", rc);
            fflush(out);
            csim_ctx_destroy(ctx);
            return rc;
        }
        fprintf(out, "World Size: %d\n", 1);
        if (verbose) {
            if (exact) fprintf(out, "Using exact decomposition of |H^t>: 2^%d\n", (t + 1) / 2);
            else fprintf(out, "Stabilizer rank of |L>: 2^%d\n", k);
        }
        if (noapprox == 0 && forceSample == 0) {  // probability.c:162-174
            const double terms = exact ? pow(2, (t + 1) / 2) : pow(2, k);
            if (samples * bins * 2 > (terms - 1)) {
                noapprox = 1;
                if (verbose) fprintf(out, "More samples than terms in exact calculation. Disabling sampling.\n");
            }
        }
        if (exact == 0) {
            fprintf(out, "L:\n");
            if (t > 0) {  // BitMatrixPrint, libcirc/utils/matrix.c:316-328
                fprintf(out, "[");
                for (int i = 0; i < k; i++) {
                    if (i != 0) fprintf(out, "\n ");
                    fprintf(out, "[");
                    for (int j = 0; j < t; j++) fprintf(out, "%d", (int)((L[i] >> j) & 1));
                    fprintf(out, "]");
                }
                fprintf(out, "]\n");
            }
        }
        fflush(out);

        const char* s_env = getenv("CSIM_SEED");
        const uint64_t seed = (s_env && *s_env) ? (uint64_t)strtoull(s_env, nullptr, 10) : (uint64_t)getpid();
        const char* r_env = getenv("CSIM_RNG");
        const int rng = (r_env && strcmp(r_env, "philox") == 0) ? CSIM_RNG_PHILOX : CSIM_RNG_LIBC;
        const uint64_t sd = rng == CSIM_RNG_LIBC ? (uint64_t)(uint32_t)seed : seed;

        int r = ctx_rc;
        if (r != CSIM_OK) {
            fprintf(out, "csim: no usable GB300 device (%d)\n", r);
            fflush(out);
            return r;
        }
        const csim_projector pg = G.view(), ph = H.view();
        double numerator = 0, denominator = 0;
        if (noapprox == 0) {
            r = csim_multi_sampled_projector(ctx, &pg, L, k, exact, norm, samples, bins, rng, sd, &numerator);
            if (r == CSIM_OK)
                r = csim_multi_sampled_projector(ctx, &ph, L, k, exact, norm, samples, bins, rng, CSIM_SEED_CONTINUE,
                                                 &denominator);
        } else {
            r = csim_exact_projector(ctx, &pg, L, k, exact, norm, &numerator);
            if (r == CSIM_OK) r = csim_exact_projector(ctx, &ph, L, k, exact, norm, &denominator);
        }
        if (r != CSIM_OK) {
            fprintf(out, "csim error %d: %s\n", r, csim_last_error(ctx));
            csim_ctx_destroy(ctx);
            fflush(out);
            return r;
        }
        csim_ctx_destroy(ctx);
        const int sigfigs = 17;
        fprintf(out, "|| Gprime |H^t> ||^2 ~= %.*e\n", sigfigs, numerator);
        fprintf(out, "|| Hprime |H^t> ||^2 ~= %.*e\n", sigfigs, denominator);
        if (denominator > 0) fprintf(out, "Output: %.*e\n", sigfigs, numerator / denominator);
        fprintf(out, "%.*e\n", sigfigs, numerator);
        fprintf(out, "%.*e\n", sigfigs, denominator);
        fflush(out);
        return CSIM_OK;
    }
bad:
    fprintf(out, "csim: malformed backend input\n");
    fflush(out);
    return CSIM_ERR_PROTOCOL;
}

// ---------------------------------------------------------------- serving daemon
// One process for a stream of queries instead of one process per query
// (libcirc/probability.py:237-244).  Reads back-to-back protocol inputs (13
// scalars, G', H') until end of input and submits each to a csim_server as
// soon as it is read, so queries that arrive while others run share rounds.
// Writes one line per query, in input order:
//     <index> <status> <numerator %.17e> <denominator %.17e>
// Seeds: CSIM_SEED + index when CSIM_SEED is set, else process id + index.
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>

namespace {

struct OwnedQuery {
    csim_query q{};
    Proj G, H;
};

bool read_query(FILE* in, OwnedQuery& oq) {
    int v[8];
    for (int i = 0; i < 8; i++)
        if (fscanf(in, "%d", &v[i]) != 1) return false;
    double fb;
    if (fscanf(in, "%lf", &fb) != 1) return false;
    int w[4];
    for (int i = 0; i < 4; i++)
        if (fscanf(in, "%d", &w[i]) != 1) return false;
    if (!read_projector(in, oq.G) || !read_projector(in, oq.H)) return false;
    csim_query& q = oq.q;
    q.quiet = v[0];
    q.verbose = v[1];
    q.noapprox = v[2];
    q.samples = v[3];
    q.bins = v[4];
    q.t = v[5];
    q.k = v[6];
    q.exact = v[7];
    q.fidbound = fb;
    q.fidelity = w[0];
    q.rank = w[1];
    q.force_l = w[2];
    q.force_sample = w[3];
    q.G = oq.G.view();
    q.H = oq.H.view();
    return true;
}

}  // namespace

extern "C" int csim_backend_serve(FILE* in, FILE* out, int device) {
    csim_server_config cfg{};
    cfg.device = device;
    const char* b_env = getenv("CSIM_HBM_BUDGET");
    cfg.hbm_budget_bytes = (b_env && *b_env) ? (int64_t)strtoll(b_env, nullptr, 10) : 0;
    csim_server* srv = nullptr;
    int rc = csim_server_create(&cfg, &srv);
    if (rc != CSIM_OK) {
        fprintf(out, "csim: no usable GB300 device (%d)\n", rc);
        fflush(out);
        return rc;
    }
    const char* s_env = getenv("CSIM_SEED");
    const uint64_t seed0 = (s_env && *s_env) ? (uint64_t)strtoull(s_env, nullptr, 10) : (uint64_t)getpid();
    const char* r_env = getenv("CSIM_RNG");
    const int rng = (r_env && strcmp(r_env, "philox") == 0) ? CSIM_RNG_PHILOX : CSIM_RNG_LIBC;

    std::mutex mu;
    std::condition_variable cv;
    std::deque<int64_t> tickets;  // in input order
    bool eof = false;
    std::thread writer([&] {
        int64_t index = 0;
        while (true) {
            int64_t tk;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return eof || !tickets.empty(); });
                if (tickets.empty()) return;
                tk = tickets.front();
                tickets.pop_front();
            }
            csim_query_result r{};
            int w = csim_wait(srv, tk, -1.0, &r);
            if (w != CSIM_OK) r.status = w;
            fprintf(out, "%lld %d %.17e %.17e\n", (long long)index++, r.status, r.numerator, r.denominator);
            fflush(out);
            csim_release(srv, tk);
        }
    });
    int64_t index = 0;
    int status = CSIM_OK;
    while (true) {
        OwnedQuery* oq = new OwnedQuery();
        if (!read_query(in, *oq)) {
            delete oq;
            int c;
            while ((c = fgetc(in)) != EOF && isspace(c)) {
            }
            if (c != EOF) status = CSIM_ERR_PROTOCOL;  // trailing garbage
            break;
        }
        oq->q.rng = rng;
        oq->q.seed = rng == CSIM_RNG_LIBC ? (uint64_t)(uint32_t)(seed0 + (uint64_t)index) : seed0 + (uint64_t)index;
        int64_t tk = 0;
        const int s = csim_submit(srv, &oq->q, &tk);  // copies the query
        delete oq;
        if (s != CSIM_OK) {
            status = s;
            break;
        }
        {
            std::lock_guard<std::mutex> lk(mu);
            tickets.push_back(tk);
        }
        cv.notify_one();
        index++;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        eof = true;
    }
    cv.notify_one();
    writer.join();
    csim_server_destroy(srv);
    if (status == CSIM_ERR_PROTOCOL) {
        fprintf(out, "csim: malformed backend input after query %lld\n", (long long)index);
        fflush(out);
    }
    return status;
}
