// csim_engine.cpp — the query engine behind csim_run_queries and the server.
//
// Runs many probability queries.  Each query runs as the backend process
// would run it (libcirc/probability.c:146-216): decompose, the noapprox rule,
// then multiSampledProjector or exactProjector on G' and H'.  All admitted
// queries share launches.
//
// Work is cut into rounds.  A round takes the next states of the admitted
// evaluations (one evaluation = one projector of one query), up to a budget
// of inner products, and runs:
//   k_draw_project  draw or copy every state, then project it (innerprod.c:97-116)
//   k_canon         the states of direct-restriction evaluations in pivot form
//   k_items_tp      (state, |L> term range) items, thread per pair
//   k_items_direct  the same items by direct restriction, thread per pair
//   k_items_warp    (state, prepH term range) items, warp per pair
//   k_reduce_slots  exact Z[w] sums per state
// Two round buffers alternate.  The host builds round r+1 and queues it behind
// round r, then reads round r's results.
//
// Per-state values are kept until an evaluation's last state is in.  The
// estimator then reduces them in draw (row) order, the same order the
// single-query entry points use.  So a result does not depend on how its
// states were split into rounds, nor on which other queries shared them.
//
// Decompositions (codeword tables, term states) stay resident on the device.
// Queries with the same t and code share them; unused ones are evicted,
// least recently used first, when a new one does not fit the memory budget.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "csim_batch.h"
#include "csim_host_common.h"

using namespace csim_host;

namespace {
// byte offsets in a round's download block: the thread-per-pair launches' work-queue counter,
// and the count of live states the direct launches leave to the block-prefix kernel
constexpr size_t kQueueOffset = 64;
constexpr size_t kRestCountOffset = 128;
}  // namespace

namespace {

using Clock = std::chrono::steady_clock;

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// thread-per-pair launches: four per occupancy class of t (heavy, light,
// direct narrow, direct wide); a light launch takes codewords of at most the
// light bound's zeros, the direct launches the evaluations the tuner gave the
// direct kernel (tune_for), narrow for the codewords of at most 32 ones
constexpr int kBuckets = 4 * CSIM_MAX_QUBITS;

// device memory that grows on demand (contents are not kept)
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap) return 0;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t c = align_up(bytes + bytes / 4);
        if (cudaMalloc(&p, c) != cudaSuccess) {
            p = nullptr;
            return CSIM_ERR_NOMEM;
        }
        cap = c;
        return 0;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// pinned host memory that grows on demand
struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes) {
        if (bytes <= cap) return 0;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t c = align_up(bytes + bytes / 4);
        if (cudaMallocHost(&p, c) != cudaSuccess) {
            p = nullptr;
            return CSIM_ERR_NOMEM;
        }
        cap = c;
        return 0;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// one decomposition of |H^t> resident on the device
struct Decomp {
    int t = 0, exact = 0, k = 0;
    int64_t chi = 0;
    std::vector<uint64_t> L;
    uint64_t* cw = nullptr;      // codewords (exact == 0), term order
    uint64_t* cws = nullptr;     // the same in ordered_codewords' order, for sampled estimators
    int64_t light = 0;           // first index of cws with at most lz zeros
    int pt = 0, lz = 0;          // thread-per-pair terms per thread and light bound (csim_host::tune_for)
    int kern = 0;                // the tuner's kernel: 3 = direct restriction, else the block-prefix kernel
    csim_state* phis = nullptr;  // term states: prepH (exact == 1), prepL (exact projector on |L>)
    uint64_t* dL = nullptr;
    size_t bytes = 0;
    int refs = 0;
    int64_t last_use = 0;
    void release() {
        if (cw) cudaFree(cw);
        if (cws) cudaFree(cws);
        if (phis) cudaFree(phis);
        if (dL) cudaFree(dL);
        cw = nullptr;
        cws = nullptr;
        phis = nullptr;
        dL = nullptr;
    }
};

struct QueryRec;

// one projector of one query evaluated on the device
struct Eval {
    QueryRec* q = nullptr;
    int which = 0;  // 0 G', 1 H'
    int kind = 1;   // 1 sampled (multiSampledProjector), 2 exactProjector
    int t = 0;
    int64_t chi = 0, ns = 0;
    int samples = 0, bins = 1;
    int64_t next = 0, done = 0;
    std::vector<double> val;  // sampled: value per state; exact: re, im per row
    std::vector<char> live;   // exact: row survived the projection
    int nstabs = 0;
    int32_t pm[64];
    uint64_t pz[64], px[64];
    uint64_t id0 = 0;  // first Philox draw id
    double value = 0;
    bool finished = false;
};

struct QueryRec {
    int64_t ticket = 0;
    csim_query q{};
    std::vector<int32_t> ph[2];
    std::vector<uint64_t> xs[2], zs[2];
    int exact = 0, k = 0, noapprox = 0;
    double norm = 0;
    uint64_t L[CSIM_MAX_QUBITS] = {0};
    int64_t chi = 0;
    LibcRand lr;
    Decomp* dec = nullptr;
    double host_value[2] = {0, 0};
    bool host_only[2] = {false, false};
    std::unique_ptr<Eval> ev[2];
    int pending = 0;
    std::atomic<int64_t> inflight{0};  // its states in rounds not yet read back
    bool admitted = false, done = false;
    csim_query_result res{};
    Clock::time_point t_submit;
};

struct Slot {
    Eval* e;
    int64_t s;
};

// one round's buffers and contents
struct RoundSet {
    DevBuf up, work, down;
    HostBuf hup, hdown;
    cudaEvent_t ev[4] = {};  // start, pair kernels start, pair kernels end, end
    std::vector<Slot> slots;
    int64_t pairs = 0;
    size_t off_codes = 0, off_sum = 0, off_sumd = 0;
};

}  // namespace

// ---------------------------------------------------------------- engine
static bool plan_query(csim_ctx* ctx, QueryRec* r);

class Engine {
  public:
    Engine(csim_ctx* ctx, int64_t round_pairs, int64_t round_states, int per_thread, int64_t budget)
        : ctx_(ctx),
          round_pairs_(round_pairs > 0 ? round_pairs : ((int64_t)1 << 26)),
          round_states_(round_states > 0 ? round_states : ((int64_t)1 << 16)),
          per_thread_(per_thread > 0 ? per_thread : 0),
          budget_(budget > 0 ? budget : ((int64_t)8 << 30)) {}

    ~Engine() {
        cudaStreamSynchronize(ctx_->stream);
        for (auto& rs : sets_) {
            rs.up.release();
            rs.work.release();
            rs.down.release();
            rs.hup.release();
            rs.hdown.release();
            for (auto& e : rs.ev)
                if (e) cudaEventDestroy(e);
        }
        for (auto& kv : decomps_) kv.second->release();
        cum_.release();
        iota_.release();
    }

    int init() {
        csim_ctx* const ctx = ctx_;  // for CK
        for (auto& rs : sets_)
            for (auto& e : rs.ev)
                if (cudaEventCreate(&e) != cudaSuccess) return fail(ctx_, CSIM_ERR_CUDA, "event create failed");
        // randomStabilizerState's cumulative tables for every n (stabilizer.c:694-716)
        std::vector<double> cum(65 * 65, 0.0);
        for (int t = 1; t <= CSIM_MAX_QUBITS; t++) cum_table(t, &cum[65 * t]);
        if (cum_.ensure(cum.size() * 8)) return fail(ctx_, CSIM_ERR_NOMEM, "cum table");
        CK(cudaMemcpy(cum_.p, cum.data(), cum.size() * 8, cudaMemcpyHostToDevice));
        // t buckets of the thread-per-pair launches: consecutive t with the same
        // resident blocks per SM share a launch sized for the bucket's largest t,
        // so no t runs at a lower occupancy than a launch of its own would give
        int occ_prev = -1;
        nbuckets_ = 0;
        for (int t = 1; t <= CSIM_MAX_QUBITS; t++) {
            const int occ = csim::items_tp_occupancy(t, t);
            if (occ <= 0) return fail(ctx_, CSIM_ERR_CUDA, "occupancy query failed");
            if (occ != occ_prev) nbuckets_++;
            occ_prev = occ;
            bucket_of_[t] = nbuckets_ - 1;
            bucket_hi_[nbuckets_ - 1] = t;
        }
        return 0;
    }

    // host plan of one query (decompose, noapprox rule); completes host-only and failed queries
    void plan(QueryRec* r) {
        if (plan_query(ctx_, r)) finished.push_back(r);
    }
    // makes the query's decomposition resident and creates its evaluations;
    // false when it does not fit the memory budget now
    int admit(QueryRec* r, bool force, bool* admitted);
    bool schedulable() const;
    int launch_round();
    int complete_round();
    int inflight() const { return (int)inflight_.size(); }
    int per_thread() const { return per_thread_; }
    bool idle() const { return inflight_.empty() && !schedulable(); }

    // finished queries (the caller collects them)
    std::vector<QueryRec*> finished;

    int64_t rounds = 0, pairs = 0, states = 0, states_live = 0;
    double device_ms = 0, pair_ms = 0;
    int64_t resident_bytes() const { return resident_; }
    int64_t resident_count() const { return (int64_t)decomps_.size(); }

  private:
    csim_ctx* ctx_;
    int64_t round_pairs_, round_states_;
    int per_thread_;
    int64_t budget_;
    int64_t resident_ = 0, use_clock_ = 0;
    std::map<std::vector<uint64_t>, std::unique_ptr<Decomp>> decomps_;
    std::vector<Eval*> active_;
    RoundSet sets_[2];
    int next_set_ = 0;
    std::deque<RoundSet*> inflight_;
    DevBuf cum_, iota_;
    int64_t iota_n_ = 0;
    int bucket_of_[CSIM_MAX_QUBITS + 1] = {0};
    int bucket_hi_[kBuckets] = {0};
    int nbuckets_ = 0;

    csim::Launch launch_on(int* d_err) { return csim::Launch{ctx_->stream, d_err, &ctx_->launches, ctx_->num_sms}; }
    int ensure_decomp(QueryRec* r, bool need_phis, bool force, Decomp** out);
    void finish_eval(Eval* e);
    void finish_query(QueryRec* r);
    void fail_query(QueryRec* r, int status);
    bool eval_ready(const Eval* e) const;
};

static bool plan_fail(QueryRec* r, int status) {
    r->res.status = status;
    r->done = true;
    return true;
}

// Host plan of one query: decompose (its fidelity sum on ctx's GPU), the noapprox
// rule and the answers that need no device work (probability.c:146-174,
// innerprod.c:47-62, :150).  Returns true when the query is complete already
// (answered on the host, or failed); its result is in r->res.
static bool plan_query(csim_ctx* ctx, QueryRec* r) {
    const csim_query& Q = r->q;
    csim_query_result& R = r->res;
    R = csim_query_result{};
    if (Q.t < 0 || Q.t > CSIM_MAX_QUBITS || (Q.rng != CSIM_RNG_LIBC && Q.rng != CSIM_RNG_PHILOX) ||
        check_projector(ctx, &Q.G) || check_projector(ctx, &Q.H) || (Q.G.nstabs && Q.G.nqubits != Q.t) ||
        (Q.H.nstabs && Q.H.nqubits != Q.t) || Q.G.nstabs > 64 || Q.H.nstabs > 64) {
        return plan_fail(r, fail(ctx, CSIM_ERR_ARG, "query %lld: bad t, rng or projectors", (long long)r->ticket));
    }
    // decompose() runs on rand()'s default stream, before the sampler is seeded (probability.c:146-153)
    LibcRand ds;
    ds.seed(1);
    r->exact = Q.exact;
    r->k = Q.k;
    const int rc = csim_decompose_on(ctx, Q.t, Q.fidbound, Q.rank, Q.fidelity, Q.force_l, Q.verbose, Q.quiet,
                                     &r->exact, &r->k, &r->norm, r->L, &ds, nullptr);
    if (rc != CSIM_OK) return plan_fail(r, rc);
    r->noapprox = Q.noapprox;
    if (Q.noapprox == 0 && Q.force_sample == 0) {  // probability.c:162-174
        const double terms = r->exact ? pow(2, (Q.t + 1) / 2) : pow(2, r->k);
        if (Q.samples * Q.bins * 2 > (terms - 1)) r->noapprox = 1;
    }
    if (r->noapprox == 0 && (Q.bins < 1 || Q.samples < 0)) {
        return plan_fail(r, fail(ctx, CSIM_ERR_ARG, "query %lld: samples=%d bins=%d", (long long)r->ticket,
                                  Q.samples, Q.bins));
    }
    R.exact = r->exact;
    R.k = r->k;
    R.noapprox = r->noapprox;
    R.norm = r->norm;
    r->chi = Q.t == 0 ? 0 : (r->exact ? ((int64_t)1 << ((Q.t + 1) / 2)) : ((int64_t)1 << r->k));
    for (int w = 0; w < 2; w++) {
        const csim_projector& P = w == 0 ? Q.G : Q.H;
        if (P.nstabs == 0) {  // innerprod.c:47 / :150
            r->host_only[w] = true;
            r->host_value[w] = pow(r->norm, 2);
        } else if (Q.t == 0) {  // innerprod.c:52-62; exactProjector's branch has no norm^2
            r->host_only[w] = true;
            r->host_value[w] = (r->noapprox ? 1.0 : pow(r->norm, 2)) * clifford_sum(&P) / (1 + (double)P.nstabs);
        }
    }
    if (!(r->host_only[0] && r->host_only[1])) {
        if (check_code(ctx, Q.t, r->exact, r->L, r->k)) return plan_fail(r, CSIM_ERR_ARG);
        if (r->noapprox && r->chi > ((int64_t)1 << 20))
            return plan_fail(r, fail(ctx, CSIM_ERR_ARG, "query %lld: chi too large for the exact projector",
                                     (long long)r->ticket));
        return false;
    }
    r->res.numerator = r->host_value[0];
    r->res.denominator = r->host_value[1];
    r->done = true;
    return true;
}

int Engine::ensure_decomp(QueryRec* r, bool need_phis, bool force, Decomp** out) {
    csim_ctx* const ctx = ctx_;  // for CK
    *out = nullptr;
    std::vector<uint64_t> key = {(uint64_t)r->q.t, (uint64_t)r->exact, (uint64_t)(r->exact ? 0 : r->k)};
    if (!r->exact) key.insert(key.end(), r->L, r->L + r->k);
    auto it = decomps_.find(key);
    Decomp* d = it == decomps_.end() ? nullptr : it->second.get();
    const int64_t chi = r->chi;
    const bool want_cw = !r->exact, want_phis = r->exact || need_phis;
    size_t add = 0;
    if (!d && want_cw) add += 2 * align_up((size_t)chi * 8) + kAlign;
    if (want_phis && !(d && d->phis)) add += align_up((size_t)chi * sizeof(csim_state));
    if (add && resident_ + (int64_t)add > budget_) {  // evict unused decompositions, least recently used first
        std::vector<std::pair<int64_t, std::vector<uint64_t>>> lru;
        for (auto& kv : decomps_)
            if (kv.second->refs == 0 && kv.second.get() != d) lru.push_back({kv.second->last_use, kv.first});
        std::sort(lru.begin(), lru.end());
        for (auto& e : lru) {
            if (resident_ + (int64_t)add <= budget_) break;
            auto jt = decomps_.find(e.second);
            cudaStreamSynchronize(ctx_->stream);
            resident_ -= (int64_t)jt->second->bytes;
            jt->second->release();
            decomps_.erase(jt);
        }
        if (resident_ + (int64_t)add > budget_ && !force) return 0;
    }
    if (!d) {
        auto nd = std::make_unique<Decomp>();
        nd->t = r->q.t;
        nd->exact = r->exact;
        nd->k = r->exact ? 0 : r->k;
        nd->chi = chi;
        nd->L.assign(r->L, r->L + (r->exact ? 0 : r->k));
        d = nd.get();
        decomps_[key] = std::move(nd);
        if (want_cw) {
            if (cudaMalloc(&d->cw, (size_t)chi * 8) != cudaSuccess ||
                cudaMalloc(&d->cws, (size_t)chi * 8) != cudaSuccess ||
                cudaMalloc(&d->dL, 8 * (size_t)CSIM_MAX_QUBITS) != cudaSuccess) {
                d->release();
                decomps_.erase(key);
                return fail(ctx_, CSIM_ERR_NOMEM, "codeword table of 2^%d terms", r->k);
            }
            d->bytes += 2 * align_up((size_t)chi * 8) + kAlign;
            TpTune tn;
            const csim_projector* Pw = r->q.G.nstabs > 0 ? &r->q.G : (r->q.H.nstabs > 0 ? &r->q.H : nullptr);
            if (const int rc = tune_for(ctx_, d->t, &tn, Pw, d->L.data(), d->k)) {
                d->release();
                decomps_.erase(key);
                return rc;
            }
            d->pt = tn.per_thread;
            d->kern = tn.kernel;
            // the items kernel shares top bits per block; the direct kernel's bound splits narrow from wide
            d->lz = (tn.kernel == 0 || tn.kernel == 3) ? tn.light : light_zeros(d->t);
            std::vector<uint64_t> ordered;
            ordered_codewords(d->L.data(), d->k, d->t, d->lz, ordered);
            d->light = light_split(ordered, d->t, d->lz);
            CK(cudaMemcpy(d->cws, ordered.data(), (size_t)chi * 8, cudaMemcpyHostToDevice));
            uint64_t rows[CSIM_MAX_QUBITS] = {0};
            for (int i = 0; i < d->k; i++) rows[i] = d->L[i];
            CK(cudaMemcpy(d->dL, rows, sizeof(rows), cudaMemcpyHostToDevice));
            if (csim::launch_codewords(launch_of(ctx_), d->dL, d->k, 0, chi, d->cw))
                return fail(ctx_, CSIM_ERR_CUDA, "codeword launch failed");
        }
        resident_ += (int64_t)d->bytes;
    }
    if (want_phis && !d->phis) {
        if (cudaMalloc(&d->phis, (size_t)chi * sizeof(csim_state)) != cudaSuccess) {
            d->phis = nullptr;
            return fail(ctx_, CSIM_ERR_NOMEM, "term states of 2^%lld terms", (long long)chi);
        }
        d->bytes += align_up((size_t)chi * sizeof(csim_state));
        resident_ += (int64_t)align_up((size_t)chi * sizeof(csim_state));
        if (d->exact) {
            if (iota_n_ < chi) {  // prepH term indices 0..chi-1
                std::vector<int64_t> idx(chi);
                for (int64_t j = 0; j < chi; j++) idx[j] = j;
                cudaStreamSynchronize(ctx_->stream);
                if (iota_.ensure((size_t)chi * 8)) return fail(ctx_, CSIM_ERR_NOMEM, "term indices");
                CK(cudaMemcpy(iota_.p, idx.data(), (size_t)chi * 8, cudaMemcpyHostToDevice));
                iota_n_ = chi;
            }
            if (csim::launch_prep(launch_of(ctx_), d->t, 1, nullptr, (const int64_t*)iota_.p, chi,
                                  (csim::GState*)d->phis))
                return fail(ctx_, CSIM_ERR_CUDA, "prepH launch failed");
        } else if (csim::launch_prep(launch_of(ctx_), d->t, 0, d->cw, nullptr, chi, (csim::GState*)d->phis)) {
            return fail(ctx_, CSIM_ERR_CUDA, "prepL launch failed");
        }
    }
    d->last_use = ++use_clock_;
    *out = d;
    return 0;
}

int Engine::admit(QueryRec* r, bool force, bool* admitted) {
    *admitted = false;
    if (r->done) {
        *admitted = true;
        return 0;
    }
    Decomp* d = nullptr;
    const int rc = ensure_decomp(r, r->noapprox != 0, force, &d);
    if (rc) {
        fail_query(r, rc);
        *admitted = true;
        return 0;
    }
    if (!d) return 0;  // does not fit yet
    d->refs++;
    r->dec = d;
    r->admitted = true;
    *admitted = true;
    const csim_query& Q = r->q;
    uint64_t philox_next = 0;
    if (Q.rng == CSIM_RNG_LIBC) r->lr.seed((uint32_t)Q.seed);
    for (int w = 0; w < 2; w++) {
        if (r->host_only[w]) continue;
        const csim_projector& P = w == 0 ? Q.G : Q.H;
        auto e = std::make_unique<Eval>();
        e->q = r;
        e->which = w;
        e->kind = r->noapprox ? 2 : 1;
        e->t = Q.t;
        e->chi = r->chi;
        e->samples = Q.samples;
        e->bins = Q.bins;
        e->ns = e->kind == 1 ? (int64_t)Q.samples * Q.bins : r->chi;
        e->nstabs = P.nstabs;
        for (int i = 0; i < P.nstabs; i++) {
            e->pm[i] = phase_m(P.phase[i]);
            e->pz[i] = P.zs[i];
            e->px[i] = P.xs[i];
        }
        e->id0 = philox_next;
        if (e->kind == 1) philox_next += (uint64_t)e->ns;
        e->val.assign(e->kind == 1 ? (size_t)e->ns : 2 * (size_t)e->ns, 0.0);
        if (e->kind == 2) e->live.assign((size_t)e->ns, 0);
        r->pending++;
        r->ev[w] = std::move(e);
    }
    for (int w = 0; w < 2; w++)
        if (r->ev[w]) {
            if (r->ev[w]->ns == 0) finish_eval(r->ev[w].get());
            else active_.push_back(r->ev[w].get());
        }
    return 0;
}

// first item (of span terms, from term 0) of a sampled evaluation whose codewords all
// have at most its decomposition's light bound of zeros in the ordered table
static int64_t light_first_item(const Eval* e, int64_t span) {
    return std::min((e->chi + span - 1) / span, (e->q->dec->light + span - 1) / span);
}

// Items of a direct-kernel evaluation whose codewords all have at most 32 ones
// (the ordered table's heavy part above 32 qubits, whole items only); the
// exactProjector's rows walk the table in term order and take none.
static int64_t direct_narrow_items(const Eval* e, int64_t span) {
    if (e->kind != 1 || e->t <= 32) return 0;
    return std::min((e->chi + span - 1) / span, e->q->dec->light / span);
}

bool Engine::eval_ready(const Eval* e) const {
    if (e->next >= e->ns) return false;
    // rand() draws: H' continues G''s stream, so its states are drawn after all of G''s
    if (e->which == 1 && e->kind == 1 && e->q->q.rng == CSIM_RNG_LIBC && e->q->ev[0] && e->q->ev[0]->kind == 1 &&
        e->q->ev[0]->next < e->q->ev[0]->ns)
        return false;
    return true;
}

bool Engine::schedulable() const {
    for (const Eval* e : active_)
        if (eval_ready(e)) return true;
    return false;
}

int Engine::launch_round() {
    csim_ctx* const ctx = ctx_;  // for CK
    RoundSet& rs = sets_[next_set_];
    next_set_ ^= 1;
    rs.slots.clear();
    rs.pairs = 0;
    // pick states: a fair share per evaluation first, then first come first served
    int nready = 0;
    for (Eval* e : active_) nready += eval_ready(e) ? 1 : 0;
    const int64_t share = std::max<int64_t>(1, round_pairs_ / std::max(1, nready));
    auto cost = [](const Eval* e) { return e->kind == 1 ? e->chi : e->chi - e->next; };
    for (int pass = 0; pass < 2; pass++) {
        for (Eval* e : active_) {
            int64_t mine = 0;
            while (eval_ready(e) && (int64_t)rs.slots.size() < round_states_) {
                const int64_t c = cost(e);
                if (!rs.slots.empty() && rs.pairs + c > round_pairs_) break;
                if (pass == 0 && mine > 0 && mine + c > share) break;
                rs.slots.push_back(Slot{e, e->next});
                e->q->inflight++;
                e->next++;
                rs.pairs += c;
                mine += c;
            }
        }
    }
    const int64_t ns = (int64_t)rs.slots.size();
    if (ns == 0) return 0;

    // rand() words of the sampled states with the C library's draws, each query's states in its own
    // stream order (G' then H'); queries are independent streams, so they are drawn on host threads
    // of their own (at t = 64 a state takes about 2000 words)
    std::vector<std::pair<int64_t, int64_t>> wr(ns, {0, 0});
    struct WordJob {
        QueryRec* q;
        int t;
        std::vector<int64_t> slots;
        std::vector<uint32_t> words;
        std::vector<int64_t> ends;
    };
    std::vector<WordJob> jobs;
    {
        std::map<QueryRec*, size_t> jix;
        for (int64_t i = 0; i < ns; i++) {
            Eval* e = rs.slots[i].e;
            if (e->kind != 1 || e->q->q.rng != CSIM_RNG_LIBC) continue;
            auto it = jix.find(e->q);
            if (it == jix.end()) {
                it = jix.emplace(e->q, jobs.size()).first;
                jobs.push_back(WordJob{e->q, e->t, {}, {}, {}});
            }
            jobs[it->second].slots.push_back(i);
        }
        auto run_job = [](WordJob& j) {
            double cum[CSIM_MAX_QUBITS + 1];
            cum_table(j.t, cum);
            j.ends.reserve(j.slots.size());
            for (size_t k = 0; k < j.slots.size(); k++) {
                draw_state_words(j.q->lr, j.t, cum, j.words);
                j.ends.push_back((int64_t)j.words.size());
            }
        };
        const int nthreads = (int)std::min<size_t>(jobs.size(), std::max(1u, std::thread::hardware_concurrency()));
        if (nthreads <= 1) {
            for (auto& j : jobs) run_job(j);
        } else {
            std::atomic<size_t> next{0};
            std::vector<std::thread> pool;
            for (int w = 0; w < nthreads; w++)
                pool.emplace_back([&] {
                    for (size_t j; (j = next.fetch_add(1)) < jobs.size();) run_job(jobs[j]);
                });
            for (auto& th : pool) th.join();
        }
    }
    int64_t nwords = 0;
    for (auto& j : jobs) {
        for (size_t k = 0; k < j.slots.size(); k++)
            wr[j.slots[k]] = {nwords + (k ? j.ends[k - 1] : 0), nwords + j.ends[k]};
        nwords += (int64_t)j.words.size();
    }
    std::map<Eval*, int> evix;  // evaluations in this round -> projector block
    // thread-per-pair items are grouped by t bucket: each bucket's launch sizes
    // its shared memory for that bucket's largest t, not the round's
    int64_t nbucket[kBuckets] = {0};
    int64_t niw = 0;
    // thread-per-pair items of an evaluation: 64 * tp_per_thread(t) terms each;
    // a launch runs as many rows per thread as its longest items need
    auto span_tp_of = [this](const Eval* e) { return 64 * (int64_t)(per_thread_ > 0 ? per_thread_ : e->q->dec->pt); };
    const int launch_pt = per_thread_ > 0 ? per_thread_ : 32;  // the largest item any t is tuned to
    int lzmax[kBuckets] = {0};  // per light launch: the largest light bound of its items
    const int64_t span_w = 64;
    for (int64_t i = 0; i < ns; i++) {
        Eval* e = rs.slots[i].e;
        if (!evix.count(e)) {
            const int ix = (int)evix.size();
            evix[e] = ix;
        }
        const int64_t jb = e->kind == 2 ? rs.slots[i].s : 0;
        const int64_t nj = e->chi - jb;
        if (!e->q->exact) {
            const int b = 4 * bucket_of_[e->t];
            const int64_t span_tp = span_tp_of(e);
            const int64_t nall = (nj + span_tp - 1) / span_tp;
            if (e->q->dec->kern == 3) {
                const int64_t nn = direct_narrow_items(e, span_tp);
                nbucket[b + 2] += nn;
                nbucket[b + 3] += nall - nn;
                continue;
            }
            const int64_t nlight = e->kind == 1 ? nall - light_first_item(e, span_tp) : 0;
            nbucket[b] += nall - nlight;
            nbucket[b + 1] += nlight;
            if (nlight) lzmax[b + 1] = std::max(lzmax[b + 1], e->q->dec->lz);
        } else {
            niw += (nj + span_w - 1) / span_w;
        }
    }
    int64_t bstart[kBuckets + 1];
    bstart[0] = 0;
    for (int b = 0; b < kBuckets; b++) bstart[b + 1] = bstart[b] + nbucket[b];
    const int64_t nitp = bstart[kBuckets];
    const int64_t nitems = nitp + niw;
    // upload block: desc | proj | words | items | ranges
    const size_t o_desc = 0;
    const size_t o_proj = align_up(o_desc + (size_t)ns * sizeof(csim::DrawDesc));
    const size_t o_words = align_up(o_proj + evix.size() * 192 * 8);
    const size_t o_items = align_up(o_words + (size_t)nwords * 4);
    const size_t o_range = align_up(o_items + (size_t)nitems * sizeof(csim::PairItem));
    const size_t o_range2 = align_up(o_range + (size_t)ns * 16);
    const size_t up_bytes = align_up(o_range2 + (size_t)ns * 16);
    bool any_direct = false;
    for (int b = 0; b < kBuckets; b++) any_direct |= b % 4 >= 2 && nbucket[b] > 0;
    // work block: states | parts | parts diag | pivot forms | direct and rest codes (direct launches)
    const size_t w_states = 0;
    const size_t w_part = align_up((size_t)ns * sizeof(csim_state));
    const size_t w_partd = align_up(w_part + (size_t)std::max<int64_t>(nitems, 1) * 64);
    const size_t w_canon = align_up(w_partd + (size_t)std::max<int64_t>(nitems, 1) * 64);
    const size_t w_cdir = align_up(w_canon + (any_direct ? (size_t)ns * csim::canon_bytes() : 0));
    const size_t w_crest = align_up(w_cdir + (any_direct ? (size_t)ns * 4 : 0));
    const size_t work_bytes = align_up(w_crest + (any_direct ? (size_t)ns * 4 : 0));
    // download block: err (16 B), the pair launches' work-queue counter (kQueueOffset) | codes | sums | sums diag
    rs.off_codes = 256;
    rs.off_sum = align_up(rs.off_codes + (size_t)ns * 4);
    rs.off_sumd = align_up(rs.off_sum + (size_t)ns * 64);
    const size_t down_bytes = align_up(rs.off_sumd + (size_t)ns * 64);
    if (rs.up.ensure(up_bytes) || rs.work.ensure(work_bytes) || rs.down.ensure(down_bytes) ||
        rs.hup.ensure(up_bytes) || rs.hdown.ensure(down_bytes))
        return fail(ctx_, CSIM_ERR_NOMEM, "round buffers (%lld states, %lld items)", (long long)ns,
                    (long long)nitems);
    unsigned char* hb = (unsigned char*)rs.hup.p;
    unsigned char* db = (unsigned char*)rs.up.p;
    unsigned char* wb = (unsigned char*)rs.work.p;
    unsigned char* dd = (unsigned char*)rs.down.p;
    uint64_t* hproj = (uint64_t*)(hb + o_proj);
    for (auto& kv : evix) {
        uint64_t* blk = hproj + 192 * kv.second;
        memset(blk, 0, 192 * 8);
        memcpy(blk, kv.first->pm, sizeof(int32_t) * kv.first->nstabs);
        memcpy(blk + 64, kv.first->pz, 8 * kv.first->nstabs);
        memcpy(blk + 128, kv.first->px, 8 * kv.first->nstabs);
    }
    {
        size_t o = 0;
        for (auto& j : jobs) {
            if (!j.words.empty()) memcpy(hb + o_words + 4 * o, j.words.data(), j.words.size() * 4);
            o += j.words.size();
        }
    }
    const uint64_t* dproj = (const uint64_t*)(db + o_proj);
    const uint32_t* dwords = (const uint32_t*)(db + o_words);
    csim::DrawDesc* hdesc = (csim::DrawDesc*)(hb + o_desc);
    csim::PairItem* hitems = (csim::PairItem*)(hb + o_items);
    int64_t* hrange = (int64_t*)(hb + o_range);    // a slot's items in its heavy or warp launch
    int64_t* hrange2 = (int64_t*)(hb + o_range2);  // and in its light launch
    const double* dcum = (const double*)cum_.p;
    const csim::GState* dstates = (const csim::GState*)(wb + w_states);
    int64_t cur[kBuckets];
    for (int b = 0; b < kBuckets; b++) cur[b] = bstart[b];
    int64_t iw = nitp;
    for (int64_t i = 0; i < ns; i++) {
        Eval* e = rs.slots[i].e;
        const int64_t s = rs.slots[i].s;
        const QueryRec* r = e->q;
        const int b = evix[e];
        csim::DrawDesc d{};
        d.n = e->t;
        d.nstabs = e->nstabs;
        d.cum = dcum + 65 * e->t;
        d.pm = (const int32_t*)(dproj + 192 * b);
        d.pz = dproj + 192 * b + 64;
        d.px = dproj + 192 * b + 128;
        if (e->kind == 2) {
            d.mode = 2;
            d.src = (const csim::GState*)(r->dec->phis + s);
        } else if (r->q.rng == CSIM_RNG_LIBC) {
            d.mode = 1;
            d.words = dwords;
            d.wbegin = wr[i].first;
            d.wend = wr[i].second;
        } else {
            d.mode = 0;
            d.seed = r->q.seed;
            d.id = e->id0 + (uint64_t)s;
        }
        hdesc[i] = d;
        const int64_t jb = e->kind == 2 ? s : 0;
        const int64_t diag = e->kind == 2 ? s : -1;
        if (!r->exact && r->dec->kern == 3) {
            // a slot's items in its bucket's direct launches: narrow ones, then wide ones
            const int64_t span_tp = span_tp_of(e);
            const int b = 4 * bucket_of_[e->t];
            const int64_t jn = jb + direct_narrow_items(e, span_tp) * span_tp;
            const uint64_t* cw = e->kind == 1 ? r->dec->cws : r->dec->cw;
            int64_t& cn = cur[b + 2];
            int64_t& cd = cur[b + 3];
            hrange[2 * i] = cn;
            for (int64_t j = jb; j < jn; j += span_tp)
                hitems[cn++] = csim::PairItem{i, j, std::min(span_tp, e->chi - j), diag, cw, nullptr};
            hrange[2 * i + 1] = cn;
            hrange2[2 * i] = cd;
            for (int64_t j = jn; j < e->chi; j += span_tp)
                hitems[cd++] = csim::PairItem{i, j, std::min(span_tp, e->chi - j), diag, cw, nullptr};
            hrange2[2 * i + 1] = cd;
        } else if (!r->exact) {
            // heavy items first, then light ones; a slot's items may sit in two
            // launches, so its range is kept per slot in each (see below)
            const int b = 4 * bucket_of_[e->t];
            const int64_t span_tp = span_tp_of(e);
            const int64_t jl = e->kind == 1 ? light_first_item(e, span_tp) * span_tp : e->chi;
            int64_t& ch = cur[b];
            int64_t& cl = cur[b + 1];
            hrange[2 * i] = ch;
            for (int64_t j = jb; j < std::min(jl, e->chi); j += span_tp)
                hitems[ch++] = csim::PairItem{i, j, std::min(span_tp, e->chi - j), diag,
                                              e->kind == 1 ? r->dec->cws : r->dec->cw, nullptr};
            hrange[2 * i + 1] = ch;
            hrange2[2 * i] = cl;
            for (int64_t j = std::max(jl, jb); j < e->chi; j += span_tp)
                hitems[cl++] = csim::PairItem{i, j, std::min(span_tp, e->chi - j), diag, r->dec->cws, nullptr};
            hrange2[2 * i + 1] = cl;
        } else {
            hrange2[2 * i] = hrange2[2 * i + 1] = 0;
            hrange[2 * i] = iw;
            for (int64_t j = jb; j < e->chi; j += span_w)
                hitems[iw++] = csim::PairItem{i, j, std::min(span_w, e->chi - j), diag, nullptr,
                                              (const csim::GState*)r->dec->phis};
            hrange[2 * i + 1] = iw;
        }
    }
    int* derr = (int*)dd;
    const csim::Launch L = launch_on(derr);
    CK(cudaEventRecord(rs.ev[0], ctx_->stream));
    CK(cudaMemcpyAsync(db, hb, up_bytes, cudaMemcpyHostToDevice, ctx_->stream));
    CK(cudaMemsetAsync(derr, 0, 16, ctx_->stream));
    __int128* part = (__int128*)(wb + w_part);
    __int128* partd = (__int128*)(wb + w_partd);
    int* dcode = (int*)(dd + rs.off_codes);
    if (csim::launch_draw_project(L, (const csim::DrawDesc*)(db + o_desc), ns, (csim::GState*)(wb + w_states), dcode))
        return fail(ctx_, CSIM_ERR_CUDA, "draw/project launch failed");
    CK(cudaEventRecord(rs.ev[1], ctx_->stream));
    const csim::PairItem* ditems = (const csim::PairItem*)(db + o_items);
    unsigned long long* const queue = (unsigned long long*)(dd + kQueueOffset);
    // direct launches: the states in pivot form; those with more non-pivot
    // coordinates than the constraint slots go to the block-prefix kernel
    const int dslots_max = ctx_->direct_slots > 0 ? ctx_->direct_slots : direct_slots(CSIM_MAX_QUBITS);
    void* const canon = wb + w_canon;
    int* const cdir = (int*)(wb + w_cdir);
    int* const crest = (int*)(wb + w_crest);
    int* const rest_count = (int*)(dd + kRestCountOffset);
    if (any_direct) {
        CK(cudaMemsetAsync(rest_count, 0, 4, ctx_->stream));
        if (csim::launch_canon(L, dstates, dcode, ns, dslots_max, canon, cdir, crest, rest_count))
            return fail(ctx_, CSIM_ERR_CUDA, "pivot form launch failed");
    }
    for (int b = 0; b < 4 * nbuckets_; b++) {
        const int nmax = bucket_hi_[b / 4];
        const csim::PairItem* it = ditems + bstart[b];
        int rc = 0;
        if (b % 4 >= 2) {
            // narrow items take 32 J rows per pair; after the wide launch, the states left to the
            // block-prefix kernel over both (adjacent in the table)
            if (nbucket[b])
                rc = csim::launch_items_direct(L, it, nbucket[b], canon, cdir, crest, launch_pt, nmax,
                                               b % 4 == 2 ? std::min(nmax, 32) : nmax, std::min(nmax, dslots_max),
                                               part + 4 * bstart[b], partd + 4 * bstart[b], queue);
            const int64_t nd = nbucket[b - 1] + nbucket[b];
            if (!rc && b % 4 == 3 && nd)
                rc = csim::launch_items_tp(L, ditems + bstart[b - 1], nd, dstates, crest, launch_pt, nmax, nmax,
                                           part + 4 * bstart[b - 1], partd + 4 * bstart[b - 1], queue, true,
                                           rest_count);
        } else if (nbucket[b]) {
            const int gmax = b % 4 == 1 ? std::min(nmax, lzmax[b]) : nmax;
            rc = csim::launch_items_tp(L, it, nbucket[b], dstates, dcode, launch_pt, nmax, gmax, part + 4 * bstart[b],
                                       partd + 4 * bstart[b], queue);
        }
        if (rc) return fail(ctx_, CSIM_ERR_CUDA, "pair launch failed");
    }
    if (csim::launch_items_warp(L, ditems + nitp, niw, dstates, dcode, part + 4 * nitp, partd + 4 * nitp))
        return fail(ctx_, CSIM_ERR_CUDA, "pair launch failed");
    CK(cudaEventRecord(rs.ev[2], ctx_->stream));
    const int64_t* drange = (const int64_t*)(db + o_range);
    const int64_t* drange2 = (const int64_t*)(db + o_range2);
    if (csim::launch_reduce_slots(L, part, drange, drange2, ns, (__int128*)(dd + rs.off_sum)) ||
        csim::launch_reduce_slots(L, partd, drange, drange2, ns, (__int128*)(dd + rs.off_sumd)))
        return fail(ctx_, CSIM_ERR_CUDA, "reduce launch failed");
    CK(cudaMemcpyAsync(rs.hdown.p, dd, down_bytes, cudaMemcpyDeviceToHost, ctx_->stream));
    CK(cudaEventRecord(rs.ev[3], ctx_->stream));
    ctx_->stats.h2d_bytes += (int64_t)up_bytes;
    ctx_->stats.d2h_bytes += (int64_t)down_bytes;
    inflight_.push_back(&rs);
    rounds++;
    return 0;
}

int Engine::complete_round() {
    csim_ctx* const ctx = ctx_;  // for CK
    if (inflight_.empty()) return 0;
    RoundSet& rs = *inflight_.front();
    inflight_.pop_front();
    CK(cudaEventSynchronize(rs.ev[3]));
    float a = 0, b = 0;
    CK(cudaEventElapsedTime(&a, rs.ev[0], rs.ev[3]));
    CK(cudaEventElapsedTime(&b, rs.ev[1], rs.ev[2]));
    device_ms += a;
    pair_ms += b;
    const unsigned char* hd = (const unsigned char*)rs.hdown.p;
    const int err = *(const int*)hd;
    const int* code = (const int*)(hd + rs.off_codes);
    const __int128* sum = (const __int128*)(hd + rs.off_sum);
    const __int128* sumd = (const __int128*)(hd + rs.off_sumd);
    if (err) {
        fail(ctx_, CSIM_ERR_DEVICE, "kernel flagged error bits 0x%x (1 range, 2 replay, 4 expsum, 8 gamma, 16 arg)",
             err);
        for (const Slot& sl : rs.slots)
            if (!sl.e->q->done) fail_query(sl.e->q, CSIM_ERR_DEVICE);
        for (const Slot& sl : rs.slots) sl.e->q->inflight--;
        return 0;
    }
    for (size_t i = 0; i < rs.slots.size(); i++) {
        Eval* e = rs.slots[i].e;
        const int64_t s = rs.slots[i].s;
        e->q->inflight--;
        if (e->q->done) continue;  // failed in an earlier round
        const int P2 = 2 * e->t;
        states++;
        if (code[i] >= 0) {
            states_live++;
            const int64_t np = e->kind == 1 ? e->chi : e->chi - s;
            pairs += np;
            e->q->res.pairs += np;
            const double pf = sqrt_half_power(code[i]);
            double re, im;
            if (e->kind == 1) {  // singleProjectorSample's value, innerprod.c:142
                zomega_to_complex(&sum[4 * i], P2, &re, &im);
                const double x = re * pf, y = im * pf;
                e->val[s] = pow(2, e->t) * (x * x + y * y);
            } else {  // exactProjector row s: diag + 2 Re(off), innerprod.c:187-195
                const __int128* o = &sum[4 * i];
                const __int128* d = &sumd[4 * i];
                const __int128 z[4] = {d[0] + 2 * o[0], d[1] + (o[1] - o[3]), d[2], d[3] - (o[1] - o[3])};
                zomega_to_complex(z, P2, &re, &im);
                e->val[2 * s] = re * pf;
                e->val[2 * s + 1] = im * pf;
                e->live[s] = 1;
            }
        }
        e->done++;
        if (e->done == e->ns) finish_eval(e);
    }
    return 0;
}

void Engine::finish_eval(Eval* e) {
    if (e->finished) return;
    e->finished = true;
    if (e->kind == 1) {  // multiSampledProjector, innerprod.c:64-84
        e->value = median_of_means(e->val.data(), e->samples, e->bins);
    } else {  // rows summed in row order, innerprod.c:187-198
        double tr = 0, ti = 0;
        for (int64_t s = 0; s < e->ns; s++)
            if (e->live[s]) {
                tr += e->val[2 * s];
                ti += e->val[2 * s + 1];
            }
        e->value = sqrt(tr * tr + ti * ti);
    }
    e->val.clear();
    e->val.shrink_to_fit();
    active_.erase(std::remove(active_.begin(), active_.end(), e), active_.end());
    QueryRec* r = e->q;
    if (--r->pending == 0 && !r->done) finish_query(r);
}

void Engine::finish_query(QueryRec* r) {
    r->res.numerator = r->host_only[0] ? r->host_value[0] : r->ev[0]->value;
    r->res.denominator = r->host_only[1] ? r->host_value[1] : r->ev[1]->value;
    r->res.status = CSIM_OK;
    r->done = true;
    if (r->dec) {
        r->dec->refs--;
        r->dec = nullptr;
    }
    finished.push_back(r);
}

void Engine::fail_query(QueryRec* r, int status) {
    if (r->done) return;
    r->res.status = status;
    r->done = true;
    for (auto& e : r->ev)
        if (e) active_.erase(std::remove(active_.begin(), active_.end(), e.get()), active_.end());
    if (r->dec) {
        r->dec->refs--;
        r->dec = nullptr;
    }
    finished.push_back(r);
}

// ---------------------------------------------------------------- queries in, results out
namespace {

void copy_query(const csim_query& in, QueryRec* r) {
    r->q = in;
    for (int w = 0; w < 2; w++) {
        const csim_projector& P = w == 0 ? in.G : in.H;
        csim_projector& D = w == 0 ? r->q.G : r->q.H;
        const int n = (P.nstabs > 0 && P.nstabs <= 64 && P.phase && P.xs && P.zs) ? P.nstabs : 0;
        r->ph[w].assign(P.phase, P.phase + n);
        r->xs[w].assign(P.xs, P.xs + n);
        r->zs[w].assign(P.zs, P.zs + n);
        if (n) {
            D.phase = r->ph[w].data();
            D.xs = r->xs[w].data();
            D.zs = r->zs[w].data();
        }
    }
}

}  // namespace

extern "C" int csim_run_queries(csim_ctx* ctx, int64_t nq, const csim_query* q, csim_query_result* r,
                                int32_t batched) {
    if (!ctx || nq < 0 || (nq && (!q || !r))) return fail(ctx, CSIM_ERR_ARG, "bad argument");
    cudaSetDevice(ctx->device);
    int first_err = CSIM_OK;
    if (!batched) {  // one query after another through the single-query entry points
        for (int64_t i = 0; i < nq; i++) {
            QueryRec rec;
            rec.ticket = i;
            copy_query(q[i], &rec);
            plan_query(ctx, &rec);
            r[i] = rec.res;
            if (rec.done) {
                if (r[i].status && !first_err) first_err = r[i].status;
                continue;
            }
            const csim_query& Q = q[i];
            int rc;
            int64_t pairs = 0;
            if (rec.noapprox == 0) {
                rc = csim_multi_sampled_projector(ctx, &Q.G, rec.L, rec.k, rec.exact, rec.norm, Q.samples, Q.bins,
                                                  Q.rng, Q.rng == CSIM_RNG_LIBC ? (uint64_t)(uint32_t)Q.seed : Q.seed,
                                                  &r[i].numerator);
                pairs += ctx->stats.pairs;
                if (rc == CSIM_OK)
                    rc = csim_multi_sampled_projector(ctx, &Q.H, rec.L, rec.k, rec.exact, rec.norm, Q.samples, Q.bins,
                                                      Q.rng, CSIM_SEED_CONTINUE, &r[i].denominator);
                pairs += ctx->stats.pairs;
            } else {
                rc = csim_exact_projector(ctx, &Q.G, rec.L, rec.k, rec.exact, rec.norm, &r[i].numerator);
                pairs += ctx->stats.pairs;
                if (rc == CSIM_OK)
                    rc = csim_exact_projector(ctx, &Q.H, rec.L, rec.k, rec.exact, rec.norm, &r[i].denominator);
                pairs += ctx->stats.pairs;
            }
            r[i].pairs = pairs;
            r[i].status = rc;
            if (rc && !first_err) first_err = rc;
        }
        return first_err;
    }
    stats_begin(ctx);
    if (!ctx->engine || ctx->engine->per_thread() != ctx->per_thread) {
        if (ctx->engine) engine_free(ctx->engine);
        ctx->engine = new Engine(ctx, (int64_t)1 << 28, (int64_t)1 << 16, ctx->per_thread, 0);
        const int rc = ctx->engine->init();
        if (rc) {
            engine_free(ctx->engine);
            ctx->engine = nullptr;
            return rc;
        }
    }
    Engine& eng = *ctx->engine;
    const int64_t rounds0 = eng.rounds, pairs0 = eng.pairs, states0 = eng.states, live0 = eng.states_live;
    const double dev0 = eng.device_ms, pair0 = eng.pair_ms;
    eng.finished.clear();
    std::vector<std::unique_ptr<QueryRec>> recs(nq);
    // on a failure the engine may still point at this call's queries: drop it
    auto abandon = [&](int rc) {
        cudaStreamSynchronize(ctx->stream);
        engine_free(ctx->engine);
        ctx->engine = nullptr;
        return rc;
    };
    for (int64_t i = 0; i < nq; i++) {
        recs[i] = std::make_unique<QueryRec>();
        recs[i]->ticket = i;
        copy_query(q[i], recs[i].get());
        eng.plan(recs[i].get());
        bool ok = false;
        if (const int rc = eng.admit(recs[i].get(), true, &ok)) return abandon(rc);
    }
    while (!eng.idle()) {
        bool launched = false;
        if (eng.inflight() < 2 && eng.schedulable()) {
            if (const int rc = eng.launch_round()) return abandon(rc);
            launched = true;
        }
        if (eng.inflight() == 2 || (!launched && eng.inflight() > 0))
            if (const int rc = eng.complete_round()) return abandon(rc);
    }
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return abandon(fail(ctx, CSIM_ERR_CUDA, "stream failed after the last round"));
    for (int64_t i = 0; i < nq; i++) {
        r[i] = recs[i]->res;
        if (r[i].status && !first_err) first_err = r[i].status;
    }
    eng.finished.clear();
    (void)rounds0;
    ctx->stats.device_ms = eng.device_ms - dev0;
    ctx->stats.pair_kernel_ms = eng.pair_ms - pair0;
    ctx->stats.states = eng.states - states0;
    ctx->stats.states_live = eng.states_live - live0;
    ctx->stats.pairs = eng.pairs - pairs0;
    stats_end(ctx);
    return first_err;
}

void engine_free(Engine* engine) { delete engine; }

// ---------------------------------------------------------------- server
// Ownership and visibility: a query belongs to `tickets` from csim_submit to
// csim_release.  Clients see a result only once the worker has published it
// under the mutex (published = true); the engine's own `done` flag is the
// worker's business.
struct csim_server {
    csim_ctx* ctx = nullptr;
    std::unique_ptr<Engine> eng;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<QueryRec*> incoming;                        // submitted, not yet planned
    std::deque<QueryRec*> waiting;                         // planned, waiting for memory (worker only)
    std::map<int64_t, std::unique_ptr<QueryRec>> tickets;  // every unreleased query
    std::map<int64_t, bool> published;                     // ticket -> result visible to clients
    int64_t next_ticket = 1;
    int64_t submitted = 0, completed = 0, failed = 0;
    csim_server_stats snap{};  // engine counters as of the worker's last step
    bool stop = false;
    int worker_error = 0;
    std::thread worker;

    void run();
};

void csim_server::run() {
    cudaSetDevice(ctx->device);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        // admit new queries (planning runs outside the lock)
        std::deque<QueryRec*> fresh;
        fresh.swap(incoming);
        lk.unlock();
        for (QueryRec* r : fresh) {
            eng->plan(r);
            if (!r->done) waiting.push_back(r);
        }
        int rc = 0;
        while (!waiting.empty()) {  // first come first served while memory allows
            QueryRec* r = waiting.front();
            bool ok = false;
            const bool alone = eng->idle();  // nothing else holds memory: admit regardless
            rc = eng->admit(r, alone, &ok);
            if (rc || !ok) break;
            waiting.pop_front();
        }
        bool launched = false;
        if (!rc && eng->inflight() < 2 && eng->schedulable()) {
            rc = eng->launch_round();
            launched = true;
        }
        if (!rc && (eng->inflight() == 2 || (!launched && eng->inflight() > 0))) rc = eng->complete_round();
        lk.lock();
        snap.rounds = eng->rounds;
        snap.pairs = eng->pairs;
        snap.resident_bytes = eng->resident_bytes();
        snap.resident_decompositions = eng->resident_count();
        snap.queued = (int64_t)waiting.size();
        snap.device_ms = eng->device_ms;
        const auto now = Clock::now();
        for (QueryRec* r : eng->finished) {
            r->res.latency_s = std::chrono::duration<double>(now - r->t_submit).count();
            if (r->res.status) failed++;
            else completed++;
            published[r->ticket] = true;
        }
        if (!eng->finished.empty()) cv_done.notify_all();
        eng->finished.clear();
        if (rc) {
            worker_error = rc;
            stop = true;
        }
        if (stop) break;
        if (eng->idle() && incoming.empty() && waiting.empty())
            cv_work.wait(lk, [&] { return stop || !incoming.empty(); });
    }
    // fail what is left, once nothing is on the device
    lk.unlock();
    cudaStreamSynchronize(ctx->stream);
    lk.lock();
    for (auto& kv : tickets)
        if (!published[kv.first]) {
            kv.second->res.status = worker_error ? worker_error : CSIM_ERR_ARG;
            kv.second->done = true;
            kv.second->inflight = 0;
            published[kv.first] = true;
            failed++;
        }
    incoming.clear();
    cv_done.notify_all();
}

extern "C" int csim_server_create(const csim_server_config* cfg, csim_server** out) {
    if (!cfg || !out) return CSIM_ERR_ARG;
    *out = nullptr;
    csim_ctx* ctx = nullptr;
    int rc = csim_ctx_create(cfg->device, &ctx);
    if (rc) return rc;
    auto s = std::make_unique<csim_server>();
    s->ctx = ctx;
    s->eng = std::make_unique<Engine>(ctx, cfg->round_pairs, cfg->round_states, cfg->per_thread,
                                      cfg->hbm_budget_bytes);
    rc = s->eng->init();
    if (rc) {
        s->eng.reset();
        csim_ctx_destroy(ctx);
        return rc;
    }
    s->worker = std::thread([p = s.get()] { p->run(); });
    *out = s.release();
    return CSIM_OK;
}

extern "C" int csim_submit(csim_server* s, const csim_query* q, int64_t* ticket) {
    if (!s || !q || !ticket) return CSIM_ERR_ARG;
    auto r = std::make_unique<QueryRec>();
    copy_query(*q, r.get());
    r->t_submit = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return s->worker_error ? s->worker_error : CSIM_ERR_ARG;
    r->ticket = s->next_ticket++;
    *ticket = r->ticket;
    s->incoming.push_back(r.get());
    s->published[r->ticket] = false;
    s->tickets[r->ticket] = std::move(r);
    s->submitted++;
    s->cv_work.notify_one();
    return CSIM_OK;
}

extern "C" int csim_poll(csim_server* s, int64_t ticket, csim_query_result* out) {
    if (!s || !out) return CSIM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return CSIM_ERR_ARG;
    if (!s->published[ticket]) return CSIM_PENDING;
    *out = it->second->res;
    return CSIM_OK;
}

extern "C" int csim_wait(csim_server* s, int64_t ticket, double timeout_s, csim_query_result* out) {
    if (!s || !out) return CSIM_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->tickets.count(ticket)) return CSIM_ERR_ARG;
    auto ready = [&] { return s->published[ticket]; };
    if (timeout_s < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) return CSIM_PENDING;
    *out = s->tickets[ticket]->res;
    return CSIM_OK;
}

extern "C" int csim_release(csim_server* s, int64_t ticket) {
    if (!s) return CSIM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end() || !s->published[ticket]) return CSIM_ERR_ARG;
    if (it->second->inflight > 0) return CSIM_PENDING;  // a failed query's states are still being read back
    s->tickets.erase(it);
    s->published.erase(ticket);
    return CSIM_OK;
}

extern "C" int csim_server_get_stats(csim_server* s, csim_server_stats* out) {
    if (!s || !out) return CSIM_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->snap;
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->queued += (int64_t)s->incoming.size();
    return CSIM_OK;
}

extern "C" void csim_server_destroy(csim_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    s->eng.reset();
    csim_ctx_destroy(s->ctx);
    delete s;
}
