"""probability() and sampleQubits() with the backend in this process, plus a
batched sampleQubits that runs many shots' chains in lockstep on the GPU.

    probability    libcirc/probability.py:66-326
    sampleQubits   libcirc/sample.py:16-86

The control flow is the reference's: the same early answers (negative
identity, identical projectors, t = 0), the same config defaults and
auto-picked samples, the same config mutations that a caller sees
afterwards, and the same numpy draws in the same order (front end in
circuitsimulator_gb300.frontend).  The difference is the backend.  Instead of
writing the stdin protocol to a new process, each query goes to the GPU
through csim_run_queries.  So with a fixed backend seed these functions give
what the reference gives with the same seed in its backend process.

Each query's backend seed comes from config["seed"] when set (an int used
for every query, as a fixed process id would be), otherwise from os.urandom
(the reference seeds each backend process with its process id).

A probability computation is written once, as a generator that yields its
backend query and receives (numerator, denominator).  probability() and
sampleQubits() answer each query as it comes.  sample_qubits_batch() collects
one query from every shot and answers them all with one batched call.  So a
shot gives the same bits alone and in a batch.
"""
import os

import numpy as np

from . import backend as _backend
from . import frontend

_default_backend = None
_ERROR0 = 0.2       # probability.py's default relative error
_FAILPROB0 = 0.05   # and failure probability


def default_backend():
    """A Backend on device 0, opened on first use (fails loudly without a GPU)."""
    global _default_backend
    if _default_backend is None:
        _default_backend = _backend.Backend(0)
    return _default_backend


def _seed_for(config):
    s = config.get("seed")
    if s is None:
        return int.from_bytes(os.urandom(4), "little") & 0x7FFFFFFF
    return int(s)


def _bool(v):
    return 1 if v else 0


def probability_steps(circ, measure, config, rng):
    """probability() as a generator: yields one backend query (a dict for
    Backend.run_queries) at most, receives (numerator, denominator), returns
    the probability (libcirc/probability.py:66-326)."""
    verbose = config.get("verbose")
    if verbose:
        config["quiet"] = False
    quiet = config.get("quiet")
    if config.get("exact") is None:
        config["exact"] = True
    if config.get("fidbound") is None:
        config["fidbound"] = 1e-5
    # with k given, fidelity only prints; quiet turns it off (probability.py:83-87)
    if not config.get("exact") and config.get("k") is not None:
        if config.get("quiet") and config.get("fidelity"):
            config["fidelity"] = False

    G, H, n, t = frontend.projectors(circ, measure, rng=rng, x=config.get("x"), y=config.get("y"))
    Gp, u = frontend.truncate(n, G)
    Hp, v = frontend.truncate(n, H)

    # -I in the numerator (probability.py:110-116)
    for i in range(len(Gp[0])):
        if Gp[0][i] == 2 and Gp[1][i] == 0 and Gp[2][i] == 0:
            return 0
    # identical projectors (probability.py:118-128); a G' shorter than H' with
    # an equal prefix counts as identical, as there
    same = True
    for i in range(len(Gp[0])):
        if i > len(Hp[0]) - 1:
            same = False
        same = same and Gp[0][i] == Hp[0][i] and Gp[1][i] == Hp[1][i] and Gp[2][i] == Hp[2][i]
    if same:
        return 2 ** (v - u)
    if len(Gp[0]) == 0 or len(Hp[0]) == 0 and not config["exact"]:
        config["exact"] = True
    if t == 0:
        return None  # the reference's Python backend, which returns None (probability.py:135-181)

    # samples and bins (probability.py:150-175).  The reference compares error
    # and failprob with its default constants by identity, so a value that is
    # not the very object it inserted itself, even an equal one, switches on the
    # auto-pick; the same test against this module's default objects follows it
    if not config.get("noapprox"):
        if not config.get("samples"):
            config["samples"] = 2000
        if not config.get("bins"):
            config["bins"] = 1
        if not config.get("error"):
            config["error"] = _ERROR0
        if not config.get("failprob"):
            config["failprob"] = _FAILPROB0
        if config.get("error") is not _ERROR0 or config.get("failprob") is not _FAILPROB0:
            chi = (2 ** t - 1) / (2 ** t + 1)
            if config.get("failprob") < 0.0076:
                config["samples"] = int(np.ceil(6 * chi * config.get("error") ** (-2)))
                config["bins"] = int(np.ceil(4.5 * np.log(1 / config.get("failprob"))))
            else:
                config["samples"] = int(np.ceil(chi * config.get("error") ** (-2) * config.get("failprob") ** (-1)))
                config["bins"] = 1

    # the 13 scalars of the backend protocol (probability.py:249-268); t is the
    # width of G''s first row, so an empty G' fails here as there
    width = G[3] - n
    if len(Gp[1]) == 0:
        raise IndexError("list index out of range")
    cfg = {"quiet": _bool(config.get("quiet")), "verbose": _bool(config.get("verbose")),
           "noapprox": _bool(config.get("noapprox")), "samples": int(config.get("samples") or 0),
           "bins": int(config.get("bins") or 0), "t": width, "k": int(config.get("k") or 0),
           "exact": _bool(config.get("exact")),
           "fidbound": float(config.get("fidbound") if config.get("fidbound") else 1e-5),
           "fidelity": _bool(config.get("fidelity")), "rank": _bool(config.get("rank")),
           "forceL": _bool(config.get("forceL")), "forceSample": _bool(config.get("forceSample"))}
    projs = [(list(Gp[0]), list(Gp[1]), list(Gp[2]), width),
             (list(Hp[0]), list(Hp[1]), list(Hp[2]), width if len(Hp[0]) else 0)]
    numerator, denominator = yield {"cfg": cfg, "projs": projs, "seed": _seed_for(config),
                                    "rng": _backend.RNG_LIBC}
    if config.get("direct"):
        return (2 ** (v - u) * numerator, denominator)
    if numerator == 0:
        return 0
    return 2 ** (v - u) * (numerator / denominator)


def _answer(be, query):
    r = be.run_queries([query], batched=True)[0]
    return r["numerator"], r["denominator"]


def _drive(gen, be):
    """Runs a step generator to its end, answering each query on `be`."""
    try:
        q = next(gen)
        while True:
            q = gen.send(_answer(be, q))
    except StopIteration as e:
        return e.value


def probability(circ, measure, config=None, rng=None, backend=None):
    """probability(circ, measure, config) of libcirc/probability.py:66, with the
    backend on the GPU.  rng: the numpy random state of the front end (the
    global one by default, as in the reference)."""
    config = {} if config is None else config
    return _drive(probability_steps(circ, measure, config, rng if rng is not None else np.random),
                  backend or default_backend())


def sample_steps(circ, measure, sample, config, rng):
    """sampleQubits as a generator of backend queries (libcirc/sample.py:16-86)."""
    verbose = config.get("verbose")
    if config.get("exact") is None:
        config["exact"] = False
    config["file"] = None

    def prob(measure, exact=None):
        if exact is not None:
            old = config["exact"]
            config["exact"] = exact
        P = yield from probability_steps(circ, measure, config, rng)
        if exact is not None:
            config["exact"] = old
        return P

    def recursive(qubits, measure):
        if len(qubits) == 1:
            Psofar = 1
            if len(measure.keys()) != 0:
                Psofar = yield from prob(measure, exact=True)
                if verbose:
                    print("Constraints present. Probability of satifying: %f\n" % Psofar)
                if Psofar == 0:
                    return "", {}, 0
                if Psofar < 1e-5:
                    print("Warning: probability of satisfying qubit constraints very low (%f). Could be impossible."
                          % Psofar)
            measure[qubits[0]] = 0
            P = yield from prob(measure)
            P0 = P / Psofar
            qubit = 0 if rng.random() < P0 else 1
            measure[qubits[0]] = qubit
            return str(qubit), measure, (P0 if qubit == 0 else (1 - P0))
        sofar, measure, Psofar = yield from recursive(qubits[:-1], measure)
        if sofar == "":
            return "", {}, 0
        measure[qubits[-1]] = 0
        P = yield from prob(measure)
        P0 = P / Psofar
        qubit = 0 if rng.random() < P0 else 1
        measure[qubits[-1]] = qubit
        return sofar + str(qubit), measure, (P0 if qubit == 0 else (1 - P0))

    output, _, _ = yield from recursive(sample, measure)
    return output


def sampleQubits(circ, measure, sample, config=None, rng=None, backend=None):
    """sampleQubits(circ, measure, sample, config) of libcirc/sample.py:16, with
    the backend on the GPU."""
    config = {} if config is None else config
    return _drive(sample_steps(circ, measure, sample, config, rng if rng is not None else np.random),
                  backend or default_backend())


def sample_qubits_batch(circ, measure, sample, config, seeds, backend=None, stats=None, groups=2):
    """Many independent sampleQubits shots in lockstep.  Shot s has its own
    numpy RandomState(seeds[s]) for the front end and the bit draws, and its
    own copies of `measure` and `config`.  The shots are split into `groups`
    interleaved groups; each group's pending queries go to the GPU in one
    csim_run_queries call, made on a worker thread, while this thread runs
    the other groups' front ends (the call releases the GIL).  Shot s returns
    the same bits as sampleQubits run alone with that random state, whatever
    the grouping.  Returns the list of output strings; `stats`, when a dict,
    gets the number of calls, the queries per call, and the seconds spent in
    the calls (`gpu_s`; of it `device_s` on the GPU, `pair_kernel_s` in the
    pair kernels) and in the front ends between them (`host_s`)."""
    import time
    from concurrent.futures import ThreadPoolExecutor

    be = backend or default_backend()
    gens, pending, out = [], [], [None] * len(seeds)
    t0 = time.perf_counter()
    for s, seed in enumerate(seeds):
        g = sample_steps(circ, dict(measure), sample, dict(config), np.random.RandomState(seed))
        gens.append(g)
        try:
            pending.append(next(g))
        except StopIteration as e:
            out[s] = e.value
            pending.append(None)
    host_s = time.perf_counter() - t0
    groups = max(1, min(groups, len(seeds)))
    members = [list(range(g, len(seeds), groups)) for g in range(groups)]
    steps, per_step, gpu_s = 0, [], [0.0, 0.0, 0.0]

    def answer(qs):
        t = time.perf_counter()
        r = be.run_queries(qs, batched=True)
        gpu_s[0] += time.perf_counter() - t
        st = be.last_stats()  # this call's device time and pair-kernel time
        gpu_s[1] += st.device_ms / 1e3
        gpu_s[2] += st.pair_kernel_ms / 1e3
        return r

    with ThreadPoolExecutor(max_workers=1) as worker:
        def submit(g):
            live = [s for s in members[g] if pending[s] is not None]
            return (live, worker.submit(answer, [pending[s] for s in live])) if live else None

        inflight = [submit(g) for g in range(groups)]  # the worker runs them in this order
        while any(f is not None for f in inflight):
            for g in range(groups):
                if inflight[g] is None:
                    continue
                live, fut = inflight[g]
                res = fut.result()
                steps += 1
                per_step.append(len(live))
                t = time.perf_counter()
                for s, r in zip(live, res):
                    try:
                        pending[s] = gens[s].send((r["numerator"], r["denominator"]))
                    except StopIteration as e:
                        out[s] = e.value
                        pending[s] = None
                host_s += time.perf_counter() - t
                inflight[g] = submit(g)
    if isinstance(stats, dict):
        stats["steps"] = steps
        stats["queries_per_step"] = per_step
        stats["gpu_s"] = gpu_s[0]
        stats["device_s"] = gpu_s[1]
        stats["pair_kernel_s"] = gpu_s[2]
        stats["host_s"] = host_s
    return out
