"""FP64 state-vector simulation of compiled Clifford+T circuits: the exact
outcome probability the stabilizer-rank estimator approximates.  Test
infrastructure for n <= 20 qubits (2^20 complex amplitudes).

Circuits are in the compiled format the front end reads (one gate per line,
one symbol per qubit; libcirc/compile/gadgetize.py:65-181 gives the
semantics): H, S, X, T act on their qubit; a line with C and X is a CNOT
(control C, target X); a line holding M on qubit m applies its other gate
only when measured qubit m reads 1.  Measured qubits take no further gates,
so that classical control equals a quantum control on m (deferred
measurement), which is how it is simulated here.  The state starts in
|0...0>; amplitude index bit q is qubit q.

Also the statistical error the reference states for its estimators
(libcirc/innerprod.py:13-41): one sampled projector with L states has mean
||P|H^t>||^2 and standard deviation sqrt((2^t-1)/(2^t+1)) ||P|H^t>||^2/sqrt(L).
"""
import numpy as np

_H = np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2.0)
_S = np.array([[1, 0], [0, 1j]], dtype=np.complex128)
_X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
_T = np.array([[1, 0], [0, np.exp(1j * np.pi / 4)]], dtype=np.complex128)
_GATES = {"H": _H, "S": _S, "X": _X, "T": _T}


def _symbols(line):
    """Per-qubit symbols of a compiled line (a lower-case letter extends the
    symbol before it, as in compilecirc.standardGate)."""
    out = []
    for ch in line:
        if ch.islower():
            out[-1] = out[-1] + ch
        else:
            out.append(ch)
    return out


def _apply_1q(psi, n, q, U, ctrl=None):
    """U on qubit q, optionally only where qubit `ctrl` is 1."""
    v = psi.reshape(1 << (n - q - 1), 2, 1 << q)
    if ctrl is None:
        a0, a1 = v[:, 0, :].copy(), v[:, 1, :].copy()
        v[:, 0, :] = U[0, 0] * a0 + U[0, 1] * a1
        v[:, 1, :] = U[1, 0] * a0 + U[1, 1] * a1
        return psi
    idx = np.arange(1 << n)
    sel = ((idx >> ctrl) & 1) == 1
    lo = idx[sel & (((idx >> q) & 1) == 0)]
    hi = lo | (1 << q)
    a0, a1 = psi[lo].copy(), psi[hi].copy()
    psi[lo] = U[0, 0] * a0 + U[0, 1] * a1
    psi[hi] = U[1, 0] * a0 + U[1, 1] * a1
    return psi


def _apply_cnot(psi, n, c, t, ctrl=None):
    idx = np.arange(1 << n)
    sel = (((idx >> c) & 1) == 1) & (((idx >> t) & 1) == 0)
    if ctrl is not None:
        sel &= ((idx >> ctrl) & 1) == 1
    lo = idx[sel]
    hi = lo | (1 << t)
    psi[lo], psi[hi] = psi[hi].copy(), psi[lo].copy()
    return psi


def run(circ):
    """Final state of a compiled circuit (text) as (psi, n)."""
    lines = [ln for ln in circ.splitlines() if ln.strip() and ln.strip() != "main:"]
    n = len(_symbols(lines[0]))
    if n > 20:
        raise ValueError("state vector limited to 20 qubits")
    psi = np.zeros(1 << n, dtype=np.complex128)
    psi[0] = 1.0
    for ln in lines:
        sym = _symbols(ln)
        if len(sym) != n:
            raise ValueError("ragged circuit line: %r" % ln)
        ctrl = sym.index("M") if "M" in sym else None
        ops = [(q, s) for q, s in enumerate(sym) if s not in ("_", "M")]
        if not ops:
            continue
        names = sorted(s for _, s in ops)
        if names == ["C", "X"]:
            c = [q for q, s in ops if s == "C"][0]
            t = [q for q, s in ops if s == "X"][0]
            _apply_cnot(psi, n, c, t, ctrl)
        elif len(ops) == 1 and ops[0][1] in _GATES:
            _apply_1q(psi, n, ops[0][0], _GATES[ops[0][1]], ctrl)
        else:
            raise ValueError("gate outside H, S, X, T, CNOT: %r" % ln)
    return psi, n


def probability(circ, measure):
    """Exact probability that qubits measure.keys() read measure.values()."""
    psi, n = run(circ)
    idx = np.arange(1 << n)
    sel = np.ones(1 << n, dtype=bool)
    for q, b in measure.items():
        sel &= ((idx >> int(q)) & 1) == int(b)
    return float(np.sum(np.abs(psi[sel]) ** 2))


def ht_stack(nt):
    """<0| H (T H)^nt |0>-squared, the reference's HT-stack value (main.py:177-190)."""
    out = _H.copy()
    for _ in range(nt):
        out = out @ _T @ _H
    return float(abs(out[0, 0]) ** 2)


def sampled_sigma_rel(t, L):
    """Relative standard deviation of one sampled projector with L states
    (libcirc/innerprod.py:35-41): sqrt((2^t - 1)/(2^t + 1)) / sqrt(L)."""
    return float(np.sqrt((2.0 ** t - 1) / (2.0 ** t + 1)) / np.sqrt(L))


def ratio_bound(t, L, failprob):
    """Relative error bound of numerator/denominator, each estimated from L
    states, that holds with probability >= 1 - failprob by Chebyshev's bound
    applied to each (failprob/2 each): |r - r0| <= r0 (e_n + e_d) / (1 - e_d)
    with e = sigma_rel / sqrt(failprob/2)."""
    e = sampled_sigma_rel(t, L) / np.sqrt(failprob / 2)
    if e >= 1:
        return float("inf")
    return float(2 * e / (1 - e))
