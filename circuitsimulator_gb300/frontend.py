"""Front end of a probability query: compiled circuit -> projectors G', H'.

Restates, in this package's own code, what the reference's Python front end
does before it starts a backend process:

    countY       libcirc/compile/gadgetize.py:12-59
    gadgetize    libcirc/compile/gadgetize.py:65-181
    projectors   libcirc/compile/projectors.py:17-83
    truncate     libcirc/compile/projectors.py:87-162

It reads compiled circuits, the output of the reference's compileCircuit:
one gate per line, one symbol per qubit, from H S X T C M _.  The outputs
equal the reference's for the same inputs and the same numpy random state.
The same randint calls are made in the same order.

Pauli generators are stored bit-sliced.  For every qubit, one Python integer
holds that qubit's X bit of every generator, and another holds its Z bit.  Two
more integers hold the phase in Z4, one bit plane each.  Conjugating all
generators by a gate is then a handful of integer operations, whatever their
number.  The phase rules are those of the reference's lookup tables, written
as bit-plane updates:
    H: X <-> Z, phase += 2 where X & Z
    X: phase += 2 where Z
    S: phase += 1 where X, Z ^= X
    CNOT(c, t): Z_c ^= Z_t, X_t ^= X_c
"""
import numpy as np


# ---------------------------------------------------------------- circuits
def standard_gate(line, list_mode=False, line_mode=False):
    """compilecirc.standardGate (libcirc/compile/compilecirc.py:239-257): a
    circuit line as a list of symbols (line_mode), or its sorted symbols
    without '_' and 'M' (a list with list_mode, else a string).  A lower-case
    letter extends the symbol before it."""
    if line == "main":
        if list_mode or line_mode:
            raise ValueError("Can't bring 'main' into list form.")
        return "main"
    if not line_mode:
        line = line.replace("_", "").replace("M", "")
    elems = []
    for ch in line:
        if ch.islower():
            elems[-1] = elems[-1] + ch
        else:
            elems.append(ch)
    if line_mode:
        return elems
    if list_mode:
        return sorted(elems)
    return "".join(sorted(elems))


def count_y(circuit):
    """(T gates, circuit-measured qubits, qubits whose measurement gates a T)
    with the reference's syntax checks (gadgetize.py:12-59)."""
    n_t = 0
    t_cache = []
    measured = []
    m_ts = []
    for line_nr, line in enumerate(circuit.splitlines(), 1):
        gate = standard_gate(line, line_mode=True)
        if "M" in gate:
            m = gate.index("M")
            if m not in measured:
                measured.append(m)
        for m in measured:
            if gate[m] not in ("M", "_"):
                raise SyntaxError("Line %d: Cannot perform operations to measured qubit %d" % (line_nr, m))
        if "T" in gate and "M" not in gate:
            n_t += 1
            q = gate.index("T")
            if q in t_cache:
                # the reference reports the last measured-qubit loop variable here
                raise SyntaxError("Line %d: Consecutive Ts on qubit %d" % (line_nr, m))
            t_cache.append(q)
        # a gate on a cached qubit ends its run of Ts (the reference edits the
        # list while iterating over it, which skips the element after a removal)
        i = 0
        while i < len(t_cache):
            if gate[t_cache[i]] != "_":
                del t_cache[i]
                i += 1
            else:
                i += 1
        if "T" in gate and "M" in gate:
            m_ts.append(gate.index("M"))
    return n_t, measured, m_ts


class Generators:
    """Bit-sliced Pauli generators on `size` qubits (see the module docstring)."""

    def __init__(self, size):
        self.size = size
        self.count = 0
        self.x = [0] * size
        self.z = [0] * size
        self.p0 = 0
        self.p1 = 0

    def add_z(self, q, negative):
        """Appends the generator (-1)^negative Z_q (gadgetize.py:73-84)."""
        g = 1 << self.count
        self.count += 1
        self.z[q] |= g
        if negative:
            self.p1 |= g

    def _add_phase(self, m, amount):
        if amount & 1:
            carry = self.p0 & m
            self.p0 ^= m
            self.p1 ^= carry
        if amount & 2:
            self.p1 ^= m

    def h(self, q):
        self._add_phase(self.x[q] & self.z[q], 2)
        self.x[q], self.z[q] = self.z[q], self.x[q]

    def xgate(self, q):
        self._add_phase(self.z[q], 2)

    def s(self, q):
        self._add_phase(self.x[q], 1)
        self.z[q] ^= self.x[q]

    def cnot(self, c, t):
        self.z[c] ^= self.z[t]
        self.x[t] ^= self.x[c]

    def rows(self):
        """(phases, x masks, z masks), one entry per generator; bit i of a mask is qubit i."""
        phases, xs, zs = [], [], []
        for g in range(self.count):
            b = 1 << g
            phases.append((1 if self.p0 & b else 0) + (2 if self.p1 & b else 0))
            xm = zm = 0
            for q in range(self.size):
                if self.x[q] & b:
                    xm |= 1 << q
                if self.z[q] & b:
                    zm |= 1 << q
            xs.append(xm)
            zs.append(zm)
        return phases, xs, zs


def gadgetize(circuit, mdict, y):
    """The projector of the gadgetized circuit (gadgetize.py:65-181): generators
    Z_M for measured qubits (sign from mdict) and Z for each T ancilla (sign
    from y), conjugated by the circuit from its last line to its first.
    Returns (phases, x masks, z masks, size)."""
    n = len(standard_gate(circuit.split("\n", 1)[0], line_mode=True))
    size = n + len(y)
    gens = Generators(size)
    for m in mdict.keys():
        gens.add_z(m, mdict[m] == 1)
    for i in range(n, size):
        gens.add_z(i, y[i - n] == 1)
    tpos = n
    for line in reversed(circuit.splitlines()):
        if line == "":
            continue
        gate = standard_gate(line, line_mode=True)
        if "M" in gate and mdict[gate.index("M")] == 0:
            continue
        std = standard_gate(line)
        idxs = [gate.index(letter) for letter in std]
        if std == "T":
            q = idxs[0]
            gens.cnot(q, tpos)
            if y[tpos - n] == 1:
                gens.s(q)
            gens.h(tpos)
            for _ in range(3):
                gens.s(tpos)
            tpos += 1
        elif len(std) == 1:
            {"H": gens.h, "X": gens.xgate, "S": gens.s}[std](idxs[0])
        else:
            gens.cnot(idxs[0], idxs[1])
    phases, xs, zs = gens.rows()
    return phases, xs, zs, size


def _parse_bits(s, length, name):
    if len(s) != length:
        raise ValueError("%s needs to have length %d" % (name, length))
    out = []
    for ch in s:
        if ch not in "01":
            raise ValueError("Only 0s and 1s allowed in %s string." % name)
        out.append(int(ch))
    return np.array(out).astype(int)


def projectors(circ, measure, rng=np.random, x=None, y=None):
    """G and H of a measurement (projectors.py:17-83).  Draws the circuit's
    measurement outcomes and the T-ancilla outcomes from `rng` in the
    reference's order, and adds the circuit's measured qubits to `measure`
    (which the caller keeps, as in the reference).  Returns (G, H, n, t), with
    G and H as (phases, x masks, z masks, size)."""
    n = len(standard_gate(circ.splitlines()[0], line_mode=True))
    t, measured, m_ts = count_y(circ)
    msel = rng.randint(2, size=len(measured)) if x is None else _parse_bits(x, len(measured), "x")
    for m in m_ts:
        if msel[measured.index(m)] == 1:
            t += 1
    mdict = {}
    for m in measured:
        v = msel[measured.index(m)]
        mdict[m] = v
        if m in measure.keys():
            continue
        measure[m] = v
    y = rng.randint(2, size=t) if y is None else _parse_bits(y, t, "y")
    G = gadgetize(circ, measure, y)
    H = gadgetize(circ, mdict, y)
    return G, H, n, t


def _parity(v):
    return bin(v).count("1") & 1


def truncate(n, P):
    """Restricts a projector to the magic-state qubits by projecting its first n
    qubits onto |0^n> (projectors.py:87-162).  Returns ((phases, x masks,
    z masks) on the remaining qubits, u), u = generators lost."""
    phases, xs, zs, size = P
    if len(phases) == 0:
        return ([], [], []), 0
    ngen = len(phases)
    # null space of the generators' X parts on the first n qubits, built by the
    # reference's column sweep: rows with a 0 in the column are kept, rows
    # with a 1 are replaced by the sums of cyclically adjacent pairs, minus one
    X = [1 << i for i in range(ngen)]
    for q in range(n):
        col = 0
        for g in range(ngen):
            if (xs[g] >> q) & 1:
                col |= 1 << g
        good, bad = [], []
        for r in X:
            (bad if _parity(r & col) else good).append(r)
        X = good + [bad[i] ^ bad[i - 1] for i in range(1, len(bad))]
    low = (1 << n) - 1
    out_ph, out_x, out_z = [], [], []
    for row in X:
        ph, gx, gz = 0, 0, 0
        for g in range(ngen):
            if (row >> g) & 1:
                # product of Pauli generators: a Z before an X contributes -1
                ph = (ph + phases[g] + 2 * bin(gz & xs[g]).count("1")) % 4
                gx ^= xs[g]
                gz ^= zs[g]
        if gx & low:
            raise ValueError("Null space wrong.")
        tx, tz = gx >> n, gz >> n
        if ph == 0 and tx == 0 and tz == 0:
            continue  # the positive identity
        out_ph.append(ph)
        out_x.append(tx)
        out_z.append(tz)
    return (out_ph, out_x, out_z), ngen - len(X)
