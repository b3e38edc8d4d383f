"""Seeded random Clifford+T circuits in the compiled-circuit format of the
reference's front end: one gate per line, one symbol per qubit (H, S, X, T,
C/X for a CNOT, '_' elsewhere), after a "main:" header.  Shared by the
workload generator (make_workloads.py) and the state-vector tests.

Gate mix per drawn gate: H/S/X/Z with probability 0.55 (Z written as H X H),
CNOT on a random ordered pair 0.30, T or T^dagger 0.15 (T^dagger written as
S S S T); drawing stops once `t_target` T gates (T and T^dagger together) are
placed.
"""


def gate_line(n, ops):
    """One circuit line: ops = {qubit: symbol}, '_' elsewhere."""
    return "".join(ops.get(q, "_") for q in range(n))


def random_circuit(n, t_target, rs):
    """(circuit text with its "main:" header, number of drawn gates); rs is a
    numpy RandomState."""
    lines = ["main:"]
    t = 0
    gates = 0
    while t < t_target:
        r = rs.random_sample()
        if r < 0.55:
            g = ["H", "S", "X", "Z"][rs.randint(4)]
            q = rs.randint(n)
            if g == "Z":  # Z = H X H
                lines += [gate_line(n, {q: "H"}), gate_line(n, {q: "X"}), gate_line(n, {q: "H"})]
            else:
                lines.append(gate_line(n, {q: g}))
        elif r < 0.85:
            a, b = rs.choice(n, size=2, replace=False)
            lines.append(gate_line(n, {int(a): "C", int(b): "X"}))
        else:
            q = rs.randint(n)
            if rs.randint(2):
                lines.append(gate_line(n, {q: "T"}))
            else:  # T^dagger = S S S T
                lines += [gate_line(n, {q: "S"})] * 3 + [gate_line(n, {q: "T"})]
            t += 1
        gates += 1
    return "\n".join(lines) + "\n", gates


def compiled(circ):
    """The compiled circuit: the gate lines without the "main:" header (what
    the reference's compileCircuit returns for these base-gate circuits)."""
    return "\n".join(ln for ln in circ.splitlines() if ln and ln != "main:") + "\n"
