"""Packed stabilizer-state layout shared by the C ABI (include/csim.h), the
CUDA kernels and the tests.

One ``csim_state`` replaces ``struct StabilizerState``
(libcirc/stabilizer/stabilizer.h:5-16): each matrix row is one uint64 whose
bit c is column c; D[a] = 2*(2*bit_a(D2) + bit_a(D1)) (stabilizer.c:55-62).
"""
import numpy as np

MAX_QUBITS = 64

STATE_DTYPE = np.dtype(
    [
        ("n", "<i4"),
        ("k", "<i4"),
        ("Q", "<i4"),
        ("reserved0", "<i4"),
        ("h", "<u8"),
        ("D1", "<u8"),
        ("D2", "<u8"),
        ("reserved1", "<u8"),
        ("G", "<u8", (MAX_QUBITS,)),
        ("Gbar", "<u8", (MAX_QUBITS,)),
        ("J", "<u8", (MAX_QUBITS,)),
    ],
    align=True,
)
assert STATE_DTYPE.itemsize == 1584


def empty_states(count):
    """Zero-filled array of ``count`` packed states."""
    return np.zeros(int(count), dtype=STATE_DTYPE)


def bits_to_word(bits):
    """0/1 sequence -> uint64 word, element c -> bit c."""
    w = 0
    for c, b in enumerate(bits):
        if int(b) & 1:
            w |= 1 << c
    return np.uint64(w)


def word_to_bits(w, n):
    w = int(w)
    return [(w >> c) & 1 for c in range(n)]


def get_d(state, i):
    return 2 * (2 * ((int(state["D2"]) >> i) & 1) + ((int(state["D1"]) >> i) & 1))


def set_d(state, i, val):
    """setD of stabilizer.c:59-62 (C truncating division)."""
    v2 = int(val / 2)
    d1 = int(np.fmod(v2, 2)) & 1
    d2 = int(np.fmod(int((v2 - int(np.fmod(v2, 2))) / 2), 2)) & 1
    m = 1 << i
    state["D1"] = np.uint64((int(state["D1"]) & ~m) | (d1 << i))
    state["D2"] = np.uint64((int(state["D2"]) & ~m) | (d2 << i))


def block_view(state):
    """The part of a state the reference's results depend on: n, k, Q, h, G,
    Gbar in full, and D / J restricted to the first k rows and columns."""
    n, k = int(state["n"]), int(state["k"])
    km = (1 << k) - 1
    return (
        n,
        k,
        int(state["Q"]),
        int(state["h"]),
        tuple(int(x) for x in state["G"][:n]),
        tuple(int(x) for x in state["Gbar"][:n]),
        int(state["D1"]) & km,
        int(state["D2"]) & km,
        tuple(int(x) & km for x in state["J"][:k]),
    )


def projector_arrays(phases, xs, zs):
    """Protocol-encoded projector (phase v in Z4, x/z bit rows) as numpy arrays."""
    return (
        np.ascontiguousarray(np.asarray(phases, dtype=np.int32)),
        np.ascontiguousarray(np.asarray(xs, dtype=np.uint64)),
        np.ascontiguousarray(np.asarray(zs, dtype=np.uint64)),
    )
