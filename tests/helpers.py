"""Shared test helpers (comparison views, random inputs)."""
import numpy as np


def full_view(s):
    s = s.reshape(-1)[0] if getattr(s, "shape", ()) else s
    n = int(s["n"])
    return (n, int(s["k"]), int(s["Q"]), int(s["h"]), int(s["D1"]), int(s["D2"]),
            tuple(int(x) for x in s["G"][:n]), tuple(int(x) for x in s["Gbar"][:n]),
            tuple(int(x) for x in s["J"][:n]))


def rand_word(rs, n):
    w = 0
    for c in range(n):
        if rs.randint(2):
            w |= 1 << c
    return w


def random_projector_rows(rs, t, nstabs):
    return (rs.randint(0, 4, size=nstabs).tolist(), [rand_word(rs, t) for _ in range(nstabs)],
            [rand_word(rs, t) for _ in range(nstabs)])


def phase_m(v):
    return 2 * ((v // 2) % 2) + (v % 2)


def z_value(eps, p, m):
    """eps 2^{p/2} e^{i pi m/4} as a complex (double)."""
    if not eps:
        return 0j
    return (2.0 ** (p / 2.0)) * np.exp(1j * np.pi * (m % 8) / 4.0)


def close(a, b, rel=1e-12, floor=1e-12):
    return abs(a - b) <= rel * max(abs(a), abs(b)) + floor
