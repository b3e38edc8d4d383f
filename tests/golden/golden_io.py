"""Read/write helpers for the golden vectors under tests/golden/.

States are stored as JSON objects with hex words: {"n", "k", "Q", "h", "D1",
"D2", "G": [...n], "Gbar": [...n], "J": [...n]}; a word's bit c is column c
(the packed layout of include/csim.h).
"""
import gzip
import json
import os

import numpy as np

from circuitsimulator_gb300.state import STATE_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))


def state_to_json(s):
    s = s.reshape(-1)[0] if hasattr(s, "reshape") and s.shape else s
    n = int(s["n"])
    return {
        "n": n,
        "k": int(s["k"]),
        "Q": int(s["Q"]),
        "h": "%x" % int(s["h"]),
        "D1": "%x" % int(s["D1"]),
        "D2": "%x" % int(s["D2"]),
        "G": ["%x" % int(x) for x in s["G"][:n]],
        "Gbar": ["%x" % int(x) for x in s["Gbar"][:n]],
        "J": ["%x" % int(x) for x in s["J"][:n]],
    }


def state_from_json(d):
    s = np.zeros(1, dtype=STATE_DTYPE)
    n = int(d["n"])
    s["n"] = n
    s["k"] = int(d["k"])
    s["Q"] = int(d["Q"])
    for f in ("h", "D1", "D2"):
        s[f] = np.uint64(int(d[f], 16))
    for f in ("G", "Gbar", "J"):
        s[f][0, :n] = np.array([int(x, 16) for x in d[f]], dtype=np.uint64)
    return s


def states_from_json(lst):
    out = np.zeros(len(lst), dtype=STATE_DTYPE)
    for i, d in enumerate(lst):
        out[i] = state_from_json(d)[0]
    return out


def save(name, obj):
    path = os.path.join(HERE, name)
    with gzip.open(path, "wt", compresslevel=9) as f:
        json.dump(obj, f, separators=(",", ":"))
    return path


def load(name):
    with gzip.open(os.path.join(HERE, name), "rt") as f:
        return json.load(f)
