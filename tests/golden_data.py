"""Loader for the committed reference fixtures (tests/golden)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixtures():
    return np.load(os.path.join(GOLDEN, "reference_fixtures.npz"))


def meta():
    with open(os.path.join(GOLDEN, "reference_terms.json")) as f:
        d = json.load(f)
    d["terms"] = {k: [(complex(c[0], c[1]), [(nm, int(s)) for nm, s in ops]) for c, ops in v]
                  for k, v in d["terms"].items()}
    return d


def terms_heisenberg(n, J=1.0):
    return [(complex(J), [(op, i), (op, i + 1)]) for i in range(1, n) for op in ("Sx", "Sy", "Sz")]


def terms_tfim(n, J=1.0, h=1.0):
    t = [(complex(-J), [("Sz", i), ("Sz", i + 1)]) for i in range(1, n)]
    return t + [(complex(h), [("Sx", i)]) for i in range(1, n + 1)]


def terms_xxz(n, delta, fields=None):
    t = []
    for i in range(1, n):
        t.append((1.0 + 0j, [("Sx", i), ("Sx", i + 1)]))
        t.append((1.0 + 0j, [("Sy", i), ("Sy", i + 1)]))
        t.append((complex(delta), [("Sz", i), ("Sz", i + 1)]))
    if fields is not None:
        t += [(complex(h), [("Sz", i + 1)]) for i, h in enumerate(fields)]
    return t
