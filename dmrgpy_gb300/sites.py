"""Local Hilbert spaces and their named operators.

Type codes and operator names follow dmrgpy's site sets
(``pyitensor/sites/siteset.py:20-40``): 2 = S=1/2, 3 = S=1, 4/5/6 = S=3/2,
2, 5/2, 0 = spinless fermion, 1 = electron (Emp, Up, Dn, UpDn), 100+d =
boson with d levels.  Matrices are returned in textbook (out, in) form;
the MPO compiler transposes them into the (in, out) storage of the MPO
tensors (``pyitensor/sites/base.py:1-17``).  Values are built from the
definitions (spin ladder algebra, fermionic creation operators with the
in-site sign convention of ``pyitensor/sites/fermion.py:39-75``), not from
tables.
"""
import functools

import numpy as np


def _spin_ops(two_s):
    s = two_s / 2.0
    d = two_s + 1
    m = s - np.arange(d)                       # |Up> = m = +S first
    sp = np.zeros((d, d))
    sp[np.arange(d - 1), np.arange(1, d)] = np.sqrt(s * (s + 1) - m[1:] * (m[1:] + 1))
    sm = sp.T.copy()
    sz = np.diag(m)
    sx = (sp + sm) / 2.0
    sy = (sp - sm) / 2j
    ops = {"Sz": sz, "Sx": sx, "Sy": sy, "ISy": 1j * sy, "Sp": sp, "S+": sp, "Sm": sm, "S-": sm,
           "Sz2": sz @ sz, "Sx2": sx @ sx, "Sy2": (sy @ sy).real, "S2": s * (s + 1) * np.eye(d)}
    labels = {2: ("Up", "Dn"), 3: ("Up", "Z0", "Dn"), 5: ("Up", "Upi", "Z0", "Dni", "Dn")}.get(d, ())
    for k, lab in enumerate(labels):
        ops["proj" + lab] = np.diag(np.eye(d)[k])
    return ops


def _fermion_modes(modes):
    """Occupation basis with the first mode most significant; c_j carries the
    sign (-1)^(occupied modes before j)."""
    nm = len(modes)
    states = [(0, 0), (1, 0), (0, 1), (1, 1)] if nm == 2 else [(0,), (1,)]
    index = {st: k for k, st in enumerate(states)}
    d = len(states)
    ops = {}
    for j, mode in enumerate(modes):
        c = np.zeros((d, d))
        a = np.zeros((d, d))
        for st in states:
            if st[j]:
                dst = list(st)
                dst[j] = 0
                c[index[tuple(dst)], index[st]] = (-1) ** sum(st[:j])
                a[index[tuple(dst)], index[st]] = 1.0
        ops["C" + mode] = c
        ops["Cdag" + mode] = c.T.copy()
        ops["A" + mode] = a
        ops["Adag" + mode] = a.T.copy()
        ops["N" + mode] = np.diag([float(st[j]) for st in states])
        ops["F" + mode] = np.diag([(-1.0) ** st[j] for st in states])
    ops["F"] = np.diag([(-1.0) ** sum(st) for st in states])
    ops["FermiPhase"] = ops["F"]
    return ops


def _spinless_ops():
    f = _fermion_modes([""])
    ops = {k: f[k] for k in ("C", "Cdag", "A", "Adag", "F", "FermiPhase")}
    ops["N"] = f["N"]
    ops["n"] = f["N"]
    ops["projEmp"] = np.diag([1.0, 0.0])
    ops["projOcc"] = np.diag([0.0, 1.0])
    return ops


def _electron_ops():
    f = _fermion_modes(["up", "dn"])
    ops = {k: f[k] for k in ("Cup", "Cdagup", "Cdn", "Cdagdn", "Aup", "Adagup", "Adn", "Adagdn",
                             "F", "FermiPhase", "Fup", "Fdn", "Nup", "Ndn")}
    ops["Nupdn"] = f["Nup"] @ f["Ndn"]
    ops["Ntot"] = f["Nup"] + f["Ndn"]
    sp = f["Cdagup"] @ f["Cdn"]
    ops["Sz"] = 0.5 * (f["Nup"] - f["Ndn"])
    ops["Sp"] = ops["S+"] = sp
    ops["Sm"] = ops["S-"] = sp.T.copy()
    ops["S2"] = 0.75 * (f["Nup"] + f["Ndn"] - 2.0 * ops["Nupdn"])
    return ops


def _boson_ops(d):
    a = np.diag(np.sqrt(np.arange(1, d, dtype=float)), 1)
    ops = {"A": a, "Adag": a.T.copy(), "N": np.diag(np.arange(d, dtype=float))}
    for k in range(d):
        ops["N%d" % k] = np.diag(np.eye(d)[k])
    return ops


@functools.lru_cache(maxsize=None)
def _ops(code):
    if code == 2:
        ops = _spin_ops(1)
    elif code == 3:
        ops = _spin_ops(2)
    elif code in (4, 5, 6):
        ops = _spin_ops(code - 1)
    elif code == 0:
        ops = _spinless_ops()
    elif code == 1:
        ops = _electron_ops()
    elif 100 < code < 200:
        ops = _boson_ops(code - 100)
    else:
        raise ValueError("site type code {} is not supported by the GB300 backend".format(code))
    return {k: np.asarray(v, dtype=complex) for k, v in ops.items()}


def dim(code):
    return next(iter(_ops(code).values())).shape[0]


def op(code, name):
    """Textbook (out, in) matrix of operator `name` on a site of type `code`.
    'Id' is the identity; 'F'/'FermiPhase' default to the identity on sites
    without fermions (``pyitensor/sites/base.py:42-57``)."""
    ops = _ops(code)
    if name == "Id":
        return np.eye(dim(code), dtype=complex)
    if name in ops:
        return ops[name]
    if name in ("F", "FermiPhase"):
        return np.eye(dim(code), dtype=complex)
    raise ValueError("Operator '{}' not recognized for site type {}".format(name, code))


def is_fermionic(name):
    """Name-based rule of ``pyitensor/sites/base.py:59-75``: names starting
    with 'C' anticommute across sites."""
    return bool(name) and name[0] == "C"
