"""Term list -> MPO, built as a finite-state machine with shared prefixes.

Input is dmrgpy's term list ``[(coef, [(opname, site), ...]), ...]``
(``multioperator.py:158-185`` ``to_terms``).  Each term is first brought to
site order with the fermionic reordering sign and Jordan-Wigner F strings
(the rules of ``pyitensor/autompo.py:47-103``), then reduced to its
non-identity span.  Purely imaginary site operators (e.g. Sy) are rewritten
as i times a real operator with the factor moved into the coefficient -- the
Sy-elimination idea of ``mpscpp3/mo_terms.h:33-120`` -- so Hamiltonians such
as Heisenberg, XXZ, TFIM and Hubbard compile to a REAL MPO and the sweep runs
in real arithmetic; anything that stays complex compiles to a complex MPO.

Construction: on every bond the automaton has a "start" state (nothing placed
yet), a "done" state (term finished) and one state per distinct operator
prefix still open across that bond.  Terms sharing a prefix share its states,
which gives the optimal bond dimension for nearest-neighbour chains (w = 5
for Heisenberg, 3 for TFIM, 6 for Hubbard).  When the automaton is wide
(long-range terms), a two-way SVD compression with the reference's 1e-14
weight cutoff (``pyitensor/mpobuilder.py:92-103``) follows.

MPO tensors are stored (w_left, d_in, d_out, w_right), d_in the ket leg.
"""
import numpy as np

from . import sites as S


def _order_and_sign(coef, factors):
    """Site-ascending stable insertion; a fermionic factor moved ahead of an
    odd number of fermionic factors flips the sign (pyitensor/autompo.py:47-61)."""
    coef = complex(coef)
    ops = []
    for name, site in factors:
        idx = 0
        while idx < len(ops) and ops[idx][1] <= site:
            idx += 1
        if idx < len(ops) and S.is_fermionic(name):
            if sum(1 for nm, _ in ops[idx:] if S.is_fermionic(nm)) % 2:
                coef = -coef
        ops.insert(idx, (name, site))
    return coef, ops


def _site_matrices(ops, types):
    """Per-site textbook matrices with Jordan-Wigner strings
    (pyitensor/autompo.py:63-103)."""
    by_site = {}
    for name, site in ops:
        by_site.setdefault(site, []).append(name)
    mats = []
    carry = False
    for site, code in enumerate(types, start=1):
        names = by_site.get(site)
        if names is None:
            mats.append(S.op(code, "F") if carry else S.op(code, "Id"))
            continue
        odd = sum(1 for nm in names if S.is_fermionic(nm)) % 2 == 1
        prod = S.op(code, names[0])
        for nm in names[1:]:
            prod = prod @ S.op(code, nm)
        if carry != odd:
            prod = prod @ S.op(code, "F")
        mats.append(prod)
        carry = carry != odd
    return mats


def compile_terms(types, terms, keep_zero=False):
    """-> (list of (coef, first_site, [matrices over the span], factor,
    term index), is_real).  Sites are 0-based here.  `factor` is the compiled
    coefficient per unit input coefficient (reordering sign times the powers
    of i moved out of imaginary site operators), so coef = factor * input
    coefficient.  Zero-coefficient terms are dropped unless keep_zero."""
    out = []
    real = True
    for t, (coef, factors) in enumerate(terms):
        c, ops = _order_and_sign(1.0, factors)
        factor = c
        c = c * complex(coef)
        if c == 0 and not keep_zero:
            continue
        mats = _site_matrices(ops, types)
        nontriv = [i for i, m in enumerate(mats) if not np.allclose(m, np.eye(m.shape[0]), atol=0.0, rtol=0.0)]
        if not nontriv:
            # pure identity: attach to site 0
            f = l = 0
        else:
            f, l = nontriv[0], nontriv[-1]
        span = []
        for m in mats[f:l + 1]:
            if np.all(m.imag == 0):
                span.append(m.real.copy())
            elif np.all(m.real == 0):
                c = c * 1j
                factor = factor * 1j
                span.append((m / 1j).real.copy())
            else:
                span.append(m)
                real = False
        out.append((c, f, span, factor, t))
    for c, _, _, _, _ in out:
        if abs(c.imag) > 1e-15 * max(1.0, abs(c)):
            real = False
    return out, real


class _OpTable:
    """Content-addressed ids for site matrices (prefix sharing key)."""

    def __init__(self):
        self.ids = {}

    def key(self, m):
        k = (m.shape, np.ascontiguousarray(m).tobytes())
        if k not in self.ids:
            self.ids[k] = len(self.ids)
        return self.ids[k]


def build_mpo(types, terms, compress_above=16, cutoff=1e-14, coupling_map=False):
    """Compile `terms` on sites of type codes `types` into a list of MPO
    tensors (w_left, d, d, w_right); returns (W, is_real).

    With coupling_map=True the automaton keeps zero-coefficient terms, is
    never compressed, and (W, is_real, cmap) is returned: cmap[t] =
    (site, ls, rs, M, factor) says that term t contributes
    factor * coef_t * M (stored (d_in, d_out)) to W[site][ls, :, :, rs], so W
    is affine in the coefficients and dW/dcoef_t is that single block."""
    n = len(types)
    dims = [S.dim(c) for c in types]
    compiled, real = compile_terms(types, terms, keep_zero=coupling_map)
    cmap = [None] * len(terms)
    dtype = np.float64 if real else np.complex128
    table = _OpTable()
    # states per bond b (between sites b-1 and b, b = 0..n): dict key -> index
    START, DONE = "start", "done"
    bond_states = [dict() for _ in range(n + 1)]
    for b in range(n + 1):
        if b < n:
            bond_states[b][START] = len(bond_states[b])
        if b > 0:
            bond_states[b][DONE] = len(bond_states[b])
    entries = [dict() for _ in range(n)]  # site -> {(lstate, rstate): matrix}

    def add(site, ls, rs, mat):
        key = (ls, rs)
        if key in entries[site]:
            entries[site][key] = entries[site][key] + mat
        else:
            entries[site][key] = mat.astype(dtype if real else complex)

    for c, f, span, factor, t in compiled:
        cval = c.real if real else c
        l = f + len(span) - 1
        if l == f:
            add(f, bond_states[f][START], bond_states[f + 1][DONE], cval * span[0])
            cmap[t] = (f, bond_states[f][START], bond_states[f + 1][DONE], span[0].T.copy(), factor)
            continue
        prefix = ()
        prev = bond_states[f][START]
        for j, m in enumerate(span[:-1]):
            site = f + j
            prefix = prefix + (table.key(m),)
            states = bond_states[site + 1]
            skey = ("open", f, prefix)
            if skey not in states:
                states[skey] = len(states)
                add(site, prev, states[skey], m)
            prev = states[skey]
        add(l, prev, bond_states[l + 1][DONE], cval * span[-1])
        cmap[t] = (l, prev, bond_states[l + 1][DONE], span[-1].T.copy(), factor)

    W = []
    for i in range(n):
        d = dims[i]
        wl, wr = len(bond_states[i]), len(bond_states[i + 1])
        T = np.zeros((wl, d, d, wr), dtype=dtype)
        if START in bond_states[i] and START in bond_states[i + 1]:
            T[bond_states[i][START], :, :, bond_states[i + 1][START]] = np.eye(d)
        if DONE in bond_states[i] and DONE in bond_states[i + 1]:
            T[bond_states[i][DONE], :, :, bond_states[i + 1][DONE]] = np.eye(d)
        for (ls, rs), m in entries[i].items():
            T[ls, :, :, rs] += m.T  # textbook (out,in) -> stored (in,out)
        W.append(T)
    if coupling_map:
        return W, real, cmap
    if max(w.shape[3] for w in W) > compress_above:
        W = compress(W, cutoff)
    return W, real


def _svd_keep(mat, cutoff):
    U, s, Vh = np.linalg.svd(mat, full_matrices=False)
    p = s ** 2
    tot = p.sum()
    if tot <= 0:
        return U[:, :1], s[:1], Vh[:1]
    p = p / tot
    tail = np.concatenate((np.cumsum(p[::-1])[::-1][1:], [0.0]))
    keep = max(1, int(np.count_nonzero(tail > cutoff)) + 1)
    keep = min(keep, len(s))
    return U[:, :keep], s[:keep], Vh[:keep]


def compress(W, cutoff=1e-14):
    """Two-way truncating SVD pass over the MPO bonds."""
    W = [w.copy() for w in W]
    n = len(W)
    for i in range(n - 1):
        wl, d1, d2, wr = W[i].shape
        U, s, Vh = _svd_keep(W[i].reshape(wl * d1 * d2, wr), cutoff)
        W[i] = U.reshape(wl, d1, d2, -1)
        W[i + 1] = np.tensordot(s[:, None] * Vh, W[i + 1], axes=([1], [0]))
    for i in range(n - 1, 0, -1):
        wl, d1, d2, wr = W[i].shape
        U, s, Vh = _svd_keep(W[i].reshape(wl, d1 * d2 * wr), cutoff)
        W[i] = Vh.reshape(-1, d1, d2, wr)
        W[i - 1] = np.tensordot(W[i - 1], U * s[None, :], axes=([3], [0]))
    return W


def mpo_to_dense(W):
    """Textbook (out, in) matrix of a small MPO (testing aid)."""
    M = W[0][0].transpose(1, 0, 2)  # (out, in, w)
    for w in W[1:]:
        x = np.tensordot(M, w, axes=([2], [0]))      # (O, I, in, out, w)
        x = x.transpose(0, 3, 1, 2, 4)
        M = x.reshape(x.shape[0] * x.shape[1], x.shape[2] * x.shape[3], x.shape[4])
    return M[:, :, 0]
