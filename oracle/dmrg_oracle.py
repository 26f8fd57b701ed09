"""NumPy restatement of dmrgpy's pure-Python two-site DMRG/TDVP sweep.

Test infrastructure only (the checker and the timed CPU baseline): never
imported by the product package.  Every function names the reference
file:line range whose algorithm it restates; paths are relative to
``src/dmrgpy/`` of joselado/dmrgpy.

Array conventions (shared with the fixtures under ``tests/golden``):

* MPS site tensor ``A[i]``: shape ``(chi_left, d, chi_right)``; the open ends
  carry explicit dimension-1 links (the reference omits them,
  ``pyitensor/mpscontainer.py:1-17``; a dimension-1 link changes no
  arithmetic).
* MPO site tensor ``W[i]``: shape ``(w_left, d_in, d_out, w_right)``; ``d_in``
  is the unprimed (ket) leg and ``d_out`` the primed (bra) leg
  (``pyitensor/sites/base.py:1-17``, ``pyitensor/mpobuilder.py:40-63``).
* Left environment ``L[a_bra, k, a_ket]``; right environment
  ``R[b_bra, n, b_ket]``.  The trivial edge environments are ``ones((1,1,1))``.
* Two-site centre tensor ``theta[a, s, t, b]`` -- the reference's
  ``order_in = [left_link, s_i, s_j, right_link]`` (``pyitensor/dmrg.py:238``).
"""

import numpy as np
from scipy.linalg import eigh_tridiagonal

__all__ = [
    "site_dim", "site_op", "is_fermionic", "hterm", "resolve_term",
    "dense_hamiltonian", "build_mpo", "truncate", "svd_truncated",
    "lanczos_ground_state", "lanczos_expm_multiply", "heff2_matvec",
    "heff1_matvec", "heff0_matvec", "extend_left", "extend_right",
    "right_environments", "left_environments", "local_ground_state",
    "dmrg_sweep", "dmrg", "random_mps", "OracleMPS", "inner", "expect",
    "bond_entropy", "tdvp_step", "mps_to_dense", "mpo_to_dense",
]

# --------------------------------------------------------------------------
# Site operators.  Convention of pyitensor/sites/base.py:1-17: the stored
# matrix is indexed [in, out], i.e. it is the transpose of the textbook
# (out, in) matrix.  Values follow from the textbook definitions below.
# --------------------------------------------------------------------------


def _spin_table(two_s):
    """Spin-S operators, basis ordered from m=+S down to m=-S
    (pyitensor/sites/spin.py:15-150 use the same ordering)."""
    s = two_s / 2.0
    d = two_s + 1
    m = np.array([s - k for k in range(d)])
    sp = np.zeros((d, d))
    for k in range(1, d):  # S+ |m_k> = sqrt(S(S+1) - m_k(m_k+1)) |m_k + 1>
        sp[k - 1, k] = np.sqrt(s * (s + 1) - m[k] * (m[k] + 1))
    sm = sp.T.copy()
    sz = np.diag(m)
    sx = 0.5 * (sp + sm)
    sy = (sp - sm) / 2j
    std = {"Sz": sz, "Sx": sx, "Sy": sy, "ISy": 1j * sy, "Sp": sp, "S+": sp,
           "Sm": sm, "S-": sm, "Sz2": sz @ sz, "Sx2": sx @ sx, "Sy2": (sy @ sy).real,
           "S2": s * (s + 1) * np.eye(d)}
    names = {2: ["Up", "Dn"], 3: ["Up", "Z0", "Dn"],
             5: ["Up", "Upi", "Z0", "Dni", "Dn"]}.get(d)
    if names:
        for k, nm in enumerate(names):
            p = np.zeros((d, d))
            p[k, k] = 1.0
            std["proj" + nm] = p
    return {k: np.asarray(v, dtype=complex).T.copy() for k, v in std.items()}


def _fock_table(modes):
    """Fermionic modes on one site; basis = occupation bit-strings with the
    first mode most significant in the (Emp, Up, Dn, UpDn) ordering used by
    pyitensor/sites/fermion.py:39-75.  c_j carries the in-site sign
    (-1)^(occupied modes before j)."""
    nm = len(modes)
    states = [tuple((idx >> (nm - 1 - j)) & 1 for j in range(nm)) for idx in range(2 ** nm)]
    if nm == 2:  # Emp, Up, Dn, UpDn
        states = [(0, 0), (1, 0), (0, 1), (1, 1)]
    d = len(states)
    pos = {st: k for k, st in enumerate(states)}

    def annihilate(j, signed):
        c = np.zeros((d, d))
        for st in states:
            if st[j] == 1:
                new = list(st)
                new[j] = 0
                sign = (-1) ** sum(st[:j]) if signed else 1
                c[pos[tuple(new)], pos[st]] = sign
        return c

    std = {}
    for j, mode in enumerate(modes):
        c = annihilate(j, True)
        a = annihilate(j, False)
        std["C" + mode] = c
        std["Cdag" + mode] = c.T.copy()
        std["A" + mode] = a
        std["Adag" + mode] = a.T.copy()
        n = np.diag([float(st[j]) for st in states])
        std["N" + mode] = n
        std["F" + mode] = np.diag([(-1.0) ** st[j] for st in states])
    parity = np.diag([(-1.0) ** sum(st) for st in states])
    std["F"] = parity
    std["FermiPhase"] = parity
    return std, states


def _spinless_table():
    std, _ = _fock_table([""])
    out = {"N": std["N"], "n": std["N"], "C": std["C"], "Cdag": std["Cdag"],
           "A": std["A"], "Adag": std["Adag"], "F": std["F"], "FermiPhase": std["F"],
           "projEmp": np.diag([1.0, 0.0]), "projOcc": np.diag([0.0, 1.0])}
    return {k: np.asarray(v, dtype=complex).T.copy() for k, v in out.items()}


def _electron_table():
    std, states = _fock_table(["up", "dn"])
    nup, ndn = std["Nup"], std["Ndn"]
    out = {"Nup": nup, "Ndn": ndn, "Nupdn": nup @ ndn, "Ntot": nup + ndn,
           "Cup": std["Cup"], "Cdagup": std["Cdagup"], "Cdn": std["Cdn"],
           "Cdagdn": std["Cdagdn"], "Aup": std["Aup"], "Adagup": std["Adagup"],
           "Adn": std["Adn"], "Adagdn": std["Adagdn"], "F": std["F"],
           "FermiPhase": std["F"], "Fup": std["Fup"], "Fdn": std["Fdn"]}
    # spin operators of the singly occupied doublet
    sp = std["Cdagup"] @ std["Cdn"]
    out["Sz"] = 0.5 * (nup - ndn)
    out["Sp"] = sp
    out["S+"] = sp
    out["Sm"] = sp.T.copy()
    out["S-"] = sp.T.copy()
    out["S2"] = 0.75 * (nup + ndn - 2 * nup @ ndn)
    return {k: np.asarray(v, dtype=complex).T.copy() for k, v in out.items()}


def _boson_table(d):
    a = np.zeros((d, d))
    for k in range(1, d):
        a[k - 1, k] = np.sqrt(k)
    out = {"N": np.diag(np.arange(d, dtype=float)), "A": a, "Adag": a.T.copy()}
    for k in range(d):
        p = np.zeros((d, d))
        p[k, k] = 1.0
        out["N" + str(k)] = p
    return {k: np.asarray(v, dtype=complex).T.copy() for k, v in out.items()}


_TABLES = {}


def _table(code):
    """Type codes of pyitensor/sites/siteset.py:20-40."""
    if code not in _TABLES:
        if code == 2:
            _TABLES[code] = _spin_table(1)
        elif code == 3:
            _TABLES[code] = _spin_table(2)
        elif code in (4, 5, 6):
            _TABLES[code] = _spin_table(code - 1)
        elif code == 0:
            _TABLES[code] = _spinless_table()
        elif code == 1:
            _TABLES[code] = _electron_table()
        elif 100 < code < 200:
            _TABLES[code] = _boson_table(code - 100)
        else:
            raise ValueError("site type code {} is not supported".format(code))
    return _TABLES[code]


def site_dim(code):
    return next(iter(_table(code).values())).shape[0]


def site_op(code, name):
    """Stored [in,out] matrix; 'Id' and the generic F fallback follow
    pyitensor/sites/base.py:42-57."""
    tab = _table(code)
    if name == "Id":
        return np.eye(site_dim(code), dtype=complex)
    if name in tab:
        return tab[name]
    if name in ("F", "FermiPhase"):
        return np.eye(site_dim(code), dtype=complex)
    raise ValueError("Operator '{}' not recognized for site type {}".format(name, code))


def is_fermionic(name):
    """pyitensor/sites/base.py:59-75: any name starting with 'C'."""
    return bool(name) and name[0] == "C"


# --------------------------------------------------------------------------
# Term compiler: pyitensor/autompo.py:47-103 and pyitensor/mpobuilder.py.
# --------------------------------------------------------------------------


def hterm(coef, factors):
    """Site-ascending insertion with the fermionic reordering sign
    (pyitensor/autompo.py:47-61)."""
    coef = complex(coef)
    ops = []
    for name, site in factors:
        idx = 0
        while idx < len(ops) and ops[idx][1] <= site:
            idx += 1
        if idx < len(ops) and is_fermionic(name):
            if sum(1 for nm, _ in ops[idx:] if is_fermionic(nm)) % 2 == 1:
                coef = -coef
        ops.insert(idx, (name, site))
    return coef, ops


def resolve_term(ops, types):
    """Per-site textbook matrices with Jordan-Wigner F strings
    (pyitensor/autompo.py:63-103)."""
    by_site = {}
    for name, site in ops:
        by_site.setdefault(site, []).append(name)
    out = []
    carry = False
    for site in range(1, len(types) + 1):
        code = types[site - 1]
        names = by_site.get(site)
        if names is None:
            out.append(site_op(code, "F").T if carry else site_op(code, "Id").T)
            continue
        odd = sum(1 for nm in names if is_fermionic(nm)) % 2 == 1
        mats = [site_op(code, nm).T for nm in names]
        if carry != odd:
            mats.append(site_op(code, "F").T)
        comb = mats[0]
        for mm in mats[1:]:
            comb = comb @ mm
        out.append(comb)
        carry = carry != odd
    return out


def dense_hamiltonian(types, terms):
    """Kronecker sum of resolved terms, site 1 most significant
    (pyitensor/autompo.py:144-164)."""
    dims = [site_dim(c) for c in types]
    total = int(np.prod(dims))
    H = np.zeros((total, total), dtype=complex)
    for coef, factors in terms:
        c, ops = hterm(coef, factors)
        mats = resolve_term(ops, types)
        full = mats[0]
        for mm in mats[1:]:
            full = np.kron(full, mm)
        H += c * full
    return H


def _mpo_shift_right(W, i, cutoff, maxdim):
    """pyitensor/mpscontainer.py:101-115 on MPO tensors (0-based i)."""
    T = W[i]
    wl, d1, d2, wr = T.shape
    U, S, Vh, keep, _ = svd_truncated(T.reshape(wl * d1 * d2, wr), cutoff, maxdim, 1)
    W[i] = U.reshape(wl, d1, d2, keep)
    SV = S[:keep, None] * Vh
    W[i + 1] = np.tensordot(SV, W[i + 1], axes=([1], [0]))


def _mpo_shift_left(W, i, cutoff, maxdim):
    """pyitensor/mpscontainer.py:117-127 on MPO tensors (0-based i)."""
    T = W[i]
    wl, d1, d2, wr = T.shape
    U, S, Vh, keep, _ = svd_truncated(T.reshape(wl, d1 * d2 * wr), cutoff, maxdim, 1)
    W[i] = Vh.reshape(keep, d1, d2, wr)
    US = U * S[None, :keep]
    W[i - 1] = np.tensordot(W[i - 1], US, axes=([3], [0]))


def build_mpo(types, terms, cutoff=1e-14, maxdim=5000):
    """One bond-dimension-1 MPO per term (pyitensor/mpobuilder.py:40-63),
    block concatenation (pyitensor/mpsalgebra.py:143-223), then a truncating
    left-to-right and right-to-left SVD pass (pyitensor/mpobuilder.py:92-103)."""
    n = len(types)
    dims = [site_dim(c) for c in types]
    if not terms:
        return [np.zeros((1, d, d, 1), dtype=complex) for d in dims]
    per_term = []
    for coef, factors in terms:
        c, ops = hterm(coef, factors)
        mats = resolve_term(ops, types)
        site_ws = [m.T.reshape(1, m.shape[0], m.shape[0], 1).astype(complex) for m in mats]
        site_ws[0] = site_ws[0] * c
        per_term.append(site_ws)
    T = len(per_term)
    if n == 1:
        return [sum(t[0] for t in per_term)]
    W = []
    for i in range(n):
        d = dims[i]
        wl = 1 if i == 0 else T
        wr = 1 if i == n - 1 else T
        comb = np.zeros((wl, d, d, wr), dtype=complex)
        for t, site_ws in enumerate(per_term):
            li = 0 if i == 0 else t
            ri = 0 if i == n - 1 else t
            comb[li, :, :, ri] = site_ws[i][0, :, :, 0]
        W.append(comb)
    for i in range(n - 1):
        _mpo_shift_right(W, i, cutoff, maxdim)
    for i in range(n - 1, 0, -1):
        _mpo_shift_left(W, i, cutoff, maxdim)
    return W


# --------------------------------------------------------------------------
# Truncation: pyitensor/svd.py.
# --------------------------------------------------------------------------

GRAM_MIN_RELATIVE_SV = 1e-7   # pyitensor/svd.py:101
GRAM_MIN_DIM = 16             # pyitensor/svd.py:105


def truncate(s, cutoff, maxdim, mindim):
    """(keep, discarded weight) -- pyitensor/svd.py:32-68."""
    n = len(s)
    p = np.asarray(s, dtype=float) ** 2
    total = p.sum()
    if total <= 0:
        return max(1, mindim), 0.0
    p = p / total
    hi = min(maxdim, n) if maxdim is not None else n
    j_upper = max(0, n - mindim)
    j_forced = min(max(0, n - hi), j_upper)
    if j_upper <= j_forced:
        j = j_forced
    else:
        p_asc = p[::-1]
        forced = float(p_asc[:j_forced].sum())
        tail = forced + np.concatenate(([0.0], np.cumsum(p_asc[j_forced:j_upper])))
        window = tail <= cutoff
        j = j_forced + (int(np.nonzero(window)[0].max()) if window.any() else 0)
    keep = n - j
    return keep, float(p[keep:].sum())


def svd_truncated(mat, cutoff, maxdim, mindim):
    """(U_keep, S_all, Vh_keep, keep, discarded): Gram-matrix route with the
    exact-SVD fallback -- pyitensor/svd.py:108-151."""
    m, n = mat.shape
    if min(m, n) >= GRAM_MIN_DIM:
        left = m <= n
        gram = mat @ mat.conj().T if left else mat.conj().T @ mat
        evals, evecs = np.linalg.eigh(gram)
        evals = evals[::-1]
        evecs = evecs[:, ::-1]
        S = np.sqrt(np.clip(evals, 0.0, None))
        keep, disc = truncate(S, cutoff, maxdim if maxdim else None, max(1, mindim))
        if S[0] > 0.0 and S[keep - 1] >= GRAM_MIN_RELATIVE_SV * S[0]:
            Wk = evecs[:, :keep]
            if left:
                U = Wk
                Vh = (Wk.conj().T @ mat) / S[:keep, None]
            else:
                Vh = Wk.conj().T
                U = (mat @ Wk) / S[None, :keep]
            return U, S, Vh, keep, disc
    U, S, Vh = np.linalg.svd(mat, full_matrices=False)
    keep, disc = truncate(S, cutoff, maxdim if maxdim else None, max(1, mindim))
    return U[:, :keep], S, Vh[:keep, :], keep, disc


# --------------------------------------------------------------------------
# Krylov solvers: pyitensor/dmrg.py:61-142 and pyitensor/tdvp.py:82-187.
# --------------------------------------------------------------------------


def _tridiag(alphas, betas):
    a = np.asarray(alphas, dtype=float)
    if len(a) == 1:
        return a.reshape(1, 1)
    b = np.asarray(betas, dtype=float)
    return np.diag(a) + np.diag(b, 1) + np.diag(b, -1)


def lanczos_ground_state(matvec, v0, niter=30, tol=1e-12):
    """Lanczos with full reorthogonalisation against every earlier vector,
    stopping when the lowest Ritz value changes by less than
    tol*max(1,|E|) -- pyitensor/dmrg.py:95-142.  Returns (E, v, k)."""
    beta0 = np.linalg.norm(v0)
    if beta0 == 0:
        v0 = np.random.default_rng(0).standard_normal(v0.shape) + 0j
        beta0 = np.linalg.norm(v0)
    q = v0 / beta0
    qs = [q]
    alphas, betas = [], []
    w = matvec(q)
    alpha = np.vdot(q, w).real
    alphas.append(alpha)
    w = w - alpha * q
    prev = float(np.linalg.eigvalsh(_tridiag(alphas, betas))[0])
    m = min(niter, v0.size)
    for _ in range(1, m):
        beta = np.linalg.norm(w)
        if beta < tol:
            break
        betas.append(beta)
        qn = w / beta
        qs.append(qn)
        w = matvec(qn)
        alpha = np.vdot(qn, w).real
        alphas.append(alpha)
        w = w - alpha * qn - beta * qs[-2]
        for qk in qs[:-1]:
            w = w - np.vdot(qk, w) * qk
        cur = float(np.linalg.eigvalsh(_tridiag(alphas, betas))[0])
        if abs(cur - prev) < tol * max(1.0, abs(cur)):
            break
        prev = cur
    ev, vec = np.linalg.eigh(_tridiag(alphas, betas))
    return ev[0], np.column_stack(qs) @ vec[:, 0], len(alphas)


def _eigh_tridiagonal_robust(alphas, betas):
    """pyitensor/tdvp.py:175-187."""
    try:
        return eigh_tridiagonal(alphas, betas)
    except np.linalg.LinAlgError:
        return eigh_tridiagonal(alphas, betas, lapack_driver="stebz")


KRYLOV_ERRGOAL = 1e-10  # pyitensor/tdvp.py:79


def lanczos_expm_multiply(matvec, v0, coeff, niter=30, tol=1e-12, errgoal=KRYLOV_ERRGOAL):
    """exp(coeff*A) v0 with Saad's a-posteriori stop -- pyitensor/tdvp.py:82-172.
    Returns (w, k)."""
    beta0 = np.linalg.norm(v0)
    if beta0 == 0:
        return v0.copy(), 0
    m = min(niter, v0.size)
    Q = np.empty((v0.size, m), dtype=complex)
    Q[:, 0] = v0 / beta0
    alphas, betas = [], []

    def exp_col0(k):
        if k == 1:
            return np.array([np.exp(coeff * alphas[0])], dtype=complex)
        ev, evec = _eigh_tridiagonal_robust(np.array(alphas[:k]), np.array(betas[:k - 1]))
        return evec @ (np.exp(coeff * ev) * evec[0, :])

    beta = 0.0
    for it in range(m):
        w = matvec(Q[:, it])
        alpha = np.vdot(Q[:, it], w).real
        alphas.append(alpha)
        w = w - alpha * Q[:, it]
        if it > 0:
            w = w - beta * Q[:, it - 1]
        Qk = Q[:, :it + 1]
        w = w - Qk @ (Qk.conj().T @ w)
        beta = np.linalg.norm(w)
        c = exp_col0(it + 1)
        if beta < tol or it == m - 1 or beta0 * beta * abs(c[-1]) < errgoal:
            return beta0 * (Qk @ c), it + 1
        betas.append(beta)
        Q[:, it + 1] = w / beta
    raise AssertionError("unreachable")


# --------------------------------------------------------------------------
# Effective Hamiltonians: pyitensor/kernels.py:298-410 (pairwise plan in the
# order theta*L, *W_i, *W_j, *R) and pyitensor/dmrg.py:224-299.
# --------------------------------------------------------------------------


def heff2_matvec(L, Wi, Wj, R, theta):
    """y[a',s',t',b'] = L[a',k,a] Wi[k,s,s',m] Wj[m,t,t',n] R[b',n,b] theta[a,s,t,b]."""
    x = np.tensordot(theta, L, axes=([0], [2]))          # (s,t,b,a',k)
    x = np.tensordot(x, Wi, axes=([0, 4], [1, 0]))       # (t,b,a',s',m)
    x = np.tensordot(x, Wj, axes=([0, 4], [1, 0]))       # (b,a',s',t',n)
    x = np.tensordot(x, R, axes=([0, 4], [2, 1]))        # (a',s',t',b')
    return x


def heff1_matvec(L, W, R, A):
    """pyitensor/dmrg.py:251-275: y[a',s',b'] = L W R A."""
    x = np.tensordot(A, L, axes=([0], [2]))              # (s,b,a',k)
    x = np.tensordot(x, W, axes=([0, 3], [1, 0]))        # (b,a',s',m)
    x = np.tensordot(x, R, axes=([0, 3], [2, 1]))        # (a',s',b')
    return x


def heff0_matvec(L, R, C):
    """pyitensor/dmrg.py:278-299: y[a',b'] = L[a',k,a] R[b',k,b] C[a,b]."""
    x = np.tensordot(C, L, axes=([0], [2]))              # (b,a',k)
    x = np.tensordot(x, R, axes=([0, 2], [2, 1]))        # (a',b')
    return x


# --------------------------------------------------------------------------
# Environments: pyitensor/dmrg.py:145-221.
# --------------------------------------------------------------------------


def extend_left(L, W, A):
    """L'[b',m,b] = L[a',k,a] conj(A[a',s',b']) W[k,s,s',m] A[a,s,b]
    (pyitensor/dmrg.py:170-191)."""
    x = np.tensordot(L, A, axes=([2], [0]))              # (a',k,s,b)
    x = np.tensordot(x, W, axes=([1, 2], [0, 1]))        # (a',b,s',m)
    x = np.tensordot(A.conj(), x, axes=([0, 1], [0, 2]))  # (b',b,m)
    return np.ascontiguousarray(x.transpose(0, 2, 1))


def extend_right(R, W, B):
    """R'[a',k,a] = B[a,s,b] R[b',m,b] W[k,s,s',m] conj(B[a',s',b'])
    (pyitensor/dmrg.py:194-201)."""
    x = np.tensordot(B, R, axes=([2], [2]))              # (a,s,b',m)
    x = np.tensordot(x, W, axes=([1, 3], [1, 3]))        # (a,b',k,s')
    x = np.tensordot(B.conj(), x, axes=([1, 2], [3, 1]))  # (a',a,k)
    return np.ascontiguousarray(x.transpose(0, 2, 1))


_EDGE = None


def _edge(dtype=complex):
    return np.ones((1, 1, 1), dtype=dtype)


def right_environments(W, A):
    """{i: R through sites i..N} for i = N+1..2, 1-based keys
    (pyitensor/dmrg.py:204-211)."""
    n = len(A)
    env = {n + 1: _edge(A[0].dtype)}
    for i in range(n, 1, -1):
        env[i] = extend_right(env[i + 1], W[i - 1], A[i - 1])
    return env


def left_environments(W, A):
    """{i: L through sites 1..i} for i = 0..N-1 (pyitensor/dmrg.py:214-221)."""
    n = len(A)
    env = {0: _edge(A[0].dtype)}
    for i in range(1, n):
        env[i] = extend_left(env[i - 1], W[i - 1], A[i - 1])
    return env


# --------------------------------------------------------------------------
# Sweep driver: pyitensor/dmrg.py:302-398.
# --------------------------------------------------------------------------


def local_ground_state(L, Wi, Wj, R, theta0, niter):
    """pyitensor/dmrg.py:302-333 (dense eigh for dim <= 3, Lanczos with the
    niter floor of 200 otherwise).  Returns (E, theta, k)."""
    shape = theta0.shape

    def mv(v):
        return heff2_matvec(L, Wi, Wj, R, v.reshape(shape)).reshape(-1)

    dim = theta0.size
    if dim <= 3:
        basis = np.eye(dim, dtype=complex)
        Hm = np.column_stack([mv(basis[:, k]) for k in range(dim)])
        w, v = np.linalg.eigh((Hm + Hm.conj().T) / 2)
        return float(w[0].real), v[:, 0].reshape(shape), dim
    e, v, k = lanczos_ground_state(mv, theta0.reshape(-1).astype(complex), niter=max(niter, 200))
    return float(e.real), v.reshape(shape), k


def split_theta(theta, cutoff, maxdim, direction):
    """pyitensor/dmrg.py:336-352: returns (A_i, A_ip1, S_all, keep, discarded)."""
    cl, d1, d2, cr = theta.shape
    U, S, Vh, keep, disc = svd_truncated(theta.reshape(cl * d1, d2 * cr), cutoff, maxdim, 1)
    if direction == "right":
        Ai = U.reshape(cl, d1, keep)
        Aj = (S[:keep, None] * Vh).reshape(keep, d2, cr)
    else:
        Ai = (U * S[None, :keep]).reshape(cl, d1, keep)
        Aj = Vh.reshape(keep, d2, cr)
    return Ai, Aj, S, keep, disc


def dmrg_sweep(A, W, maxdim, cutoff, niter, stats=None):
    """One left-to-right then right-to-left two-site sweep, in place;
    returns the last bond's eigenvalue (pyitensor/dmrg.py:355-382)."""
    n = len(A)
    energy = None
    renv = right_environments(W, A)
    lenv = {0: _edge(A[0].dtype)}
    for i in range(1, n):
        theta0 = np.tensordot(A[i - 1], A[i], axes=([2], [0]))
        energy, theta, k = local_ground_state(lenv[i - 1], W[i - 1], W[i], renv[i + 2], theta0, niter)
        A[i - 1], A[i], S, keep, disc = split_theta(theta, cutoff, maxdim, "right")
        if stats is not None:
            stats.append((i, "right", energy, k, keep, disc))
        lenv[i] = extend_left(lenv[i - 1], W[i - 1], A[i - 1])
    renv = {n + 1: _edge(A[0].dtype)}
    for i in range(n - 1, 0, -1):
        theta0 = np.tensordot(A[i - 1], A[i], axes=([2], [0]))
        energy, theta, k = local_ground_state(lenv[i - 1], W[i - 1], W[i], renv[i + 2], theta0, niter)
        A[i - 1], A[i], S, keep, disc = split_theta(theta, cutoff, maxdim, "left")
        if stats is not None:
            stats.append((i, "left", energy, k, keep, disc))
        renv[i + 1] = extend_right(renv[i + 2], W[i], A[i])
    return energy


def dmrg(A, W, maxdims, cutoffs, niters=2, stats=None):
    """pyitensor/dmrg.py:385-398 with a Sweeps schedule
    (pyitensor/sweeps.py:14-48): one entry per sweep."""
    nsweep = len(maxdims)
    cutoffs = cutoffs if isinstance(cutoffs, (list, tuple)) else [cutoffs] * nsweep
    niters = niters if isinstance(niters, (list, tuple)) else [niters] * nsweep
    energy = None
    for s in range(nsweep):
        energy = dmrg_sweep(A, W, maxdims[s], cutoffs[s], niters[s], stats)
    return energy


# --------------------------------------------------------------------------
# MPS helpers: random initial state (pyitensor/mpsalgebra.py:315-353),
# canonical moves (pyitensor/mpscontainer.py:81-127), inner products
# (pyitensor/mpsalgebra.py:66-106) and the bond entropy
# (pyitensor/chain.py:468-480).
# --------------------------------------------------------------------------


class OracleMPS:
    def __init__(self, tensors, center=None):
        self.A = [np.asarray(t) for t in tensors]
        self.center = center

    def copy(self):
        return OracleMPS([t.copy() for t in self.A], self.center)

    def _shift_right(self, i, cutoff=0.0, maxdim=None):
        T = self.A[i - 1]
        cl, d, cr = T.shape
        U, S, Vh, keep, _ = svd_truncated(T.reshape(cl * d, cr), cutoff, maxdim, 1)
        self.A[i - 1] = U.reshape(cl, d, keep)
        self.A[i] = np.tensordot(S[:keep, None] * Vh, self.A[i], axes=([1], [0]))

    def _shift_left(self, i, cutoff=0.0, maxdim=None):
        T = self.A[i - 1]
        cl, d, cr = T.shape
        U, S, Vh, keep, _ = svd_truncated(T.reshape(cl, d * cr), cutoff, maxdim, 1)
        self.A[i - 1] = Vh.reshape(keep, d, cr)
        self.A[i - 2] = np.tensordot(self.A[i - 2], U * S[None, :keep], axes=([2], [0]))

    def position(self, b, cutoff=0.0, maxdim=None):
        if self.center is None:
            raise RuntimeError("position(): orthogonality center is unknown")
        while self.center < b:
            self._shift_right(self.center, cutoff, maxdim)
            self.center += 1
        while self.center > b:
            self._shift_left(self.center, cutoff, maxdim)
            self.center -= 1
        return self

    def normalize(self):
        nrm = inner(self.A, self.A).real ** 0.5
        c = self.center or 1
        self.A[c - 1] = self.A[c - 1] * (1.0 / nrm)
        return self


def random_mps(dims, m, rng=np.random):
    """Bond dims min(prod d, m) from both ends, complex Gaussian entries drawn
    from the global generator in site order, lossless left-to-right
    canonicalisation, normalisation (pyitensor/mpsalgebra.py:315-353)."""
    n = len(dims)
    left_cum = 1
    bond = []
    for d in dims[:-1]:
        left_cum = min(left_cum * d, m)
        bond.append(left_cum)
    right_cum = 1
    for k in range(n - 2, -1, -1):
        right_cum = min(right_cum * dims[k + 1], m)
        bond[k] = min(bond[k], right_cum)
    tensors = []
    for i in range(n):
        cl = bond[i - 1] if i > 0 else 1
        cr = bond[i] if i < n - 1 else 1
        ref_shape = tuple(([cl] if i > 0 else []) + [dims[i]] + ([cr] if i < n - 1 else []))
        arr = rng.randn(*ref_shape) + 1j * rng.randn(*ref_shape)
        tensors.append(arr.reshape(cl, dims[i], cr))
    psi = OracleMPS(tensors, center=1)
    psi.position(n)
    psi.normalize()
    return psi


def inner(A, B):
    """<A|B> by left transfer matrices."""
    E = np.ones((1, 1), dtype=complex)
    for a, b in zip(A, B):
        x = np.tensordot(E, b, axes=([1], [0]))          # (a', s, b)
        E = np.tensordot(a.conj(), x, axes=([0, 1], [0, 1]))
    return complex(E.reshape(-1)[0])


def expect(bra, W, ket):
    """<bra|W|ket> by left environments."""
    L = np.ones((1, 1, 1), dtype=complex)
    for a, w, b in zip(bra, W, ket):
        x = np.tensordot(L, b, axes=([2], [0]))
        x = np.tensordot(x, w, axes=([1, 2], [0, 1]))
        L = np.tensordot(a.conj(), x, axes=([0, 1], [0, 2])).transpose(0, 2, 1)
    return complex(L.reshape(-1)[0])


def bond_entropy(psi, b):
    """von Neumann entropy of the bond (b, b+1), p > 1e-12 only
    (pyitensor/chain.py:468-480)."""
    ps = psi.copy()
    ps.position(b)
    theta = np.tensordot(ps.A[b - 1], ps.A[b], axes=([2], [0]))
    cl, d1, d2, cr = theta.shape
    _, S, _, keep, _ = svd_truncated(theta.reshape(cl * d1, d2 * cr), 0.0, None, 1)
    p = S.astype(float) ** 2
    tot = p.sum()
    probs = p[:keep] / tot if tot > 0 else p[:keep]
    return float(-sum(x * np.log(x) for x in probs if x > 1e-12))


def mps_to_dense(A):
    v = A[0]
    for a in A[1:]:
        v = np.tensordot(v, a, axes=([-1], [0]))
    return v.reshape(-1)


def mpo_to_dense(W):
    """Textbook (out, in) matrix of an MPO, site 1 most significant."""
    T = W[0]  # (1, in, out, w)
    n_in = T.shape[1]
    M = T[0].transpose(1, 0, 2)  # (out, in, w)
    out_dim, in_dim = M.shape[0], M.shape[1]
    for w in W[1:]:
        d = w.shape[1]
        x = np.tensordot(M, w, axes=([2], [0]))          # (O, I, in, out, w)
        x = x.transpose(0, 3, 1, 2, 4)                  # (O, out, I, in, w)
        out_dim *= d
        in_dim *= d
        M = x.reshape(out_dim, in_dim, x.shape[-1])
    del n_in
    return M[:, :, 0]


# --------------------------------------------------------------------------
# TDVP: pyitensor/tdvp.py:190-368 and pyitensor/svd.py:198-244.
# --------------------------------------------------------------------------


def _evolve2(L, Wi, Wj, R, theta, coeff, niter):
    shape = theta.shape
    out, _ = lanczos_expm_multiply(
        lambda v: heff2_matvec(L, Wi, Wj, R, v.reshape(shape)).reshape(-1),
        theta.reshape(-1).astype(complex), coeff, niter=niter)
    return out.reshape(shape)


def _evolve1(L, W, R, A, coeff, niter):
    shape = A.shape
    out, _ = lanczos_expm_multiply(
        lambda v: heff1_matvec(L, W, R, v.reshape(shape)).reshape(-1),
        A.reshape(-1).astype(complex), coeff, niter=niter)
    return out.reshape(shape)


def _evolve0(L, R, C, coeff, niter):
    shape = C.shape
    out, _ = lanczos_expm_multiply(
        lambda v: heff0_matvec(L, R, v.reshape(shape)).reshape(-1),
        C.reshape(-1).astype(complex), coeff, niter=niter)
    return out.reshape(shape)


def _half_sweep_lr(A, W, tau, cutoff, maxdim, niter):
    """pyitensor/tdvp.py:220-246."""
    n = len(A)
    renv = right_environments(W, A)
    lenv = {0: _edge(complex)}
    for i in range(1, n):
        theta = np.tensordot(A[i - 1], A[i], axes=([2], [0]))
        theta = _evolve2(lenv[i - 1], W[i - 1], W[i], renv[i + 2], theta, -1j * tau, niter)
        A[i - 1], C, _, _, _ = split_theta(theta, cutoff, maxdim, "right")
        A[i] = C
        lenv[i] = extend_left(lenv[i - 1], W[i - 1], A[i - 1])
        if i < n - 1:
            A[i] = _evolve1(lenv[i], W[i], renv[i + 2], C, 1j * tau, niter)


def _half_sweep_rl(A, W, tau, cutoff, maxdim, niter):
    """pyitensor/tdvp.py:249-273."""
    n = len(A)
    lenv = left_environments(W, A)
    renv = {n + 1: _edge(complex)}
    for i in range(n - 1, 0, -1):
        theta = np.tensordot(A[i - 1], A[i], axes=([2], [0]))
        theta = _evolve2(lenv[i - 1], W[i - 1], W[i], renv[i + 2], theta, -1j * tau, niter)
        C, A[i], _, _, _ = split_theta(theta, cutoff, maxdim, "left")
        A[i - 1] = C
        renv[i + 1] = extend_right(renv[i + 2], W[i], A[i])
        if i > 1:
            A[i - 1] = _evolve1(lenv[i - 1], W[i - 1], renv[i + 1], C, 1j * tau, niter)


def _half_sweep_lr_onesite(A, W, tau, niter):
    """pyitensor/tdvp.py:276-314 with the QR split of pyitensor/svd.py:198-244."""
    n = len(A)
    renv = right_environments(W, A)
    lenv = {0: _edge(complex)}
    for i in range(1, n + 1):
        Anew = _evolve1(lenv[i - 1], W[i - 1], renv[i + 1], A[i - 1], -1j * tau, niter)
        if i == n:
            A[i - 1] = Anew
            continue
        cl, d, cr = Anew.shape
        Q, Cm = np.linalg.qr(Anew.reshape(cl * d, cr), mode="reduced")
        k = Q.shape[1]
        A[i - 1] = Q.reshape(cl, d, k)
        orig_next = A[i]
        lenv[i] = extend_left(lenv[i - 1], W[i - 1], A[i - 1])
        Cev = _evolve0(lenv[i], renv[i + 1], Cm, 1j * tau, niter)
        A[i] = np.tensordot(Cev, orig_next, axes=([1], [0]))


def _half_sweep_rl_onesite(A, W, tau, niter):
    """pyitensor/tdvp.py:317-347."""
    n = len(A)
    lenv = left_environments(W, A)
    renv = {n + 1: _edge(complex)}
    for i in range(n, 0, -1):
        Anew = _evolve1(lenv[i - 1], W[i - 1], renv[i + 1], A[i - 1], -1j * tau, niter)
        if i == 1:
            A[i - 1] = Anew
            continue
        cl, d, cr = Anew.shape
        Qh, Rm = np.linalg.qr(Anew.reshape(cl, d * cr).conj().T, mode="reduced")
        Cm, V = Rm.conj().T, Qh.conj().T
        k = V.shape[0]
        A[i - 1] = V.reshape(k, d, cr)
        orig_prev = A[i - 2]
        renv[i] = extend_right(renv[i + 1], W[i - 1], A[i - 1])
        Cev = _evolve0(lenv[i - 1], renv[i], Cm, 1j * tau, niter)
        A[i - 2] = np.tensordot(orig_prev, Cev, axes=([2], [0]))


def tdvp_step(A, W, dt, cutoff, maxdim, niter=50, num_center=2):
    """pyitensor/tdvp.py:350-368: left-to-right then right-to-left half
    sweeps of dt/2 each, in place on the list of site tensors."""
    A[:] = [np.asarray(a, dtype=complex) for a in A]
    W = [np.asarray(w, dtype=complex) for w in W]
    tau = dt / 2.0
    if num_center == 1:
        _half_sweep_lr_onesite(A, W, tau, niter)
        _half_sweep_rl_onesite(A, W, tau, niter)
    else:
        _half_sweep_lr(A, W, tau, cutoff, maxdim, niter)
        _half_sweep_rl(A, W, tau, cutoff, maxdim, niter)
    return A
