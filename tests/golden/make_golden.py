"""Generate the golden fixtures in this directory by running dmrgpy's own
pure-Python backend (``src/dmrgpy/pyitensor``) on small inputs.

Run from the repository root with the reference checkout on disk:

    python tests/golden/make_golden.py /path/to/dmrgpy

The reference imports numba at module level in two places it never uses on
this path (``algebra/kpmextrapolate.py:2``, ``edtk/dynamics.py:213``), so a
stand-in module with identity ``jit``/``njit`` is registered before import.
The fixtures hold plain arrays in the layout documented in
``oracle/dmrg_oracle.py`` plus the term lists as JSON.
"""
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _install_numba_stub():
    mod = types.ModuleType("numba")

    def jit(*a, **k):
        if a and callable(a[0]) and len(a) == 1 and not k:
            return a[0]
        return lambda f: f
    mod.jit = jit
    mod.njit = jit
    mod.prange = range
    sys.modules["numba"] = mod


def _arr_lpr(psi, i):
    from dmrgpy.pyitensor.mpsalgebra import _link_at
    T = psi.A(i)
    n = psi.length()
    phys = next(ind for ind in T.inds if ind.hastags("Site"))
    left = _link_at(psi, i, i - 1)
    right = _link_at(psi, i, i + 1)
    order = [x for x in (left, phys, right) if x is not None]
    a = T.transpose_to(order)
    cl = left.dim if left else 1
    cr = right.dim if right else 1
    return np.ascontiguousarray(a.reshape(cl, phys.dim, cr))


def _mpo_arrays(H):
    from dmrgpy.pyitensor.mpsalgebra import _link_at
    n = H.length()
    out = []
    for i in range(1, n + 1):
        T = H.A(i)
        s = next(ind for ind in T.inds if ind.hastags("Site") and ind.plev == 0)
        sp = s.prime(1)
        left = _link_at(H, i, i - 1)
        right = _link_at(H, i, i + 1)
        order = [x for x in (left, s, sp, right) if x is not None]
        a = T.transpose_to(order)
        out.append(np.ascontiguousarray(a.reshape(left.dim if left else 1, s.dim, s.dim,
                                                  right.dim if right else 1)))
    return out


def _env_array(env_tensor, bra, mpo_link, ket):
    if env_tensor is None:
        return np.ones((1, 1, 1), dtype=complex)
    return np.ascontiguousarray(env_tensor.transpose_to([bra, mpo_link, ket]))


def terms_heisenberg(n, J=1.0):
    t = []
    for i in range(1, n):
        for op in ("Sx", "Sy", "Sz"):
            t.append((complex(J), [(op, i), (op, i + 1)]))
    return t


def terms_tfim(n, J=1.0, h=1.0):
    t = [(complex(-J), [("Sz", i), ("Sz", i + 1)]) for i in range(1, n)]
    t += [(complex(h), [("Sx", i)]) for i in range(1, n + 1)]
    return t


def terms_xxz(n, delta):
    t = []
    for i in range(1, n):
        t.append((1.0 + 0j, [("Sx", i), ("Sx", i + 1)]))
        t.append((1.0 + 0j, [("Sy", i), ("Sy", i + 1)]))
        t.append((complex(delta), [("Sz", i), ("Sz", i + 1)]))
    return t


def main(ref_root):
    _install_numba_stub()
    sys.path.insert(0, os.path.join(ref_root, "src"))
    import warnings
    warnings.simplefilter("ignore")
    from dmrgpy import fermionchain
    from dmrgpy.pyitensor import AutoMPO, to_mpo, randomMPS, Sweeps
    from dmrgpy.pyitensor.chain import Chain
    from dmrgpy.pyitensor.dmrg import (_all_right_environments, _all_left_environments,
                                       _extend_left, two_site_heff, one_site_heff,
                                       _lanczos_ground_state, dmrg)
    from dmrgpy.pyitensor.mpsalgebra import _link_at, inner
    from dmrgpy.pyitensor.sites import SiteX
    from dmrgpy.pyitensor.svd import svd
    from dmrgpy.pyitensor.tdvp import tdvp_step
    from dmrgpy.pyitensor.mpscontainer import MPS
    from dmrgpy.pyitensor.index import Index
    from dmrgpy.pyitensor.tensor import ITensor

    meta = {"generator": "tests/golden/make_golden.py", "reference": "joselado/dmrgpy pyitensor"}
    terms_store = {}

    # Hubbard terms through the reference's own Jordan-Wigner transform
    fc = fermionchain.Spinful_Fermionic_Chain_Native(4)
    h = 0
    for i in range(3):
        h = h + fc.Cdagup[i] * fc.Cup[i + 1] + fc.Cdagdn[i] * fc.Cdn[i + 1]
    h = -1.0 * (h + h.get_dagger())
    for i in range(4):
        h = h + 4.0 * (fc.Nup[i] - 0.5) * (fc.Ndn[i] - 0.5)
    terms_store["hubbard4"] = h.to_terms()
    fs = fermionchain.Fermionic_Chain(8)
    hs = 0
    for i in range(7):
        hs = hs + fs.Cdag[i] * fs.C[i + 1]
    hs = hs + hs.get_dagger()
    for i in range(7):
        hs = hs + 0.7 * fs.N[i] * fs.N[i + 1]
    for i in range(8):
        hs = hs - 0.3 * fs.N[i]
    terms_store["spinless8"] = hs.to_terms()
    terms_store["heis6"] = terms_heisenberg(6)
    terms_store["heis_s1_5"] = terms_heisenberg(5)
    terms_store["tfim6"] = terms_tfim(6, 1.0, 0.8)
    terms_store["xxz8"] = terms_xxz(8, 0.5)
    types_store = {"hubbard4": [1] * 4, "spinless8": [0] * 8, "heis6": [2] * 6,
                   "heis_s1_5": [3] * 5, "tfim6": [2] * 6, "xxz8": [2] * 8}

    arrays = {}
    # 1. dense Hamiltonians of the reference MPOs (term compiler parity)
    for key, terms in terms_store.items():
        sites = SiteX(types_store[key])
        H = to_mpo(AutoMPO.from_terms(sites, terms), cutoff=1e-14, maxdim=5000)
        Ws = _mpo_arrays(H)
        dense = AutoMPO.from_terms(sites, terms).dense_matrix()
        arrays["mpo_dense_" + key] = dense
        arrays["mpo_wdims_" + key] = np.array([w.shape[0] for w in Ws] + [Ws[-1].shape[3]])

    # 2. matvec / environment fixtures from a random MPS
    def heff_fixture(tag, types, terms, chi, bond, seed):
        np.random.seed(seed)
        sites = SiteX(types)
        H = to_mpo(AutoMPO.from_terms(sites, terms), cutoff=1e-14, maxdim=5000)
        psi = randomMPS(sites, chi)
        n = len(types)
        renv = _all_right_environments(H, psi)
        lenv = _all_left_environments(H, psi)
        i = bond
        L, Lbra = lenv[i - 1]
        R, Rbra = renv[i + 2]
        mv, order_in, shape, x0 = two_site_heff(L, Lbra, H, psi, i, R, Rbra)
        y = mv(x0)
        left_link = _link_at(psi, i, i - 1)
        right_link = _link_at(psi, i + 1, i + 2)
        hl = _link_at(H, i, i - 1)
        hr = _link_at(H, i + 1, i + 2)
        cl = left_link.dim if left_link else 1
        cr = right_link.dim if right_link else 1
        d1, d2 = sites.dim(i), sites.dim(i + 1)
        Ws = _mpo_arrays(H)
        arrays[tag + "_L"] = _env_array(L, Lbra, hl, left_link)
        arrays[tag + "_R"] = _env_array(R, Rbra, hr, right_link)
        arrays[tag + "_Wi"] = Ws[i - 1]
        arrays[tag + "_Wj"] = Ws[i]
        arrays[tag + "_theta"] = x0.reshape(cl, d1, d2, cr)
        arrays[tag + "_y"] = y.reshape(cl, d1, d2, cr)
        # one-site effective Hamiltonian on site i+1 with L through i, R through i+2
        Lnew, Lnewbra = _extend_left(L, Lbra, H, psi, i)
        mid = _link_at(psi, i, i + 1)
        arrays[tag + "_Lnext"] = _env_array(Lnew, Lnewbra, _link_at(H, i, i + 1), mid)
        arrays[tag + "_Ai"] = _arr_lpr(psi, i)
        mv1, o1, s1, x1 = one_site_heff(Lnew, Lnewbra, H, psi, i + 1, R, Rbra)
        arrays[tag + "_A1"] = _arr_lpr(psi, i + 1)
        arrays[tag + "_y1"] = mv1(x1).reshape(arrays[tag + "_A1"].shape)
        # right environment one step further left (R through i+1)
        arrays[tag + "_Rprev"] = _env_array(renv[i + 1][0], renv[i + 1][1], _link_at(H, i, i + 1), mid)
        arrays[tag + "_Aj"] = _arr_lpr(psi, i + 1)

    heff_fixture("mv_heis", [2] * 8, terms_heisenberg(8), 12, 3, 11)
    heff_fixture("mv_edge", [2] * 6, terms_heisenberg(6), 8, 1, 12)
    heff_fixture("mv_s1", [3] * 6, terms_heisenberg(6), 9, 2, 13)
    heff_fixture("mv_hub", [1] * 4, terms_store["hubbard4"], 16, 2, 14)

    # 3. random MPS reproduction
    np.random.seed(7)
    sites = SiteX([2] * 6)
    psi = randomMPS(sites, 8)
    for i in range(1, 7):
        arrays["rmps_A%d" % i] = _arr_lpr(psi, i)

    # 4. truncation
    rng = np.random.default_rng(3)
    Um, _ = np.linalg.qr(rng.standard_normal((40, 40)) + 1j * rng.standard_normal((40, 40)))
    Vm, _ = np.linalg.qr(rng.standard_normal((60, 40)) + 1j * rng.standard_normal((60, 40)))
    sv = np.exp(-0.6 * np.arange(40))
    M = (Um * sv) @ Vm.conj().T
    arrays["svd_M"] = M
    i1, i2 = Index(40, "Link"), Index(60, "Link")
    T = ITensor((i1, i2), M)
    for tag, cut, md in (("a", 1e-12, None), ("b", 1e-8, 30), ("c", 0.0, 10)):
        U, S, V, spec = svd(T, [i1], cutoff=cut, maxdim=md)
        arrays["svd_%s_S" % tag] = np.array(spec.singular_values)
        arrays["svd_%s_trunc" % tag] = np.array([spec.truncerr])
        arrays["svd_%s_rec" % tag] = (U * S * V).transpose_to([i1, i2])

    # 5. Lanczos on a dense Hermitian operator
    A = rng.standard_normal((80, 80)) + 1j * rng.standard_normal((80, 80))
    A = A + A.conj().T
    v0 = rng.standard_normal(80) + 1j * rng.standard_normal(80)
    e, v = _lanczos_ground_state(lambda x: A @ x, v0, niter=200)
    arrays["lz_A"] = A
    arrays["lz_v0"] = v0
    arrays["lz_E"] = np.array([e])
    arrays["lz_v"] = v

    # 6. ground-state energies through the reference session
    results = {}

    def gs(tag, types, terms, maxm, nsweeps, seed, ed=False, entropy_bond=None):
        np.random.seed(seed)
        c = Chain(types)
        c.set_sweep_params(maxm, nsweeps, 1e-12, 0.0)
        c.set_hamiltonian(terms)
        t0 = time.time()
        e = c.gs_energy()
        dt = time.time() - t0
        r = {"E": e, "seconds": dt, "maxm": maxm, "nsweeps": nsweeps, "seed": seed}
        if ed:
            sites = SiteX(types)
            r["E_ed"] = float(np.linalg.eigvalsh(AutoMPO.from_terms(sites, terms).dense_matrix())[0])
        if entropy_bond is not None:
            r["S_vN"] = c.bond_entropy(c.gs_wavefunction(), entropy_bond)
            n = len(types)
            r["szsz_1N"] = c.vev([(1.0 + 0j, [("Sz", 1), ("Sz", n)])], c.gs_wavefunction()).real
        results[tag] = r
        print(tag, r, flush=True)

    gs("heis32_chi64", [2] * 32, terms_heisenberg(32), 64, 10, 0, entropy_bond=16)
    gs("heis12_chi64", [2] * 12, terms_heisenberg(12), 64, 6, 1, ed=True, entropy_bond=6)
    gs("tfim4", [2] * 4, [(-1.0 + 0j, [("Sz", i), ("Sz", i + 1)]) for i in range(1, 4)]
       + [(1.0 + 0j, [("Sx", i)]) for i in range(1, 5)], 16, 6, 2, ed=True)
    gs("s1_heis10_chi32", [3] * 10, terms_heisenberg(10), 32, 6, 3, entropy_bond=5)
    gs("s1_heis8_chi81", [3] * 8, terms_heisenberg(8), 81, 6, 6, ed=True, entropy_bond=4)
    gs("hub4_chi32", [1] * 4, terms_store["hubbard4"], 32, 6, 4, ed=True)
    gs("spinless8_chi32", [0] * 8, terms_store["spinless8"], 32, 6, 5, ed=True)

    # 7. TDVP from the Neel state (two-site and one-site) on XXZ N=8
    def neel(sites, n):
        links = [Index(1, tags="Link") for _ in range(n - 1)]
        ts = []
        for i in range(n):
            phys = sites.si(i + 1)
            inds = ([links[i - 1]] if i > 0 else []) + [phys] + ([links[i]] if i < n - 1 else [])
            a = np.zeros(tuple(x.dim for x in inds), dtype=complex)
            idx = [0] * len(inds)
            idx[1 if i > 0 else 0] = i % 2
            a[tuple(idx)] = 1.0
            ts.append(ITensor(tuple(inds), a))
        m = MPS(ts)
        m.center = 1
        return m

    n = 8
    sites = SiteX([2] * n)
    H = to_mpo(AutoMPO.from_terms(sites, terms_store["xxz8"]), cutoff=1e-14, maxdim=5000)
    arrays["tdvp_W_dims"] = np.array([n])
    for nc in (2, 1):
        psi = neel(sites, n)
        if nc == 1:
            # one-site TDVP keeps bond dims fixed: start from a two-site-evolved state
            psi = tdvp_step(psi, H, 0.1, cutoff=1e-12, maxdim=16, niter=50, num_center=2)
        for step in range(3):
            psi = tdvp_step(psi, H, 0.05, cutoff=1e-12, maxdim=16, niter=50, num_center=nc)
            vec = None
            arrs = [_arr_lpr(psi, i) for i in range(1, n + 1)]
            v = arrs[0]
            for a in arrs[1:]:
                v = np.tensordot(v, a, axes=([-1], [0]))
            arrays["tdvp%d_step%d" % (nc, step)] = v.reshape(-1)
        if nc == 2:
            arrays["tdvp2_start"] = np.array([0])
    for k, v in list(arrays.items()):
        if isinstance(v, np.ndarray) and v.dtype == complex and np.abs(v.imag).max(initial=0) == 0:
            pass
    np.savez_compressed(os.path.join(HERE, "reference_fixtures.npz"), **arrays)
    with open(os.path.join(HERE, "reference_terms.json"), "w") as f:
        json.dump({"meta": meta,
                   "types": types_store,
                   "terms": {k: [[[c.real, c.imag], [[nm, s] for nm, s in ops]] for c, ops in v]
                             for k, v in terms_store.items()},
                   "ground_states": results}, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
