"""The GB300 backend driven through dmrgpy's own API (the drop-in boundary).

dmrgpy is imported from its installed copy (``baseline/_ref`` at the
repository root, or anywhere on ``sys.path``) with a stand-in ``numba``
module, because ``algebra/kpmextrapolate.py:2`` imports numba at module
level for code this path never runs.  Without dmrgpy the tests are skipped.

CPU tests: the registered tags route like the python backend, the session
class is a subclass of dmrgpy's python-backend session, and the handle
conversions at the boundary are exact.  GPU tests: ``Spin_Chain(...,
itensor_version=tag)`` against ``itensor_version="python"`` through
``gs_energy``, ``get_gs``, ``vev``, ``get_entropy``, the
``evolve_and_measure`` glue and the session's ``tdvp_step`` and
``quench_tdvp``: energies to 1e-10 per site, observables to 1e-8 at an
exact bond dimension, time-evolved values to 1e-8."""
import os
import sys
import types
import warnings

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _dmrgpy():
    ref = os.path.join(ROOT, "baseline", "_ref")
    if os.path.isdir(ref) and ref not in sys.path:
        sys.path.append(ref)
    if "numba" not in sys.modules:
        try:
            import numba  # noqa: F401
        except ImportError:
            mod = types.ModuleType("numba")

            def jit(*a, **k):
                if a and callable(a[0]) and len(a) == 1 and not k:
                    return a[0]
                return lambda f: f
            mod.jit = jit
            mod.njit = jit
            mod.prange = range
            sys.modules["numba"] = mod
    warnings.simplefilter("ignore")
    return pytest.importorskip("dmrgpy")


def _heisenberg(sc, n):
    h = 0
    for i in range(n - 1):
        h = h + sc.Sx[i] * sc.Sx[i + 1] + sc.Sy[i] * sc.Sy[i + 1] + sc.Sz[i] * sc.Sz[i + 1]
    return h


def test_registered_session_is_a_python_backend_session():
    _dmrgpy()
    from dmrgpy import cppext
    from dmrgpy.pyitensor import chain as pychain
    import dmrgpy_gb300
    for prec in ("fp64", "tf32x3"):
        tag = dmrgpy_gb300.register(prec)
        assert tag == "python" and tag in (2, 3, "python") and hash(tag) != hash("python")
        cls = cppext.get_backend(tag).Chain
        assert issubclass(cls, pychain.Chain) and cls.contraction_precision == prec
        assert cppext.get_backend("python") is not cppext.get_backend(tag)


def test_handle_conversions_are_exact():
    _dmrgpy()
    from dmrgpy.pyitensor.mpsalgebra import randomMPS
    from dmrgpy.pyitensor.sites import SiteX
    from dmrgpy.pyitensor.mpobuilder import to_mpo
    from dmrgpy.pyitensor.autompo import AutoMPO
    from dmrgpy_gb300 import session as S
    np.random.seed(4)
    sites = SiteX([2, 3, 2, 2, 3])
    psi = randomMPS(sites, 6)
    arrs = S.mps_to_arrays(psi)
    back = S.arrays_to_mps(arrs, sites)
    v1 = O.mps_to_dense(arrs)
    v2 = O.mps_to_dense(S.mps_to_arrays(back))
    assert np.max(np.abs(v1 - v2)) == 0.0
    terms = [(0.7 + 0j, [("Sz", 1), ("Sz", 2)]), (0.3 + 0j, [("Sx", 2), ("Sx", 3)]), (1.1 + 0j, [("Sz", 5)])]
    H = to_mpo(AutoMPO.from_terms(sites, terms), cutoff=1e-14, maxdim=100)
    dense_ref = AutoMPO.from_terms(sites, terms).dense_matrix()
    assert np.max(np.abs(O.mpo_to_dense(S.mpo_to_arrays(H)) - dense_ref)) < 1e-12


def _pair(n, maxm, nsweeps, prec, seed=0):
    dmrgpy = _dmrgpy()
    from dmrgpy import spinchain
    import dmrgpy_gb300
    tag = dmrgpy_gb300.register(prec)
    out = {}
    for name, version in (("python", "python"), ("gb300", tag)):
        np.random.seed(seed)
        sc = spinchain.Spin_Chain([2] * n, itensor_version=version)
        sc.maxm = maxm
        sc.nsweeps = nsweeps
        sc.set_hamiltonian(_heisenberg(sc, n))
        out[name] = sc
    return dmrgpy, out


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "tf32x3"])
def test_spin_chain_ground_state_through_dmrgpy(prec):
    n = 10
    _, sc = _pair(n, 32, 6, prec)
    # the same seed before each run: both draw the reference's random MPS
    np.random.seed(11)
    e_py = sc["python"].gs_energy()
    np.random.seed(11)
    e_gb = sc["gb300"].gs_energy()
    assert type(sc["gb300"]._session).__name__.startswith("GB300Session")
    assert abs(e_gb - e_py) / n <= 1e-10, (e_gb, e_py)
    wf_py, wf_gb = sc["python"].get_gs(), sc["gb300"].get_gs()
    op_py = sc["python"].Sz[0] * sc["python"].Sz[n - 1]
    op_gb = sc["gb300"].Sz[0] * sc["gb300"].Sz[n - 1]
    assert abs(sc["gb300"].vev(op_gb) - sc["python"].vev(op_py)) < 1e-8
    assert abs(wf_gb.get_entropy(n // 2) - wf_py.get_entropy(n // 2)) < 1e-8


@pytest.mark.gpu
def test_real_time_evolution_through_dmrgpy():
    """evolve_and_measure (TDVP glue) and the session's tdvp_step and
    quench_tdvp against the python backend from the same ground state."""
    n = 8
    _, sc = _pair(n, 16, 6, "fp64", seed=2)
    from dmrgpy import timedependent
    for c in sc.values():
        np.random.seed(5)
        c.gs_energy()
    ts_py, cs_py = timedependent.evolve_and_measure(sc["python"], operator=sc["python"].Sz[2], nt=4, dt=0.05)
    ts_gb, cs_gb = timedependent.evolve_and_measure(sc["gb300"], operator=sc["gb300"].Sz[2], nt=4, dt=0.05)
    assert np.max(np.abs(np.asarray(cs_gb) - np.asarray(cs_py))) < 1e-8
    # one TDVP step of the session on an excited (non-stationary) state
    terms_h = sc["python"].hamiltonian.to_terms()
    terms_op = (sc["python"].Sx[3]).to_terms()
    s_py, s_gb = sc["python"]._session, sc["gb300"]._session
    H_py, H_gb = s_py.build_operator(terms_h), s_gb.build_operator(terms_h)
    phi_py = s_py.apply_operator(terms_op, s_py.gs_wavefunction())
    phi_gb = s_gb.apply_operator(terms_op, s_gb.gs_wavefunction())
    out_py = s_py.tdvp_step(H_py, phi_py, 0.1)
    out_gb = s_gb.tdvp_step(H_gb, phi_gb, 0.1)
    from dmrgpy_gb300 import session as S
    v_py = O.mps_to_dense(S.mps_to_arrays(out_py))
    v_gb = O.mps_to_dense(S.mps_to_arrays(out_gb))
    # the two ground states may differ by a sign
    ph = np.vdot(v_gb, v_py)
    ph = ph / abs(ph)
    assert np.max(np.abs(v_gb * ph - v_py)) < 1e-8
    # quench_tdvp: <gs|A_j(t) A_i|gs>-type correlator
    c_py, _ = s_py.quench_tdvp(terms_h, terms_op, terms_op, 3, 0.05)
    c_gb, _ = s_gb.quench_tdvp(terms_h, terms_op, terms_op, 3, 0.05)
    assert np.max(np.abs(np.asarray(c_gb) - np.asarray(c_py))) < 1e-8
