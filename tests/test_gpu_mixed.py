"""Split-TF32 sweep + FP64 refinement against the FP64 GPU sweep from the
same seeded initial state (S=1 Heisenberg, chi up to 128, cutoff 0 so the
maxdim-bound subspace truncation is exercised).  Bar: |dE|/N <= 1e-10 after
refinement, the same bar the FP64 path meets against the reference."""
import numpy as np
import pytest

from golden_data import terms_heisenberg

pytestmark = pytest.mark.gpu


def _run(precision, n, schedule, seed):
    from dmrgpy_gb300 import mpo as M
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.engine import Engine
    W, real = M.build_mpo([3] * n, terms_heisenberg(n))
    eng = Engine(W, real=real, precision=precision)
    np.random.seed(seed)
    A = eng.to_device(MP.random_arrays([3] * n, schedule[0]))
    eng.canonicalize_right_to_left_of(A)
    e = eng.dmrg(A, schedule, 0.0, 2)
    return e, eng.energy_fp64(A), eng


def test_tf32x3_sweep_matches_fp64_sweep_after_refinement():
    n = 24
    schedule = [32, 64] + [128] * 10
    e64, e64_ref, _ = _run("fp64", n, schedule, 11)
    e32, e32_ref, eng = _run("tf32x3", n, schedule, 11)
    # the FP64 sweep's last Ritz value and its own refined energy agree
    assert abs(e64 - e64_ref) / n < 1e-11
    # the split-TF32 sweep lands on the same variational energy after the FP64 refinement
    assert abs(e32_ref - e64_ref) / n <= 1e-10, (e32_ref, e64_ref)
    # and the unrefined TF32 Ritz value is FP32-accurate
    assert abs(e32 - e64_ref) / abs(e64_ref) < 1e-5


def _hubbard_terms(n, t=1.0, u=4.0):
    """Spinful Hubbard chain, particle-hole symmetric (half filling without
    quantum numbers): -t sum (c+_i c_i+1 + h.c.) + U sum n_up n_dn - U/2 sum n."""
    out = []
    for i in range(1, n):
        for s in ("up", "dn"):
            out.append((complex(-t), [("Cdag" + s, i), ("C" + s, i + 1)]))
            out.append((complex(-t), [("Cdag" + s, i + 1), ("C" + s, i)]))
    for i in range(1, n + 1):
        out.append((complex(u), [("Nup", i), ("Ndn", i)]))
        out.append((complex(-u / 2), [("Nup", i)]))
        out.append((complex(-u / 2), [("Ndn", i)]))
    return out


def test_tf32x3_hubbard_energy_and_double_occupancy():
    """Config 3 (spinful Hubbard, d=4, w=6) at a reduced size: the split-TF32
    sweep + FP64 refinement against the FP64 sweep from the same state,
    energy per site and the double-occupancy profile <n_up n_dn>_i (read off
    the adjoint pass as the derivative with respect to each U term)."""
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.engine import Engine
    from dmrgpy_gb300.gradients import CouplingProblem
    n = 12
    terms = _hubbard_terms(n)
    schedule = [16, 32] + [64] * 8
    res = {}
    for prec in ("fp64", "tf32x3"):
        prob = CouplingProblem([1] * n, terms, precision=prec)
        eng = prob.engine
        np.random.seed(7)
        A = eng.to_device(MP.random_arrays([4] * n, 16))
        eng.canonicalize_right_to_left_of(A)
        eng.dmrg(A, schedule, 0.0, 2)
        e = eng.energy_fp64(A)
        _, g = prob.gradient(A)
        docc = np.array([g[k].real for k, (c, f) in enumerate(terms) if len(f) == 2 and f[0][0] == "Nup"])
        res[prec] = (e, docc)
    e64, d64 = res["fp64"]
    e32, d32 = res["tf32x3"]
    assert abs(e32 - e64) / n <= 1e-9, (e32, e64)
    assert np.max(np.abs(d32 - d64)) < 1e-5, np.max(np.abs(d32 - d64))
    assert np.all((d64 > 0) & (d64 < 0.25))
