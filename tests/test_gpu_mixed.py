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
