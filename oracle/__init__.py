"""CPU oracle for the two-site DMRG/TDVP sweep -- test infrastructure only.

This package restates, in plain NumPy, the algorithm of dmrgpy's pure-Python
backend (``src/dmrgpy/pyitensor``) for the hot path: the two-site effective
Hamiltonian matvec, the Lanczos ground-state solver, the Gram-route truncated
SVD, the environment extensions, the sweep driver, TDVP with the Krylov
exponential, the random initial MPS and the term -> MPO compiler.  Each
function cites the reference file:line it follows.

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import it, and only as the checker / the timed CPU baseline.
The GPU product path (``dmrgpy_gb300``) never imports it.

Parity pins: ``tests/golden/*.npz`` were produced by running the reference
itself (``tests/golden/make_golden.py``); ``tests/test_oracle_golden.py``
checks this package against them and against the reference test-suite's own
golden energies (``tests/reference_data.py``, ``tests/test_spin_chain.py``).
"""

from .dmrg_oracle import *  # noqa: F401,F403
