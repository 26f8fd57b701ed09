"""The many-chain workload at size: transverse-field Ising chains
H = -J sum_i Sz_i Sz_{i+1} + h sum_i Sx_i (N sites, open ends, J = 1), one
field h per chain drawn uniformly from [0.5, 1.5] and one bond cap per chain
drawn from {16, 32, 64, 128} (seeded), swept together by
:class:`dmrgpy_gb300.batch.BatchEngine`: every bond step of all chains is one
grouped launch per operation, the Lanczos blocks replay captured CUDA graphs.

After the sweeps, dE/dh of every chain comes from the adjoint pass
(:class:`dmrgpy_gb300.gradients.CouplingProblem`, the field terms' summed
coupling gradients) and is checked against
  * <dH/dh> = sum_i <Sx_i> measured on the state (transition contractions),
  * central finite differences (E(h + dh) - E(h - dh)) / (2 dh), dh = 1e-5,
    of batched energies swept from the converged states.

    python -m dmrgpy_gb300.batch_workload --chains 256 --n 64 --sweeps 8

Prints one JSON line per sweep (seconds, energy per site range), then one
summary line: seconds per lock-step sweep, bond updates per second, the
energy per site range and the largest disagreements of the gradients.

Measured on one GB300 (`--sweeps 2 --no-gradients`): 9.6 s for the first
lock-step sweep and 12.4 s for the second (bonds at their caps), i.e. 2,600
bond updates per second over the 256 chains, ~95 ms per bond step of all
chains.  The likely bound of a bond step: the batched truncation factorises
each chain's two-site tensor with the one-CTA FP64 Jacobi SVD, which at a
bond cap of 128 (256 x 256 tensors) runs on a single SM's FP64 pipe.  The
full run with gradients (8 sweeps, 256 adjoint passes driven chain by chain
from the host, 2 x 3 finite-difference sweeps) did not finish within 480 s;
its parts were not timed separately.
"""
import argparse
import json
import time

import numpy as np

from . import mpo as _mpo


def tfim_terms(n, J, h):
    t = [(complex(-J), [("Sz", i), ("Sz", i + 1)]) for i in range(1, n)]
    return t + [(complex(h), [("Sx", i)]) for i in range(1, n + 1)]


def _batch(n, hs):
    from .batch import BatchEngine
    Ws = [_mpo.build_mpo([2] * n, tfim_terms(n, 1.0, h))[0] for h in hs]
    return BatchEngine(Ws, real=True)


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--chains", type=int, default=256)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--sweeps", type=int, default=8)
    ap.add_argument("--fd-sweeps", type=int, default=3)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--no-gradients", action="store_true", help="sweeps only (no adjoint or finite differences)")
    args = ap.parse_args(argv)
    n, C = args.n, args.chains
    rng = np.random.default_rng(args.seed)
    hs = rng.uniform(0.5, 1.5, C)
    chis = [int(c) for c in rng.choice([16, 32, 64, 128], C)]

    be = _batch(n, hs)
    As = be.random_states([2] * n, 4, seeds=[1000 + p for p in range(C)])
    be.canonicalize(As)
    torch.cuda.synchronize()
    times = []
    renv = None
    energies = None
    for sw in range(args.sweeps):
        t0 = time.perf_counter()
        energies, renv = be.sweep(As, chis, 0.0, renv)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
        e = np.asarray(energies, dtype=np.float64) / n
        # one progress line per sweep, so that a run cut short still reports
        print(json.dumps({"sweep": sw + 1, "s": times[-1], "energy_per_site_min": float(e.min()),
                          "energy_per_site_max": float(e.max())}), flush=True)
    energies = np.asarray(energies, dtype=np.float64)
    out = {
        "workload": "%d TFIM chains, N=%d, J=1, h~U[0.5,1.5], chi_max~{16,32,64,128}, batched two-site DMRG "
                    "(grouped launches, graph-replayed Lanczos), FP64" % (C, n),
        "sweeps": args.sweeps,
        "s_per_sweep_last": times[-1],
        "s_per_sweep_first": times[0],
        "bond_updates_per_s": C * 2 * (n - 1) / times[-1],
        "energy_per_site_min": float((energies / n).min()),
        "energy_per_site_max": float((energies / n).max()),
    }
    if args.no_gradients:
        print(json.dumps(out))
        return

    # dE/dh by the adjoint pass, and <dH/dh> = sum_i <Sx_i> on the state
    from .engine import Engine
    from .gradients import CouplingProblem
    prob = CouplingProblem([2] * n, tfim_terms(n, 1.0, hs[0]))
    Wsx, _ = _mpo.build_mpo([2] * n, [(1.0 + 0j, [("Sx", i)]) for i in range(1, n + 1)])
    meas = Engine(Wsx, real=True)
    ident = meas.identity_mpo([2] * n)
    t0 = time.perf_counter()
    dedh = np.zeros(C)
    sx = np.zeros(C)
    for p in range(C):
        prob.set_coefs([c for c, _ in tfim_terms(n, 1.0, hs[p])])
        _, g = prob.gradient(As[p])
        dedh[p] = float(np.sum(g[-n:]).real)
        norm = meas.transition(ident, As[p], As[p]).real
        sx[p] = float(meas.transition(meas.W, As[p], As[p]).real / norm)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0

    # central finite differences of batched energies, swept from the
    # converged states with the shifted fields
    dh = 1e-5
    e_pm = []
    for sgn in (1.0, -1.0):
        bs = _batch(n, hs + sgn * dh)
        Bs = [[a.clone() for a in A] for A in As]
        e_pm.append(np.asarray(bs.dmrg(Bs, chis, args.fd_sweeps), dtype=np.float64))
        del Bs, bs
    fd = (e_pm[0] - e_pm[1]) / (2 * dh)

    scale = np.maximum(1.0, np.abs(dedh))
    out.update({
        "gradient_s": t_grad,
        "max_rel_adjoint_vs_expectation": float(np.max(np.abs(dedh - sx) / scale)),
        "max_rel_adjoint_vs_fd": float(np.max(np.abs(dedh - fd) / scale)),
        "median_rel_adjoint_vs_fd": float(np.median(np.abs(dedh - fd) / scale)),
        "fd_dh": dh,
        "fd_sweeps": args.fd_sweeps,
    })
    print(json.dumps(out))


if __name__ == "__main__":
    main()
