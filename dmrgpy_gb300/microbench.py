"""Time one sweep kernel in isolation on seeded random operands.

    python -m dmrgpy_gb300.microbench --op heff2 --chi 1024 --d 3 --w 5 --precision tf32x3

Ops: heff2 (two-site H_eff matvec, per Krylov iteration: prepared operands),
env (left environment extension), subspace (fixed-rank truncation of a
(chi d) x (d chi) two-site tensor), svd (FP64 one-sided Jacobi truncation),
merge (two-site merge GEMM), gram / gram64 (X^T X of a (chi d) x chi
block by exact digit products on the tensor cores / in FP64 on the CUDA
cores).  Prints one JSON line with the mean time per
call (CUDA events on the launching stream, after warm-up) and the
algorithmic FLOP rate.  Used to pick bond dimensions and to give profilers a
small, self-contained target.
"""
import argparse
import ctypes
import json

from . import _lib
from . import mpo as M
from .engine import Engine


def _heisenberg(n):
    return [(1.0 + 0j, [(op, i), (op, i + 1)]) for i in range(1, n) for op in ("Sx", "Sy", "Sz")]


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="heff2", choices=["heff2", "env", "subspace", "svd", "merge", "gram", "gram64"])
    ap.add_argument("--chi", type=int, default=1024)
    ap.add_argument("--d", type=int, default=3)
    ap.add_argument("--precision", default="tf32x3", choices=["fp64", "tf32x3"])
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    args = ap.parse_args(argv)
    code = {2: 2, 3: 3}.get(args.d, 3)
    W, real = M.build_mpo([code] * 6, _heisenberg(6))
    eng = Engine(W, real=True, precision=args.precision)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    chi, d = args.chi, W[2].shape[1]
    w = W[2].shape[0]
    dev = eng.device

    def rnd(*shape):
        return torch.randn(*shape, dtype=torch.float64, device=dev, generator=g)

    L, R = rnd(chi, w, chi), rnd(chi, w, chi)
    theta = rnd(chi, d, d, chi)
    A = rnd(chi, d, chi)
    s = torch.cuda.current_stream()
    if args.op == "heff2":
        h = eng.heff2(L, eng.W[2], eng.W[3], R, theta.shape)
        y = torch.empty_like(theta)
        need = eng.lib.dmrg_heff_workspace_bytes(ctypes.byref(h))
        ptr, size = eng.ws.get(need)
        _lib.check("dmrg_heff_prepare", eng.lib.dmrg_heff_prepare(ctypes.byref(h), ptr, size, eng.stream))

        def call():
            eng.lib.dmrg_heff_apply_prepared(ctypes.byref(h), theta.data_ptr(), y.data_ptr(), ptr, size, eng.stream)
        flops = Engine.heff2_flops(chi, d, d, chi, w, w, w)
    elif args.op == "env":
        def call():
            eng.env_left(L, eng.W[2], A)
        flops = 2.0 * (2.0 * chi ** 3 * d * w + chi ** 2 * d * d * w * w)
    elif args.op == "subspace":
        m = chi * d
        M2 = theta.reshape(m, m)

        # no warm start: the library draws and orthonormalises the start
        # basis itself (the first sweep's case; warm-started calls in a
        # converged sweep skip that orthonormalisation)
        def call():
            eng.subspace_split(M2, chi, None, 0, 0)
        flops = 2.0 * 3 * m * m * chi
    elif args.op in ("gram", "gram64"):
        m = chi * d
        X = rnd(m, chi)
        G = torch.empty((chi, chi), dtype=torch.float64, device=dev)
        method = _lib.GRAM_DIGITS if args.op == "gram" else _lib.GRAM_FP64
        need = eng.lib.dmrg_gram_workspace_bytes(method, m, chi)
        gptr, gsize = eng.ws.get(max(need, 1))

        def call():
            _lib.check("dmrg_gram", eng.lib.dmrg_gram(method, m, chi, X.data_ptr(), chi, G.data_ptr(), gptr,
                                                      gsize, eng.stream))
        flops = 1.0 * m * chi * chi   # the symmetric half
    elif args.op == "svd":
        m = chi * d
        M2 = theta.reshape(m, m)

        def call():
            eng.svd(M2, 0.0, chi, 1, 0)
        flops = 0.0
    else:
        def call():
            eng.merge(A, A)
        flops = 2.0 * (chi * d) * chi * (d * chi)
    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # the NVTX range lets a profiler skip the warm-up (and first-call tuning)
    # launches: ncu --nvtx --nvtx-include "timed/"
    torch.cuda.nvtx.range_push("timed")
    e0.record(s)
    for _ in range(args.reps):
        call()
    e1.record(s)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / args.reps
    if args.op == "heff2":
        _lib.check("dmrg_heff_status", eng.lib.dmrg_heff_status(ctypes.byref(h), ptr, size, eng.stream))
    print(json.dumps({"op": args.op, "chi": chi, "d": d, "w": w, "precision": args.precision, "s_per_call": t,
                      "tflops": flops / t / 1e12 if flops else None}))


if __name__ == "__main__":
    main()
