"""Benchmark of the GB300 two-site DMRG sweep.

Workload (the headline configuration): S=1 Heisenberg chain, N=100 sites,
d=3, MPO bond dimension w=5, J=1, open boundaries; seeded random initial MPS
(chi=64); two-site DMRG with the bond dimension ramped 64 -> 256 -> 1024 and
cutoff 0 so that every bulk bond carries chi=1024.  One step = one full
two-site sweep (left-to-right then right-to-left, 198 bond updates) at
chi=1024 with split-TF32 contractions, FP64 Lanczos reductions and an FP64
refinement of the energy at the end (not timed per step).  Data are
synthetic (no dataset); the working set (environments ~4 GB, MPS ~2.5 GB)
is far larger than L2, so no explicit L2 flush is needed.

JSON line keys beyond the common contract:
  roofline     the split-TF32 H_eff matvec at a chi=1024 bond, timed with
               CUDA events on the launching stream;
  cpu_baseline the CPU oracle (NumPy restatement of the reference sweep)
               on the host cores, one bond at chi=1024;
  sweep        per-phase seconds, Lanczos iterations, refined energy and
               the end-spin correlator <S^z_1 S^z_N>;
  fp64_gpu     one measured FP64 GPU sweep at chi=1024 from the split-TF32
               state: seconds, refined energy, |dE|/N and the correlator
               difference against the split-TF32 state;
  e2e          one sweep through dmrgpy_gb300.Chain with the MPS in host
               memory before and after.

--impl reference runs the oracle on the host cores instead (one bond update
of the same workload per step).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sweep s & H_eff TFLOP/s at χ=1024: split-TF32+refine vs FP64 GPU, |ΔE|/N≤1e-10"
N_SITES = 100
CHI = 1024
D = 3


def terms_heisenberg(n):
    return [(1.0 + 0j, [(op, i), (op, i + 1)]) for i in range(1, n) for op in ("Sx", "Sy", "Sz")]


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), float(d["hbm_gbs"]), "measured"
    except Exception:
        return 1900.0, 6800.0, "fallback"


def profile_summary():
    """DRAM bytes per matvec and the per-kernel ncu figures (time share,
    tensor-pipe utilisation) from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "heff_tf32x3_chi1024.json")
    try:
        with open(p) as f:
            d = json.load(f)
    except Exception:
        return None, None
    ks = d.get("kernels") or []
    tot = sum(k.get("us", 0.0) for k in ks) or 1.0
    kernels = [{"kernel": k.get("kernel"), "us": k.get("us"), "share": k.get("us", 0.0) / tot,
                "tensor_pipe_pct": k.get("tensor"), "dram_pct": k.get("dram")} for k in ks]
    return d.get("dram_bytes_per_matvec"), kernels


# ---------------------------------------------------------------- CPU oracle sample
def max_over_ranks(value, dist, device):
    """The largest of the ranks' values (the job's time is that of its
    slowest replica); the value itself in a single process."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, dist, device):
    """The sum of the ranks' values (the work of all replicas: they run
    different seeds, so their Lanczos counts differ)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count()


def reference_bond_step(L, Wi, Wj, R, theta, A, k, maxdim):
    """One chi=1024 bond update of the reference algorithm on the host with
    the oracle (NumPy complex128, as the reference computes): k H_eff
    matvecs (each one run and timed, the Krylov count of the GPU sweep),
    the truncated SVD and one environment extension; the wall time of the
    whole step is measured."""
    import numpy as np
    import oracle as O
    t0 = time.perf_counter()
    x = theta
    t_mv = []
    for _ in range(k):
        a = time.perf_counter()
        y = O.heff2_matvec(L, Wi, Wj, R, x)
        t_mv.append(time.perf_counter() - a)
        x = y / np.linalg.norm(y)
    cl, d1, d2, cr = theta.shape
    a = time.perf_counter()
    O.svd_truncated(x.reshape(cl * d1, d2 * cr), 0.0, maxdim, 1)
    t_svd = time.perf_counter() - a
    a = time.perf_counter()
    O.extend_left(L, Wi, A)
    t_env = time.perf_counter() - a
    return {"t_matvecs": t_mv, "t_svd": t_svd, "t_env": t_env, "t_step": time.perf_counter() - t0}


def run_reference(args):
    """--impl reference: the oracle restatement of the reference sweep on
    the host cores.  A step is one bond update of the headline workload at
    chi=1024 (S=1 Heisenberg, d=3, the MPO from the oracle's own builder,
    seeded random environments and two-site tensor of the chi=1024 shapes):
    3 matvecs (the mean Lanczos count of the GPU sweep at this bond size),
    the truncated SVD and an environment extension, timed as one wall-clock
    step.  A full sweep is 198 such steps."""
    import numpy as np
    import oracle as O
    from dmrgpy_gb300.engine import Engine
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    W = O.build_mpo([3] * 6, terms_heisenberg(6))
    Wi, Wj = W[2], W[3]
    rng = np.random.default_rng(0)
    w = Wi.shape[0]
    c = np.complex128
    L = rng.standard_normal((CHI, w, CHI)).astype(c)
    R = rng.standard_normal((CHI, w, CHI)).astype(c)
    th = rng.standard_normal((CHI, D, D, CHI)).astype(c)
    A = rng.standard_normal((CHI, D, CHI)).astype(c)
    k = 3
    flops = Engine.heff2_flops(CHI, D, D, CHI, w, Wi.shape[3], Wj.shape[3], complex_=False)
    for _ in range(args.warmup):
        reference_bond_step(L, Wi, Wj, R, th, A, 1, CHI)
    tot, res = 0.0, None
    for _ in range(args.steps):
        res = reference_bond_step(L, Wi, Wj, R, th, A, k, CHI)
        tot += res["t_step"]
    value = k * flops * args.steps / tot / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic: seeded random chi=1024 environments and two-site tensor",
            "config": {"workload": "S=1 Heisenberg N=100 d=3 w=5 chi=1024: one bond update per step "
                                   "(198 per sweep)", "parallelism": "host"},
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": host_cores(), "kind": "port",
                             "sample": "one chi=1024 bond update of the oracle (NumPy complex128 like the "
                                       "reference): %d matvecs, each run, + truncated SVD + environment "
                                       "extension, wall time per step" % k},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "components_s": res, "sweep_s_equivalent": 198 * tot / args.steps}
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import numpy as np
    import torch
    from dmrgpy_gb300 import _lib
    from dmrgpy_gb300 import mpo as M
    from dmrgpy_gb300 import mps as MP
    from dmrgpy_gb300.engine import Engine, SweepStats

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl")
        dist = dist_mod
    lib = _lib.load()
    W, real = M.build_mpo([3] * N_SITES, terms_heisenberg(N_SITES))
    eng = Engine(W, real=real, precision="tf32x3", device="cuda:%d" % local)
    np.random.seed(1234 + rank)
    A = eng.to_device(MP.random_arrays([D] * N_SITES, 64))
    eng.canonicalize_right_to_left_of(A)
    # ramp (not timed): chi 64 -> 256, then the warm-up steps at chi=1024
    t_ramp = time.perf_counter()
    for chi in (64, 256):
        eng.sweep(A, chi, 0.0, 2)
    for _ in range(args.warmup):
        eng.sweep(A, CHI, 0.0, 2)
    torch.cuda.synchronize()
    t_ramp = time.perf_counter() - t_ramp
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    eng.stats = SweepStats()
    clocks = ClockSampler()
    clocks.start()
    l0 = lib.dmrg_kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    # the NVTX range lets a profiler restrict itself to the timed sweeps
    # (ncu --nvtx --nvtx-include "timed_sweeps/")
    torch.cuda.nvtx.range_push("timed_sweeps")
    ev0.record()
    energy = None
    for _ in range(args.steps):
        energy = eng.sweep(A, CHI, 0.0, 2, record=True)
    ev1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    launches = lib.dmrg_kernel_launches() - l0
    clk = clocks.stop()
    t_dev = ev0.elapsed_time(ev1) / 1e3
    dev = "cuda:%d" % local
    elapsed = max_over_ranks(max(t_dev, 0.0), dist, dev)
    st = eng.stats
    flops = sum_over_ranks(st.matvec_flops, dist, dev)
    value = flops / elapsed / 1e12
    iters = [r["iters"] for r in st.records]
    chis = [max(r["chil"], r["chir"]) for r in st.records]

    # --- roofline of the split-TF32 matvec at the middle bond (chi=1024)
    mid = N_SITES // 2
    renv = eng.right_envs(A)
    lenv = eng.left_envs(A[:mid + 1])
    theta = eng.merge(A[mid - 1], A[mid]).contiguous()
    h = eng.heff2(lenv[mid - 1], eng.W[mid - 1], eng.W[mid], renv[mid + 2], theta.shape)
    y = eng.apply(h, theta)
    cl, d1, d2, cr = theta.shape
    f_mv = Engine.heff2_flops(cl, d1, d2, cr, h.wl, h.wm, h.wr)
    need = lib.dmrg_heff_workspace_bytes(h)
    ptr, size = eng.ws.get(need)
    import ctypes
    reps = 20
    # prepare once (operand split), then time the per-iteration matvec
    from dmrgpy_gb300._lib import check
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    check("dmrg_heff_prepare", lib.dmrg_heff_prepare(ctypes.byref(h), ptr, size, eng.stream))
    for _ in range(3):
        check("dmrg_heff_apply_prepared", lib.dmrg_heff_apply_prepared(ctypes.byref(h), theta.data_ptr(),
                                                                       y.data_ptr(), ptr, size, eng.stream))
    torch.cuda.synchronize()
    s0.record()
    for _ in range(reps):
        lib.dmrg_heff_apply_prepared(ctypes.byref(h), theta.data_ptr(), y.data_ptr(), ptr, size, eng.stream)
    s1.record()
    torch.cuda.synchronize()
    check("dmrg_heff_status", lib.dmrg_heff_status(ctypes.byref(h), ptr, size, eng.stream))
    t_mv = s0.elapsed_time(s1) / 1e3 / reps
    bf16, hbm, peak_kind = measured_peaks()
    achieved = f_mv / t_mv / 1e12
    traffic, ncu_kernels = profile_summary()
    roof = {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16,
            "traffic": traffic, "peak_source": peak_kind, "ncu_kernels": ncu_kernels,
            "kernel": "two-site H_eff matvec per Krylov iteration (split-TF32 tcgen05 GEMMs + MPO step), "
                      "chi=1024 d=3 w=5",
            "flops_per_launch": f_mv, "launch_s": t_mv,
            "tf32x3_ceiling_tflops": bf16 / 2.0 / 3.0,
            "frac_of_tf32x3_ceiling": achieved / (bf16 / 2.0 / 3.0)}

    # --- FP64 refinement of the energy of the split-TF32 state (not in the
    # timed steps) and the end-spin correlator, both on the device
    t0 = time.perf_counter()
    e_ref = eng.energy_fp64(A)
    t_refine = time.perf_counter() - t0
    Wc, _ = M.build_mpo([3] * N_SITES, [(1.0 + 0j, [("Sz", 1), ("Sz", N_SITES)])])
    corr_eng = Engine(Wc, real=True, precision="fp64", device="cuda:%d" % local)
    szsz32 = corr_eng.energy_fp64(A)

    # --- the FP64 GPU path (the metric's comparison), measured: one full FP64
    # sweep at chi=1024 continuing from the split-TF32 state (right
    # environments rebuilt in FP64 first, not timed), its refined energy and
    # correlator; |dE|/N compares the two refined energies
    fp64 = None
    if not args.no_fp64:
        e64 = Engine(W, real=real, precision="fp64", device="cuda:%d" % local)
        A64 = [a.clone() for a in A]
        e64._renv = e64.right_envs(A64)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        f0.record()
        e64_last = e64.sweep(A64, CHI, 0.0, 2, record=True)
        f1.record()
        torch.cuda.synchronize()
        t64 = f0.elapsed_time(f1) / 1e3
        w64 = time.perf_counter() - w0
        e64_ref = e64.energy_fp64(A64)
        szsz64 = corr_eng.energy_fp64(A64)
        it64 = [r["iters"] for r in e64.stats.records]
        fp64 = {"sweep_s": t64, "wall_s": w64, "phase_s": dict(e64.stats.t),
                "matvecs": e64.stats.matvecs, "lanczos_iters_mean": float(np.mean(it64)) if it64 else None,
                "energy_last_bond": e64_last, "energy_refined": e64_ref,
                "abs_dE_per_site": abs(e_ref - e64_ref) / N_SITES,
                "szsz_1N": szsz64, "abs_d_szsz_1N": abs(szsz32 - szsz64),
                "speedup_sweep": t64 / (elapsed / args.steps),
                "note": "one measured FP64 GPU sweep at chi=1024 (FP64 matvecs, FP64 subspace + Rayleigh-Ritz "
                        "truncation, FP64 environments) from the split-TF32 state; |dE|/N = |E_refined(split-TF32 "
                        "state) - E_refined(FP64-swept state)| / N"}
        del e64, A64

    # --- end-to-end through the public session API (dmrgpy_gb300.Chain, the
    # object dmrgpy's glue drives): the MPS handed over from host memory,
    # the MPO compiled, one split-TF32 sweep at chi=1024, the MPS back on
    # the host
    from dmrgpy_gb300 import Chain
    host = eng.to_host(A)
    h2d = sum(a.nbytes for a in host)
    chain = Chain([3] * N_SITES, precision="tf32x3")
    chain.set_sweep_params(CHI, 1, 0.0, 0.0)
    chain.set_hamiltonian(terms_heisenberg(N_SITES))
    chain.set_wavefunction(MP.MPS(host, center=1))
    del host
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_chain = chain.gs_energy()
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    d2h = sum(a.nbytes for a in chain.gs_wavefunction().tensors)
    e2e = {"value": chain.last_stats.matvec_flops / t_e2e / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "sweep_s": t_e2e, "energy_last_bond": e_chain,
           "note": "Chain(precision='tf32x3'): set_wavefunction(host MPS) + gs_energy() with one sweep at "
                   "chi=1024: MPO compile, MPS host->device, right environments, the sweep, MPS device->host"}
    del chain

    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3/f64",
            "data": "synthetic: seeded random initial MPS, no dataset",
            "config": {"workload": "S=1 Heisenberg N=100 d=3 w=5 J=1 OBC two-site DMRG sweep, chi=1024 "
                                   "(ramp 64->256->1024, cutoff 0), split-TF32 + FP64 refine",
                       "chi": CHI, "n_sites": N_SITES, "d": D, "w": 5, "l2": "working set >> L2 (no flush)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "clocks": clk, "gpu_launches": int(launches), "e2e": e2e, "roofline": roof, "fp64_gpu": fp64,
            "sweep": {"sweep_s": elapsed / args.steps, "wall_s": t_wall / args.steps,
                      "phase_s": {k: v / args.steps for k, v in st.t.items()},
                      "matvecs_per_sweep": st.matvecs / args.steps,
                      "lanczos_iters_mean": float(np.mean(iters)) if iters else None,
                      "chi_max": max(chis) if chis else None,
                      "energy_last_bond_tf32": energy, "energy_refined_fp64": e_ref,
                      "energy_per_site": e_ref / N_SITES, "refine_s": t_refine, "szsz_1N": szsz32,
                      "schedule_s_before_timed": t_ramp}}
    if rank == 0 and not args.no_cpu:
        k_mean = int(round(np.mean(iters))) if iters else 10
        Lh = lenv[mid - 1].cpu().numpy()
        Rh = renv[mid + 2].cpu().numpy()
        thh = theta.cpu().numpy()
        Ah = A[mid - 1].cpu().numpy()
        c = np.complex128
        res = reference_bond_step(Lh.astype(c), W[mid - 1].astype(c), W[mid].astype(c), Rh.astype(c),
                                  thh.astype(c), Ah.astype(c), k_mean, CHI)
        cpu_val = k_mean * f_mv / res["t_step"] / 1e12
        line["cpu_baseline"] = {"value": cpu_val, "unit": "TFLOP/s", "cores": host_cores(), "kind": "port",
                                "sample": "one chi=1024 bond update of this state on the host: oracle NumPy "
                                          "(complex128 like the reference), %d matvecs (the mean Lanczos count "
                                          "of the GPU sweep), each run, + truncated SVD + env extension, wall "
                                          "time" % k_mean,
                                "components_s": res, "sweep_s_equivalent": 198 * res["t_step"]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle sample")
    ap.add_argument("--no-fp64", action="store_true", help="skip the measured FP64 GPU sweep")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
