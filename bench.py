#!/usr/bin/env python
"""Benchmark: FP64 APGD time to residual 1e-6 on the 200 000-contact friction problem, on one GB300.

Workload (one "step"): DualFrictionProblem::solveWith(ProjectedGradient, r) with the reference's defaults
(APGD, SOC law, line search 8 / 1.25 / 0.5) at tol 1e-6, from r = 0, on the seeded grid problem (50 000 rigid
bodies, 200 000 contacts, W assembled on the GPU), with an iteration budget (20 000) that the solve does not
reach: it stops at the tolerance (7 846 iterations on this problem). The GPU and the CPU oracle run
bit-identical iterations, so both arms do the same work.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--no-secondary]

Our arm prints `value` (ms per solve, inputs resident in HBM, CUDA events on the library's stream), `e2e`
(the C-ABI call with host buffers: upload of W/b/mu/r, solve, download of r), the roofline of the
persistent solver kernel, FP64 pipe use, the CPU baseline (the oracle on the host cores, on a bounded sample:
the first 1000 iterations of the same solve, scaled to the full solve's iteration count) and `secondary`: the
other measured targets (500-iteration cap, FP32-refined time to 1e-6 and its error against the FP64 result,
SPG, colored Gauss-Seidel, the 4096-problem batch against a loop of single solves, adjoint / forward).
`--impl reference` times the CPU restatement of the reference (the oracle, OpenMP on all host cores) on the
same workload: one full solve to calibrate the iteration count, then bounded samples. With N > 1 (torchrun)
every rank solves its own replica (a single problem does not shard); `--workload batch|adjoint` shards the
independent problems of those batches over the ranks instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(REPO, "so-bogus_gb300")]

TOL = 1e-6
MAX_ITERS = 20_000        # budget of the time-to-residual solve; APGD reaches 1e-6 well before it here
CAP_500 = 500             # the iteration budget of the configuration's wording, reported beside the headline
CPU_SAMPLE_ITERS = 1000   # the oracle's bounded sample: the first 1000 iterations of the same solve
FP32_ITERS = 20000        # FP32-refined: FP32 iterations until the stall test ends them (at most this many),
                          # then FP64 ones to the tolerance
HY_REFRESH = 50           # FP32 correction products in those FP64 iterations: x_ref refreshed this often
BATCH_HY_REFRESH = 5      # the same in the 4096-problem batch (its 300 FP64 iterations leave no room for a floor)
MAX_ADJ_FWD_ITERS = 20000
METRIC = "time-to-residual 1e-6 (ms), FP64 APGD, 200k contacts"
WORKLOAD = "fp64_apgd_200k_contacts_to_1e-6"


def config_dict(n, nnzb_full, max_iters, extra=None):
    d = {"workload": WORKLOAD, "contacts": n, "bodies": 50_000, "w_blocks_full": nnzb_full,
         "w_blocks_lower": (nnzb_full + n) // 2, "solver": "APGD (reference defaults), SOC law",
         "tol": TOL, "max_iters": max_iters, "start": "r = 0", "generator": "grid, seed 1",
         "l2": "inputs exceed L2 (W both triangles = %.0f MB > 129 MB)" % (nnzb_full * 76 / 1e6),
         "parallelism": "replicas (one problem per GPU)"}
    if extra:
        d.update(extra)
    return d


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profiles(algorithmic_bytes):
    """DRAM bytes of the solver launch: the ncu capture of the same kernel on the same problem (a solve capped at
    20 iterations, committed summary) gives DRAM bytes per algorithmic byte; traffic grows with the passes over
    W, so the launch's traffic is that ratio times its algorithmic bytes. None when the summary is absent."""
    p = os.path.join(REPO, "profiles", "pg_persistent_apgd_200k.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_algorithmic_byte:"):
            try:
                return float(line.split(":", 1)[1].strip()) * algorithmic_bytes
            except ValueError:
                return None
    return None


def pinned_copy(a, keep: list):
    """A copy of the host array `a` in page-locked memory (torch's pinned allocator); `keep` holds the buffer."""
    import torch

    t = torch.empty(max(1, a.nbytes), dtype=torch.uint8, pin_memory=True)
    keep.append(t)
    p = t.numpy()[: a.nbytes].view(a.dtype).reshape(a.shape)
    p[...] = a
    return p


def max_over_ranks(value: float, world: int, device: str = "cpu") -> float:
    """The maximum of a per-rank value over all ranks (every rank gets it); the value itself when world == 1.
    The tensor lives on `device` (a CUDA device under NCCL, the CPU under gloo)."""
    if world <= 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def make_problem():
    from bogus_gpu import generator

    return generator.make("c2")


# --------------------------------------------------------------------------------------------------------
class OracleSolve:
    """The oracle (CPU restatement of the reference) on the benchmark problem, OpenMP on all host cores."""

    def __init__(self, d, lower=None):
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import pyoracle

        pyoracle.build()
        self.po = pyoracle
        self.d = d
        if lower is None:
            P = pyoracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
            lower = P.assemble()
        self.lower = lower
        rp, cl, vl = lower
        self.O = pyoracle.DualProblem(rp, cl, np.asarray(vl).reshape(-1), d.b, d.mu)

    def solve(self, max_iters):
        """APGD from r = 0 with the benchmark's tolerance: (ms, residual, r, iterations)."""
        t0 = time.perf_counter()
        res, r, it = self.O.solve_pg(np.zeros(3 * self.d.n), variant=3, coulomb=False, tol=TOL, max_iters=max_iters)
        return (time.perf_counter() - t0) * 1e3, res, r, it

    @property
    def cores(self):
        return self.po.num_threads()


def run_reference(args, rank, world):
    """The reference arm: the oracle on all host cores. The first warm-up step solves to the tolerance once (the
    full solve's iteration count and time); every other step is a bounded sample of the same solve, its first
    CPU_SAMPLE_ITERS iterations, scaled by the full solve's iteration count."""
    if world > 1 and rank != 0:
        return
    d = make_problem()
    orc = OracleSolve(d)
    full_ms, full_res, _, full_it = orc.solve(args.max_iters)  # calibration (untimed)
    sample_iters = min(CPU_SAMPLE_ITERS, args.max_iters)
    times = []
    for step in range(max(0, args.warmup - 1) + args.steps):
        ms, _, _, it = orc.solve(sample_iters)
        if step >= max(0, args.warmup - 1):
            times.append(ms * full_it / max(1, it))
    v = statistics.mean(times)
    nnz_full = 2 * len(orc.lower[1]) - d.n
    sample = (f"first {sample_iters} APGD iterations of the same solve per step, scaled to the full solve's "
              f"{full_it} iterations; one full solve measured {full_ms:.0f} ms")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded grid generator)",
        "config": config_dict(d.n, nnz_full, args.max_iters, {"iterations": full_it, "final_residual": full_res,
                                              "reached_tol": bool(full_res < TOL)}),
        "cpu_baseline": {"value": v, "unit": "ms", "cores": orc.cores, "kind": "port", "sample": sample,
                         "full_solve_ms": full_ms},
        "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------------------------------
def run_ours(args, rank, world, local_rank):
    import torch

    import bogus_gpu

    torch.cuda.set_device(local_rank)
    dev = local_rank
    d = make_problem()
    D = bogus_gpu.DualFrictionProblem(dev)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    asm = D.solve_stats()
    n = d.n
    nnz_full = D.nnzb()
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(args.max_iters)
    r = torch.zeros(3 * n, dtype=torch.float64, device=f"cuda:{dev}")
    stream = torch.cuda.ExternalStream(D.stream(), device=f"cuda:{dev}")

    def step():
        with torch.cuda.stream(stream):
            r.zero_()
        return D.solve_pg_device(pg, r.data_ptr(), staticProblem=True)

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    kernel_ms, bytes_, fmas, iters, res = [], [], [], [], []
    with torch.cuda.stream(stream):
        ev0.record(stream)
    for _ in range(args.steps):
        rr, it = step()
        st = D.solve_stats()
        kernel_ms.append(st["device_ms"])
        bytes_.append(st["algorithmic_bytes"])
        fmas.append(st["fp64_fma"])
        iters.append(it)
        res.append(rr)
    with torch.cuda.stream(stream):
        ev1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ck = clocks.stop()
    ms_step = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, world, f"cuda:{dev}")
    r_fp64 = r.cpu().numpy()

    # end to end through the C ABI with host buffers: upload W (lower), b, mu and r, solve, download r. The
    # host arrays live in pinned (page-locked) memory, as a simulation that streams problems to the GPU keeps them.
    rp, cl, vl = D.W_lower()
    keep = []
    rp, cl, vl = (pinned_copy(a, keep) for a in (rp, cl, np.ascontiguousarray(vl.reshape(-1))))
    bh, muh = pinned_copy(d.b.reshape(-1), keep), pinned_copy(d.mu, keep)
    rh = pinned_copy(np.zeros(3 * n), keep)
    e2e_steps = max(1, min(args.steps, 3))
    h2d = rp.nbytes + cl.nbytes + vl.nbytes + bh.nbytes + muh.nbytes + rh.nbytes
    d2h = rh.nbytes
    E = bogus_gpu.DualFrictionProblem(dev)
    E.set(rp, cl, vl, bh, muh)  # warm (allocations)
    E.solveWith(pg, rh)
    e2e_ms = []
    for _ in range(e2e_steps):
        rh[...] = 0.0
        t0 = time.perf_counter()
        E.set(rp, cl, vl, bh, muh)
        E.solveWith(pg, rh)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    del E

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    kms = statistics.mean(kernel_ms)
    achieved = statistics.mean(bytes_) / (kms * 1e-3) / 1e9
    fp64_peak = bogus_gpu.measure_fp64_peak(dev)
    fp64_ach = 2.0 * statistics.mean(fmas) / (kms * 1e-3) / 1e12
    traffic = traffic_from_profiles(statistics.mean(bytes_))
    line = {
        "metric": METRIC, "value": ms_step, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded grid generator)",
        "config": config_dict(n, nnz_full, args.max_iters, {"iterations": iters[-1], "final_residual": res[-1],
                                            "reached_tol": bool(res[-1] < TOL)}),
        "assembly_ms": asm["device_ms"],
        "e2e": {"value": statistics.mean(e2e_ms), "unit": "ms", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_kind, "kernel": "k_pg_persistent",
                     "algorithmic_bytes_per_launch": statistics.mean(bytes_), "kernel_ms": kms},
        "fp64": {"achieved_tflops": fp64_ach, "peak_tflops": fp64_peak, "frac": fp64_ach / fp64_peak,
                 "note": "FMA work of the W passes only; GB300's FP64 rate bounds the FP64 kernels"},
        "gpu_launches": args.steps,
        "clocks": ck,
    }
    if world == 1 and not args.no_cpu_baseline:
        # the oracle on a bounded sample: the first CPU_SAMPLE_ITERS iterations of the same solve (about 5 s on
        # 16 Grace cores), scaled by the full solve's iteration count; the GPU's capped solve is compared with it
        orc = OracleSolve(d, D.W_lower())
        sample_iters = min(CPU_SAMPLE_ITERS, args.max_iters)
        cms, cres, cr, cit = orc.solve(sample_iters)
        pgs = bogus_gpu.ProjectedGradient()
        pgs.setTol(TOL)
        pgs.setMaxIters(sample_iters)
        rs = np.zeros(3 * n)
        gres = D.solveWith(pgs, rs)
        line["cpu_baseline"] = {
            "value": cms * iters[-1] / max(1, cit), "unit": "ms", "cores": orc.cores, "kind": "port",
            "sample": f"first {cit} APGD iterations of the same solve ({cms:.0f} ms), scaled to the full solve's "
                      f"{iters[-1]} iterations",
            "identical_result": bool(gres == cres and D.last_iterations == cit and np.array_equal(rs, cr))}
    if world == 1 and not args.no_secondary:
        line["secondary"] = measure_secondary(args, D, d, r_fp64, ms_step)
    print(json.dumps(line), flush=True)


def measure_secondary(args, D, d, r_fp64, fp64_ms):
    """The other measured targets, on the same GPU after the timed region (each labelled with its residual and
    iteration count; device times from CUDA events on the library's stream, best of a few solves)."""
    import bogus_gpu

    out = {}

    def best_of(solver, k=2, **kw):
        best = None
        for _ in range(k):
            r = np.zeros(3 * d.n)
            res = D.solveWith(solver, r, **kw)
            st = D.solve_stats()
            if best is None or st["device_ms"] < best[1]["device_ms"]:
                best = (res, st, r)
        return best

    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(CAP_500)
    res, st, _ = best_of(pg)
    out["apgd_500_iterations"] = {"device_ms": st["device_ms"], "iterations": st["iterations"], "residual": res,
                                  "note": "the same solve stopped at 500 iterations (the configuration's budget)"}
    # FP32-refined: FP32 iterations until FP32 rounding stops their progress (the library's stall test, default 4
    # stagnant iterations in a row), then FP64 ones to the tolerance
    pgm = bogus_gpu.ProjectedGradient()
    pgm.setTol(TOL)
    pgm.setMaxIters(FP32_ITERS)
    pgm.setMixedPrecision(True, args.max_iters)
    res, st, rm = best_of(pgm)
    err = float(np.linalg.norm(rm - r_fp64) / np.linalg.norm(r_fp64))
    out["fp32_refined_to_1e-6"] = {
        "device_ms": st["device_ms"], "fp32_ms": st["fp32_device_ms"],
        "fp32_iterations": st["iterations"] - st["refine_iterations"], "fp64_iterations": st["refine_iterations"],
        "residual": res, "reached_tol": bool(res < TOL), "speedup_vs_fp64": fp64_ms / st["device_ms"],
        "rel_error_vs_fp64": err,
        "error_note": "||r_mixed - r_fp64|| / ||r_fp64||, r_fp64 the FP64 solve to 1e-6 (bit-identical to the "
                      "oracle's iterates); W is singular here, so two iterates at residual 1e-6 may differ along "
                      "its null space"}
    # the FP32-refined form whose FP64 iterations take FP32 correction products (x_ref refreshed every 50
    # iterations), then a plain FP64 check of the tolerance
    pgh = bogus_gpu.ProjectedGradient()
    pgh.setTol(TOL)
    pgh.setMaxIters(FP32_ITERS)
    pgh.setMixedPrecision(True, args.max_iters)
    pgh.setFp32CorrectionProducts(HY_REFRESH)
    res, st, rh = best_of(pgh)
    out["fp32_refined_fp32_products_to_1e-6"] = {
        "device_ms": st["device_ms"], "fp32_ms": st["fp32_device_ms"],
        "fp32_iterations": st["iterations"] - st["refine_iterations"],
        "fp32_product_iterations": st["fp32_product_iterations"],
        "fp64_iterations": st["refine_iterations"] - st["fp32_product_iterations"],
        "residual": res, "reached_tol": bool(res < TOL), "speedup_vs_fp64": fp64_ms / st["device_ms"],
        "rel_error_vs_fp64": float(np.linalg.norm(rh - r_fp64) / np.linalg.norm(r_fp64)),
        "refresh": HY_REFRESH}
    # options with no counterpart in the reference: APGD's momentum product formed by linearity (one pass over
    # W fewer per momentum step; the oracle restates the same variant, tests check it bit for bit), alone and
    # with the FP32-refined form (where it applies to the FP64 iterations)
    for key, mixed in (("apgd_momentum_by_linearity_to_1e-6", False),
                       ("fp32_refined_momentum_by_linearity_to_1e-6", True)):
        pgl = bogus_gpu.ProjectedGradient()
        pgl.setTol(TOL)
        pgl.setMomentumByLinearity(True)
        if mixed:
            pgl.setMaxIters(FP32_ITERS)
            pgl.setMixedPrecision(True, args.max_iters)
        else:
            pgl.setMaxIters(args.max_iters)
        res, st, rl = best_of(pgl)
        out[key] = {
            "device_ms": st["device_ms"], "iterations": st["iterations"], "residual": res,
            "reached_tol": bool(res < TOL), "speedup_vs_fp64": fp64_ms / st["device_ms"],
            "w_passes_per_iteration": st["w_passes"] / max(1, st["iterations"]),
            "rel_error_vs_fp64": float(np.linalg.norm(rl - r_fp64) / np.linalg.norm(r_fp64))}
        if mixed:
            out[key].update({"fp32_ms": st["fp32_device_ms"],
                             "fp32_iterations": st["iterations"] - st["refine_iterations"],
                             "fp64_iterations": st["refine_iterations"]})
    pgs = bogus_gpu.ProjectedGradient()
    pgs.setTol(TOL)
    pgs.setMaxIters(args.max_iters)
    pgs.setDefaultVariant(bogus_gpu.SPG)
    res, st, _ = best_of(pgs)
    out["spg_to_1e-6"] = {"device_ms": st["device_ms"], "iterations": st["iterations"], "residual": res,
                          "reached_tol": bool(res < TOL)}
    gs = bogus_gpu.GaussSeidel()
    gs.coloring().update(True)
    gs.setTol(TOL)
    gs.setMaxIters(200)
    trace = []
    gs.callback().connect(lambda it, rr: trace.append((it, rr)))
    r = np.zeros(3 * d.n)
    res = D.solveWith(gs, r)
    st = D.solve_stats()
    sweeps = D.last_iterations
    out["gauss_seidel_colored_coulomb"] = {
        "sweeps": sweeps, "device_ms": st["device_ms"], "ms_per_sweep": st["device_ms"] / max(1, sweeps),
        "residual": res, "reached_tol": bool(res < TOL), "trace": trace[::2],
        "note": "does not reach 1e-6: residual 5.1e-3 after 1000 sweeps (8.5 s) on this problem"}
    out["batch_4096"] = measure_batch(args, sample_stride=16)
    out["adjoint_64x20000"] = measure_adjoint(args, steps=1)
    return out


def run_profile(iters: int, mixed: bool = False, products: bool = False) -> None:
    """One APGD solve of the benchmark problem capped at `iters` iterations (the solver kernel under ncu);
    products: the FP64 iterations with FP32 correction products (no FP32 part), then the plain FP64 check."""
    import bogus_gpu

    d = make_problem()
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(iters)
    if mixed:
        pg.setMixedPrecision(True, 1)
    if products:
        pg.setMaxIters(0)
        pg.setMixedPrecision(True, iters)
        pg.setFp32CorrectionProducts(HY_REFRESH)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r)
    st = D.solve_stats()
    print(json.dumps({"profile_iters": iters, "residual": res, "stats": st}))


BATCH_MAX_ITERS = 500


def _sync_time(fn, world):
    """Wall time of fn() between device synchronisations (and barriers across ranks), max over ranks."""
    import torch

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3
    if world > 1:
        torch.distributed.barrier()
    return max_over_ranks(ms, world, "cuda"), out


def measure_batch(args, sample_stride=16, rank=0, world=1, dev=0, steps=None):
    """4096 independent problems (16..4096 contacts, log-uniform) in one persistent launch per rank (the problems
    shared over the ranks by a greedy bin-pack on their W blocks), against a loop of the single-problem GPU path
    on a stratified sample of the problems (every sample_stride-th by size; rank 0, one GPU only). Each sampled
    problem's batched result is compared with its own single-problem solve and, on every fourth sampled
    problem, with the oracle."""
    import torch

    import bogus_gpu
    from bogus_gpu import generator, shard

    steps = steps or max(1, min(args.steps, 3))
    d, cptr = generator.batch(4096)
    nprob = len(cptr) - 1
    costs = shard.w_blocks_per_problem(d, cptr)
    parts = shard.partition(costs, world)
    mine = parts[rank]
    sub, scptr = (d, cptr) if world == 1 else shard.subset(d, cptr, mine)
    D = bogus_gpu.DualFrictionProblem(dev)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(sub))
    D.setBatch(scptr)
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(BATCH_MAX_ITERS)
    r = torch.zeros(3 * sub.n, dtype=torch.float64, device=f"cuda:{dev}")
    stream = torch.cuda.ExternalStream(D.stream(), device=f"cuda:{dev}")

    def solve(solver):
        with torch.cuda.stream(stream):
            r.zero_()
        return D.solveBatch_device(solver, r.data_ptr())

    solve(pg)
    times, kernel = [], []
    for _ in range(steps):
        ms, (res, its) = _sync_time(lambda: solve(pg), world)
        times.append(ms)
        kernel.append(D.solve_stats()["device_ms"])
    st = D.solve_stats()
    r_batch = r.cpu().numpy()
    # the FP32-refined batch with the same iteration budget per problem: up to 200 FP32 iterations, then FP64
    pgm = bogus_gpu.ProjectedGradient()
    pgm.setTol(TOL)
    pgm.setMaxIters(200)
    pgm.setMixedPrecision(True, BATCH_MAX_ITERS - 200)
    solve(pgm)
    mixed_ms, (res_m, its_m) = _sync_time(lambda: solve(pgm), world)
    st_m = D.solve_stats()
    # the momentum product formed by linearity (an option, not the reference's arithmetic), same budget
    pgl = bogus_gpu.ProjectedGradient()
    pgl.setTol(TOL)
    pgl.setMaxIters(BATCH_MAX_ITERS)
    pgl.setMomentumByLinearity(True)
    solve(pgl)
    lin_ms, (res_l, its_l) = _sync_time(lambda: solve(pgl), world)
    st_l = D.solve_stats()
    # both: the FP32-refined batch with the momentum product by linearity on its FP64 iterations
    pgml = bogus_gpu.ProjectedGradient()
    pgml.setTol(TOL)
    pgml.setMaxIters(200)
    pgml.setMixedPrecision(True, BATCH_MAX_ITERS - 200)
    pgml.setMomentumByLinearity(True)
    solve(pgml)
    ml_ms, (res_ml, its_ml) = _sync_time(lambda: solve(pgml), world)
    # the FP32-refined batch whose FP64 iterations take FP32 correction products, same budget
    pgmh = bogus_gpu.ProjectedGradient()
    pgmh.setTol(TOL)
    pgmh.setMaxIters(200)
    pgmh.setMixedPrecision(True, BATCH_MAX_ITERS - 200)
    pgmh.setFp32CorrectionProducts(BATCH_HY_REFRESH)
    solve(pgmh)
    mh_ms, (res_mh, its_mh) = _sync_time(lambda: solve(pgmh), world)
    # the launch shape chosen by the tuner (measured on this batch) against the default rule, same results
    rule_shape = D.batchShape()
    D.setBatchTuning(True)
    t0 = time.perf_counter()
    solve(pg)  # tunes (candidates measured at 30 iterations each), then solves
    torch.cuda.synchronize()
    tune_wall_ms = (time.perf_counter() - t0) * 1e3
    tuned_times = []
    for _ in range(steps):
        ms, (res_t, its_t) = _sync_time(lambda: solve(pg), world)
        tuned_times.append(ms)
    tuned_same = bool(np.array_equal(res_t, res) and np.array_equal(its_t, its) and
                      np.array_equal(r.cpu().numpy(), r_batch))
    tuned = {"shape": D.batchShape(), "rule_shape": rule_shape, "batched_ms": statistics.median(tuned_times),
             "tuning_wall_ms": tune_wall_ms, "candidates": [[list(sh), ms] for sh, ms in D.batchTuningLog()],
             "identical_results": tuned_same,
             "shape_key": "(schedule 0: one CTA per problem / 1: teams, CTAs per SM, team size)"}
    D.setBatchTuning(False)
    # the captured CUDA graph (upload of r, solve, download of r and results) against the plain host-buffer call
    keep = []
    rh = pinned_copy(np.zeros(3 * sub.n), keep)
    plain, graph = [], []
    for k in range(steps + 1):
        rh[...] = 0.0
        t0 = time.perf_counter()
        D.solveBatchWith(pg, rh)
        plain.append((time.perf_counter() - t0) * 1e3)
        rh[...] = 0.0
        t0 = time.perf_counter()
        res_g, its_g = D.solveBatchGraph(pg, rh)
        graph.append((time.perf_counter() - t0) * 1e3)
    graph_same = bool(np.array_equal(res_g, res) and np.array_equal(its_g, its) and np.array_equal(rh, r_batch))
    graphed = {"plain_call_ms": statistics.median(plain[1:]), "graph_replay_ms": statistics.median(graph[1:]),
               "capture_call_ms": graph[0], "identical_results": graph_same,
               "note": "host-buffer calls (pinned r), wall time per call including copies; the first graph call "
                       "captures"}
    allres = shard.gather_results(mine, np.stack([res, its, res_m, res_l, res_ml, res_mh], 1), nprob, world)
    out = {"problems": nprob, "contacts": int(d.n), "ranks": world, "max_iters": BATCH_MAX_ITERS,
           "batched_ms": statistics.median(times), "kernel_ms": statistics.median(kernel),
           "tuned": tuned, "cuda_graph": graphed,
           "algorithmic_gbs": st["algorithmic_bytes"] / (st["device_ms"] * 1e-3) / 1e9,
           "fp32_refined": {"split": "up to 200 FP32 + 300 FP64 iterations per problem", "batched_ms": mixed_ms,
                            "kernel_ms": st_m["device_ms"], "fp32_ms": st_m["fp32_device_ms"]},
           "momentum_by_linearity": {"batched_ms": lin_ms, "kernel_ms": st_l["device_ms"],
                                     "w_passes": st_l["w_passes"], "w_passes_reference_form": st["w_passes"]},
           "fp32_refined_momentum_by_linearity": {"split": "up to 200 FP32 + 300 FP64 iterations per problem, the "
                                                           "FP64 ones with the momentum product by linearity",
                                                  "batched_ms": ml_ms},
           "fp32_refined_fp32_products": {"split": "up to 200 FP32 + 300 FP64 iterations per problem, the FP64 ones "
                                                   f"with FP32 correction products (x_ref refreshed every {BATCH_HY_REFRESH})",
                                          "batched_ms": mh_ms},
           "timing": f"median of {steps} solves after a warm-up, wall time between device synchronisations"}
    if world > 1:
        out["partition"] = {"rule": "greedy bin-pack on W blocks", "blocks_per_rank": [int(costs[q].sum()) for q in parts],
                            "problems_per_rank": [int(q.size) for q in parts]}
    if rank != 0:
        return out
    out["iterations_max"] = int(allres[:, 1].max())
    out["iterations_mean"] = float(allres[:, 1].mean())
    out["converged_fraction"] = float(np.mean(allres[:, 0] < TOL))
    out["fp32_refined"]["converged_fraction"] = float(np.mean(allres[:, 2] < TOL))
    out["fp32_refined"]["speedup_vs_fp64_batch"] = out["batched_ms"] / mixed_ms
    out["momentum_by_linearity"]["converged_fraction"] = float(np.mean(allres[:, 3] < TOL))
    out["momentum_by_linearity"]["speedup_vs_fp64_batch"] = out["batched_ms"] / lin_ms
    out["fp32_refined_momentum_by_linearity"]["converged_fraction"] = float(np.mean(allres[:, 4] < TOL))
    out["fp32_refined_momentum_by_linearity"]["speedup_vs_fp64_batch"] = out["batched_ms"] / ml_ms
    out["fp32_refined_fp32_products"]["converged_fraction"] = float(np.mean(allres[:, 5] < TOL))
    out["fp32_refined_fp32_products"]["speedup_vs_fp64_batch"] = out["batched_ms"] / mh_ms
    if world == 1 and sample_stride:
        # the single-problem path, problem by problem (inputs set beforehand, each solve timed with its r copies)
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import pyoracle

        rp, cl, vl = D.W_lower()
        vl = vl.reshape(-1, 9)
        order = np.argsort(np.diff(cptr), kind="stable")
        sample = order[::sample_stride]
        single = bogus_gpu.DualFrictionProblem(dev)
        t_single = 0.0
        same_single = same_oracle = True
        checked = 0
        for k, p in enumerate(sample):
            c0, c1 = int(cptr[p]), int(cptr[p + 1])
            prp, pcl, pvl = rp[c0:c1 + 1] - rp[c0], cl[rp[c0]:rp[c1]] - c0, vl[rp[c0]:rp[c1]].reshape(-1)
            single.set(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
            rr = np.zeros(3 * (c1 - c0))
            t0 = time.perf_counter()
            res_s = single.solveWith(pg, rr)
            t_single += time.perf_counter() - t0
            same_single = same_single and res_s == res[p] and single.last_iterations == its[p] and \
                np.array_equal(rr, r_batch[3 * c0:3 * c1])
            if k % 4 == 0:
                O = pyoracle.DualProblem(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
                res_o, r_o, it_o = O.solve_pg(np.zeros(3 * (c1 - c0)), variant=3, coulomb=False, tol=TOL,
                                              max_iters=BATCH_MAX_ITERS)
                same_oracle = same_oracle and res_o == res[p] and it_o == its[p] and np.array_equal(r_o, rr)
                checked += 1
        scale = nprob / len(sample)
        out["loop_single_gpu"] = {
            "sample_problems": int(len(sample)), "sample_ms": t_single * 1e3, "estimated_full_loop_ms": t_single * 1e3 * scale,
            "sample": f"every {sample_stride}th problem by size, solved one by one through DualFrictionProblem.solveWith "
                      "(problem set beforehand; the timed call uploads r, solves and downloads r)"}
        out["speedup_vs_loop"] = t_single * 1e3 * scale / out["batched_ms"]
        out["identical_to_single_solves_on_sample"] = bool(same_single)
        out["identical_to_oracle"] = {"problems": checked, "identical": bool(same_oracle)}
    return out


def run_batch(args, rank=0, world=1, dev=0) -> None:
    out = measure_batch(args, rank=rank, world=world, dev=dev, sample_stride=16 if world == 1 else 0,
                        steps=args.steps)
    if rank == 0:
        line = {"metric": "batched APGD, 4096 problems, tol 1e-6 / 500 iterations (ms)", "value": out["batched_ms"],
                "unit": "ms", "n_gpus": world, "steps": args.steps, "higher_is_better": False, "scaling": "strong",
                "dtype": "f64", "data": "synthetic (seeded batch generator)",
                "config": {"workload": "batched_apgd_4096_problems", "parallelism": f"problems sharded over {world} ranks"
                           if world > 1 else "one GPU"}, "batch": out}
        print(json.dumps(line), flush=True)


def run_gs(args) -> None:
    """Gauss-Seidel on the 200 000-contact problem, both sweep orders: GPU time per sweep against the oracle."""
    import bogus_gpu

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    d = make_problem()
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    rp, cl, vl = D.W_lower()
    O = pyoracle.DualProblem(rp, cl, vl.reshape(-1), d.b, d.mu)
    out = {"workload": "gauss_seidel_200k_contacts", "law": "Coulomb (GaussSeidel default)"}
    for coloring in (False, True):
        gs = bogus_gpu.GaussSeidel()
        gs.coloring().update(coloring)
        gs.setMaxIters(25)
        r = np.zeros(3 * d.n)
        D.solveWith(gs, r)
        r = np.zeros(3 * d.n)
        res = D.solveWith(gs, r)
        gpu_ms = D.solve_stats()["device_ms"]

        def cpu_sweep_ms(threads):
            # per sweep, without the one-off setup (coloring, permutation, local blocks, first evaluation)
            pyoracle.set_gs_threads(threads)
            res_o, r_o, _ = O.solve_gs(np.zeros(3 * d.n), max_iters=25, coloring=coloring)
            pyoracle.set_gs_threads(1)
            return pyoracle.last_gs_sweep_ms() / 25, res_o, r_o

        cpu_ms, res_o, r_o = cpu_sweep_ms(1)
        entry = {"sweeps": 25, "gpu_ms_per_sweep": gpu_ms / 25, "cpu_oracle_ms_per_sweep": cpu_ms,
                 "residual": res, "identical": bool(res == res_o and np.array_equal(r, r_o))}
        if coloring:
            # the reference's per-color OpenMP loop on every host core (its iterates depend on thread timing)
            threads = os.cpu_count() or 1
            ms_par, res_par, _ = cpu_sweep_ms(threads)
            entry["cpu_threads"] = threads
            entry["cpu_parallel_ms_per_sweep"] = ms_par
            entry["cpu_parallel_residual"] = res_par
        out["colored" if coloring else "natural_order"] = entry
    # matrix-free sweep (ProductGaussSeidel) on the primal data: no W, M^-1 H^T x kept per body
    P = bogus_gpu.PrimalFrictionProblem.from_generated(d)
    pgs = bogus_gpu.ProductGaussSeidel()
    pgs.setMaxIters(25)
    r = np.zeros(3 * d.n)
    P.solveWith(pgs, r)
    r = np.zeros(3 * d.n)
    res = P.solveWith(pgs, r)
    gpu_ms = P.solve_stats()["device_ms"]
    PO = pyoracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    t0 = time.perf_counter()
    PO.solve_product_gs(np.zeros(d.nbodies * 6), d.b.reshape(-1), d.mu, np.zeros(3 * d.n), max_iters=0)
    t1 = time.perf_counter()
    res_o, r_o, _ = PO.solve_product_gs(np.zeros(d.nbodies * 6), d.b.reshape(-1), d.mu, np.zeros(3 * d.n), max_iters=25)
    t2 = time.perf_counter()
    cpu_ms = ((t2 - t1) - (t1 - t0)) * 1e3
    out["matrix_free"] = {"sweeps": 25, "gpu_ms_per_sweep": gpu_ms / 25, "cpu_oracle_ms_per_sweep": cpu_ms / 25,
                          "residual": res, "identical": bool(res == res_o and np.array_equal(r, r_o))}
    print(json.dumps(out), flush=True)


def run_mixed(args) -> None:
    """FP32-refined APGD on the 200 000-contact problem, time to residual 1e-6 for several FP32 / FP64 splits (m
    FP32 iterations, then FP64 ones to the tolerance) and with the stall test ending the FP32 part, against the
    FP64 solve to 1e-6; with each result its relative distance to the FP64 result."""
    import bogus_gpu

    d = make_problem()
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))

    def timed(pg):
        best = None
        for k in range(max(1, args.warmup) + args.steps):
            r = np.zeros(3 * d.n)
            res = D.solveWith(pg, r, staticProblem=True)
            st = D.solve_stats()
            if k >= max(1, args.warmup) and (best is None or st["device_ms"] < best[1]["device_ms"]):
                best = (res, st, r)
        return best

    pg64 = bogus_gpu.ProjectedGradient()
    pg64.setTol(TOL)
    pg64.setMaxIters(args.max_iters)
    res_p, st_p, r64 = timed(pg64)
    splits = {}
    # fixed FP32 budgets (stall test off), then the stall test with a budget it does not reach, then that with
    # FP32 correction products in the FP64 iterations (x_ref refreshed every 25, 50, 100 iterations), and those
    # products alone (no FP32 part)
    for m32, stall, hy in ((1000, 0, 0), (2000, 0, 0), (3000, 0, 0), (4000, 0, 0), (6000, 0, 0), (20000, 4, 0),
                           (20000, 4, 25), (20000, 4, 50), (20000, 4, 100), (0, 4, 50)):
        pgm = bogus_gpu.ProjectedGradient()
        pgm.setTol(TOL)
        pgm.setMaxIters(m32)
        pgm.setMixedPrecision(True, args.max_iters)
        pgm.setFp32StallIterations(stall)
        pgm.setFp32CorrectionProducts(hy)
        res_m, st_m, rm = timed(pgm)
        key = f"{m32}" if stall == 0 else f"stall_test_{stall}"
        if hy:
            key = f"fp32_products_refresh_{hy}" + ("_no_fp32_part" if m32 == 0 else "")
        splits[key] = {"device_ms": st_m["device_ms"], "fp32_ms": st_m["fp32_device_ms"],
                       "fp32_iterations": st_m["iterations"] - st_m["refine_iterations"],
                       "fp32_product_iterations": st_m["fp32_product_iterations"],
                       "fp64_iterations": st_m["refine_iterations"] - st_m["fp32_product_iterations"],
                       "residual": res_m,
                       "reached_tol": bool(res_m < TOL), "speedup_vs_fp64": st_p["device_ms"] / st_m["device_ms"],
                       "rel_error_vs_fp64": float(np.linalg.norm(rm - r64) / np.linalg.norm(r64))}
    print(json.dumps({
        "workload": "fp32_refined_apgd_200k_contacts_to_1e-6", "law": "SOC", "contacts": d.n,
        "fp64": {"device_ms": st_p["device_ms"], "iterations": st_p["iterations"], "residual": res_p,
                 "ms_per_iteration": st_p["device_ms"] / max(1, st_p["iterations"])},
        "fp32_refined_by_fp32_iterations": splits,
        "timing": f"best of {args.steps} after {max(1, args.warmup)} warm-up solves, CUDA events on the library "
                  "stream"}), flush=True)


def run_admm(args) -> None:
    """Primal ADMM (PrimalFrictionProblem::solveWith(ADMM&, 0, v, r), reference defaults: accelerated, step 1e-2)
    on the 200 000-contact / 50 000-body problem, 100 iterations: GPU against the oracle (one core)."""
    import bogus_gpu

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    d = make_problem()
    P = bogus_gpu.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    admm = bogus_gpu.ADMM()
    admm.setTol(1e-12)
    admm.setMaxIters(100)
    best = None
    for k in range(args.warmup + args.steps):
        v, r = np.zeros(d.nbodies * 6), np.zeros(3 * d.n)
        res = P.solveWith(admm, 0.0, v, r)
        st = P.solve_stats()
        if k >= args.warmup and (best is None or st["device_ms"] < best[1]["device_ms"]):
            best = (res, st)
    res, st = best
    O = pyoracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    t0 = time.perf_counter()
    res_o, v_o, r_o, it_o = O.solve_admm(d.minv, 0.0, d.mu, np.zeros(d.nbodies * 6), d.b.reshape(-1),
                                         np.zeros(d.nbodies * 6), np.zeros(3 * d.n), tol=1e-12, max_iters=100)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    print(json.dumps({
        "workload": "admm_200k_contacts", "iterations": st["iterations"], "residual": res,
        "gpu_ms": st["device_ms"], "gpu_ms_per_iteration": st["device_ms"] / max(1, st["iterations"]),
        "algorithmic_gbs": st["algorithmic_bytes"] / (st["device_ms"] * 1e-3) / 1e9,
        "cpu_oracle_ms": cpu_ms, "cpu_cores": pyoracle.num_threads(), "identical": bool(res == res_o),
        "timing": f"best of {args.steps} after {args.warmup} warm-up solves (CUDA events); oracle once"}),
        flush=True)


def run_dama(args) -> None:
    """DualAMA (PrimalFrictionProblem::solveWith(DualAMAType&, v, r, false), reference defaults: accelerated,
    steps 0.1, 6 line-search trials) on the 200 000-contact / 50 000-body problem with the Coulomb law, 100
    iterations from v = M^-1 f, r = 0: GPU against the oracle (one core)."""
    import bogus_gpu

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    d = make_problem()
    mass = np.linalg.inv(d.minv)
    f = np.zeros(d.nbodies * 6)
    P = bogus_gpu.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu, f=f, M=mass)
    dama = bogus_gpu.DualAMA()
    dama.setTol(1e-12)
    dama.setMaxIters(100)
    best = None
    for k in range(args.warmup + args.steps):
        v, r = np.zeros(d.nbodies * 6), np.zeros(3 * d.n)
        res = P.solveWith(dama, v, r)
        st = P.solve_stats()
        if k >= args.warmup and (best is None or st["device_ms"] < best[1]["device_ms"]):
            best = (res, st, v, r)
    res, st, v, r = best
    O = pyoracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    t0 = time.perf_counter()
    res_o, v_o, r_o, it_o = O.solve_dual_ama(mass, d.mu, f, d.b.reshape(-1), np.zeros(d.nbodies * 6),
                                             np.zeros(3 * d.n), tol=1e-12, max_iters=100)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    print(json.dumps({
        "workload": "dual_ama_200k_contacts", "iterations": st["iterations"], "residual": res,
        "gpu_ms": st["device_ms"], "gpu_ms_per_iteration": st["device_ms"] / max(1, st["iterations"]),
        "algorithmic_gbs": st["algorithmic_bytes"] / (st["device_ms"] * 1e-3) / 1e9,
        "cpu_oracle_ms": cpu_ms, "cpu_cores": pyoracle.num_threads(),
        "identical": bool(res == res_o and np.array_equal(v, v_o) and np.array_equal(r, r_o)),
        "timing": f"best of {args.steps} after {args.warmup} warm-up solves (CUDA events); oracle once"}),
        flush=True)


def measure_adjoint(args, steps=2, rank=0, world=1, dev=0):
    """Gradient workload: 64 problems x 20 000 contacts (bodies = contacts / 3, compliance 0.05 I), forward =
    batched APGD to 1e-10 per problem, loss L = g . r with g ~ N(0, 1); backward = the adjoint (dL/db, dL/dmu)
    over the batch, then dL/dH, dL/dw, dL/df. Both laws: the Coulomb problem (the configuration's law, adjoint by
    bi-conjugate gradients stabilised) and the SOC problem (conjugate gradients). Reports t_adjoint / t_forward
    (device times). With several ranks each solves its share of the problems (all of equal size)."""
    import bogus_gpu
    from bogus_gpu import generator, shard

    d, cptr = generator.adjoint_batch(nproblems=getattr(args, "adjoint_problems", 64))
    nprob = len(cptr) - 1
    parts = shard.partition(np.diff(cptr), world)
    mine = parts[rank]
    sub, scptr = (d, cptr) if world == 1 else shard.subset(d, cptr, mine)
    P = bogus_gpu.PrimalFrictionProblem(sub.minv, sub.objA, sub.objB, sub.HA, sub.HB, sub.b.reshape(-1), sub.mu,
                                        device=dev)
    D = bogus_gpu.DualFrictionProblem(dev)
    D.computeFrom(P)
    D.add_compliance(generator.ADJOINT_COMPLIANCE)
    D.setBatch(scptr)
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(1e-10)
    pg.setMaxIters(MAX_ADJ_FWD_ITERS)
    g = np.random.default_rng(6).standard_normal(3 * d.n)
    g_mine = g.reshape(-1, 3)[np.concatenate([np.arange(cptr[p], cptr[p + 1]) for p in mine])].reshape(-1)
    out = {"problems": nprob, "contacts": int(d.n), "ranks": world, "compliance": generator.ADJOINT_COMPLIANCE}
    laws = (("coulomb", True), ("soc", False))
    which = getattr(args, "adjoint_law", "both")
    for law, coulomb in (laws if which == "both" else [lw for lw in laws if lw[0] == which]):
        fwd, adj, prim = [], [], []
        # the Coulomb forward runs up to 20 000 iterations (tens of seconds): it is timed without a warm-up
        warm = 0 if coulomb else 1
        for k in range(warm + steps):
            r = np.zeros(3 * sub.n)
            res, its = D.solveBatchWith(pg, r, staticProblem=not coulomb)
            tf = D.solve_stats()["device_ms"]
            D.adjoint(r, g_mine, tol=1e-10, coulomb=coulomb)
            ta = D.solve_stats()["device_ms"]
            t1 = time.perf_counter()
            D.adjoint_primal(P)
            t2 = time.perf_counter()
            if k >= warm:
                fwd.append(tf)
                adj.append(ta)
                prim.append((t2 - t1) * 1e3)
        tf = max_over_ranks(statistics.median(fwd), world, "cuda")
        ta = max_over_ranks(statistics.median(adj), world, "cuda")
        allres = shard.gather_results(mine, np.stack([res, its], 1), nprob, world)
        e = {"forward_ms": tf, "adjoint_ms": ta, "t_adjoint_over_t_forward": ta / tf,
             "adjoint_iterations": D.last_adjoint_iterations, "adjoint_rel_residual": D.last_adjoint_residual,
             "adjoint_solver": "BiCGSTAB (2 W passes per iteration)" if coulomb else "CG (1 W pass per iteration)",
             "primal_gradients_wall_ms": statistics.median(prim)}
        if allres is not None:
            e["forward_iterations_max"] = int(allres[:, 1].max())
            e["forward_converged_fraction"] = float(np.mean(allres[:, 0] < 1e-10))
        out[law] = e
    out["timing"] = (f"median of {steps} (SOC: after a warm-up); device times (CUDA events) of the batched solve "
                     "kernel and of the adjoint kernel (max over ranks)")
    out["t_adjoint_over_t_forward"] = out["coulomb" if "coulomb" in out else "soc"]["t_adjoint_over_t_forward"]
    return out


def run_adjoint(args, rank=0, world=1, dev=0) -> None:
    out = measure_adjoint(args, steps=args.steps, rank=rank, world=world, dev=dev)
    if rank == 0:
        law = "Coulomb" if "coulomb" in out else "SOC"
        line = {"metric": f"adjoint / forward time, {out['problems']} x 20 000 contacts, {law} law",
                "value": out["t_adjoint_over_t_forward"],
                "unit": "ratio", "n_gpus": world, "steps": args.steps, "higher_is_better": False,
                "scaling": "strong", "dtype": "f64", "data": "synthetic (seeded adjoint batch generator)",
                "config": {"workload": f"adjoint_{out['problems']}x20000_contacts"}, "adjoint": out}
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the secondary measurements of the headline line")
    ap.add_argument("--max-iters", type=int, default=MAX_ITERS,
                    help="iteration budget of the time-to-residual solves (default: the benchmark's)")
    ap.add_argument("--profile", type=int, default=0,
                    help="run one solve capped at this many iterations and exit (for ncu captures)")
    ap.add_argument("--workload", default="apgd",
                    choices=["apgd", "batch", "gs", "mixed", "admm", "dama", "adjoint"],
                    help="apgd: the benchmark line; batch / adjoint (sharded over ranks under torchrun), gs, mixed, "
                         "admm, dama: the secondary measurements on their own")
    ap.add_argument("--adjoint-problems", type=int, default=64,
                    help="--workload adjoint: problems of 20 000 contacts in the batch (64: the benchmark's)")
    ap.add_argument("--adjoint-law", default="both", choices=["both", "coulomb", "soc"],
                    help="--workload adjoint: the laws to run")
    ap.add_argument("--profile-mixed", action="store_true",
                    help="with --profile: the FP32-refined solve (FP32 iterations, then 1 FP64 iteration)")
    ap.add_argument("--profile-fp32-products", action="store_true",
                    help="with --profile: FP64 iterations with FP32 correction products (no FP32 part)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    single = {"mixed": run_mixed, "admm": run_admm, "dama": run_dama, "gs": run_gs}
    if args.workload in single:
        single[args.workload](args)
        return
    if args.profile:
        run_profile(args.profile, args.profile_mixed, args.profile_fp32_products)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl", device_id=torch.device(f"cuda:{local_rank}"))
    if args.workload == "batch":
        run_batch(args, rank, world, local_rank)
    elif args.workload == "adjoint":
        run_adjoint(args, rank, world, local_rank)
    else:
        run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
