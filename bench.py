#!/usr/bin/env python
"""Benchmark: FP64 APGD solve of the 200 000-contact friction problem on one GB300 (time to residual).

Workload (one "step"): DualFrictionProblem::solveWith(ProjectedGradient, r) with the reference's defaults
(APGD, SOC law, line search 8 / 1.25 / 0.5) at tol 1e-6 with at most 500 iterations, from r = 0, on the
seeded grid problem (50 000 rigid bodies, 200 000 contacts, W assembled on the GPU). The solve stops at
the tolerance or after 500 iterations, whichever comes first; the GPU and the CPU oracle run bit-identical
iterations, so both arms do the same work.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Our arm prints `value` (ms per solve, inputs resident in HBM, CUDA events on the library's stream), `e2e`
(the C-ABI call with host buffers: upload of W/b/mu/r, solve, download of r), the roofline of the
persistent solver kernel, FP64 pipe use and the CPU baseline (the oracle on the host cores).
`--impl reference` times the CPU restatement of the reference (the oracle, OpenMP on all host cores) on the
same workload. With N > 1 (torchrun) every rank solves its own replica (a single problem does not shard).
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
MAX_ITERS = 500
MAX_ADJ_FWD_ITERS = 20000
METRIC = "time-to-residual 1e-6 (ms), FP64 APGD, 200k contacts"
WORKLOAD = "fp64_apgd_200k_contacts"


def config_dict(n, nnzb_full, extra=None):
    d = {"workload": WORKLOAD, "contacts": n, "bodies": 50_000, "w_blocks_full": nnzb_full,
         "w_blocks_lower": (nnzb_full + n) // 2, "solver": "APGD (reference defaults), SOC law",
         "tol": TOL, "max_iters": MAX_ITERS, "start": "r = 0", "generator": "grid, seed 1",
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
def cpu_oracle_solve(d, threads=None):
    """The oracle (CPU restatement of the reference) on all host cores: returns (ms, residual, iterations)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    pyoracle.build()
    if threads:
        pyoracle.set_num_threads(threads)
    P = pyoracle.PrimalProblem(d.minv, d.objA, d.objB, d.HA, d.HB)
    rp, cl, vl = P.assemble()
    O = pyoracle.DualProblem(rp, cl, vl, d.b, d.mu)
    t0 = time.perf_counter()
    res, r, it = O.solve_pg(np.zeros(3 * d.n), variant=3, coulomb=False, tol=TOL, max_iters=MAX_ITERS)
    ms = (time.perf_counter() - t0) * 1e3
    return ms, res, it, pyoracle.num_threads(), (rp, cl, vl)


def run_reference(args, rank, world):
    if world > 1 and rank != 0:
        return
    d = make_problem()
    times = []
    res = it = cores = None
    nnz_full = 0
    for step in range(args.warmup + args.steps):
        ms, res, it, cores, lower = cpu_oracle_solve(d)
        nnz_full = 2 * len(lower[1]) - d.n
        if step >= args.warmup:
            times.append(ms)
    v = statistics.mean(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded grid generator)",
        "config": config_dict(d.n, nnz_full or 0, {"iterations": it, "final_residual": res}),
        "cpu_baseline": {"value": v, "unit": "ms", "cores": cores, "kind": "port",
                         "sample": f"full solve ({it} APGD iterations) of the same problem, per step"},
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
    pg.setMaxIters(MAX_ITERS)
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
        "config": config_dict(n, nnz_full, {"iterations": iters[-1], "final_residual": res[-1],
                                            "assembly_ms": asm["device_ms"]}),
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
        cms, cres, cit, cores, _ = cpu_oracle_solve(d)
        line["cpu_baseline"] = {"value": cms, "unit": "ms", "cores": cores, "kind": "port",
                                "sample": f"one full solve ({cit} iterations, residual {cres:.3e}) of the same problem"}
        line["cpu_baseline"]["identical_result"] = bool(cit == iters[-1] and cres == res[-1])
    print(json.dumps(line), flush=True)


def run_profile(iters: int, mixed: bool = False) -> None:
    """One APGD solve of the benchmark problem capped at `iters` iterations (the solver kernel under ncu)."""
    import bogus_gpu

    d = make_problem()
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(iters)
    if mixed:
        pg.setMixedPrecision(True, 1)
    r = np.zeros(3 * d.n)
    res = D.solveWith(pg, r)
    st = D.solve_stats()
    print(json.dumps({"profile_iters": iters, "residual": res, "stats": st}))


def run_batch(args) -> None:
    """4096 independent problems (16..4096 contacts, log-uniform) in one persistent launch, against a loop of the
    single-problem GPU path and the CPU oracle on a stratified sample of the problems."""
    import torch

    import bogus_gpu
    from bogus_gpu import generator

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    d, cptr = generator.batch(4096)
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))
    D.setBatch(cptr)
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(TOL)
    pg.setMaxIters(MAX_ITERS)
    n = d.n
    r = torch.zeros(3 * n, dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.ExternalStream(D.stream(), device="cuda:0")

    def step():
        with torch.cuda.stream(stream):
            r.zero_()
        return D.solveBatch_device(pg, r.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res, its = step()
    torch.cuda.synchronize()
    batched_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    st = D.solve_stats()
    # the FP32-refined batch with the same 500-iteration budget per problem: up to 200 FP32 iterations, then up
    # to 300 FP64 ones (a 500 + 50 split spends most of its time in FP32 iterations that cannot reach 1e-6)
    pgm = bogus_gpu.ProjectedGradient()
    pgm.setTol(TOL)
    pgm.setMaxIters(200)
    pgm.setMixedPrecision(True, MAX_ITERS - 200)
    for _ in range(2):
        with torch.cuda.stream(stream):
            r.zero_()
        res_m, its_m = D.solveBatch_device(pgm, r.data_ptr())
    st_m = D.solve_stats()
    # the single-problem path, problem by problem, on every 16th problem by size (stratified), scaled by 16
    rp, cl, vl = D.W_lower()
    vl = vl.reshape(-1, 9)
    order = np.argsort(np.diff(cptr), kind="stable")
    sample = order[::16]
    single = bogus_gpu.DualFrictionProblem(0)
    import pyoracle
    t_single = 0.0
    t_cpu = 0.0
    same = True
    for p in sample:
        c0, c1 = int(cptr[p]), int(cptr[p + 1])
        prp, pcl, pvl = rp[c0:c1 + 1] - rp[c0], cl[rp[c0]:rp[c1]] - c0, vl[rp[c0]:rp[c1]].reshape(-1)
        single.set(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
        rr = np.zeros(3 * (c1 - c0))
        t0 = time.perf_counter()
        res_s = single.solveWith(pg, rr)
        t_single += time.perf_counter() - t0
        O = pyoracle.DualProblem(prp, pcl, pvl, d.b[c0:c1], d.mu[c0:c1])
        t0 = time.perf_counter()
        res_o, r_o, it_o = O.solve_pg(np.zeros(3 * (c1 - c0)), variant=3, coulomb=False, tol=TOL, max_iters=MAX_ITERS)
        t_cpu += time.perf_counter() - t0
        same = same and res_s == res_o == res[p] and it_o == its[p]
    scale = len(cptr) - 1
    scale = scale / len(sample)
    print(json.dumps({
        "workload": "batched_apgd_4096_problems", "problems": len(cptr) - 1, "contacts": n,
        "batched_ms": batched_ms, "kernel_ms": st["device_ms"], "iterations_max": int(its.max()),
        "iterations_mean": float(its.mean()), "converged_fraction": float(np.mean(res < TOL)),
        "loop_single_gpu_ms_est": t_single * 1e3 * scale, "cpu_oracle_ms_est": t_cpu * 1e3 * scale,
        "cpu_threads": pyoracle.num_threads(), "sample": f"{len(sample)} problems (every 16th by size), scaled",
        "speedup_vs_loop": t_single * 1e3 * scale / batched_ms, "identical_on_sample": bool(same),
        "algorithmic_gbs": st["algorithmic_bytes"] / (st["device_ms"] * 1e-3) / 1e9,
        "fp32_refined": {"split": "up to 200 FP32 + 300 FP64 iterations per problem",
                         "kernel_ms": st_m["device_ms"], "fp32_ms": st_m["fp32_device_ms"],
                         "converged_fraction": float(np.mean(res_m < TOL)),
                         "speedup_vs_fp64_batch": st["device_ms"] / st_m["device_ms"]}}), flush=True)


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
    """FP32-refined APGD on the 200 000-contact problem: 500 FP32 iterations then up to 50 FP64 ones, against
    the FP64 solve run to the same FP64 residual (time to the same residual, both on the GPU)."""
    import bogus_gpu

    d = make_problem()
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(bogus_gpu.PrimalFrictionProblem.from_generated(d))

    def timed(pg):
        best = None
        for k in range(args.warmup + args.steps):
            r = np.zeros(3 * d.n)
            res = D.solveWith(pg, r, staticProblem=True)
            st = D.solve_stats()
            if k >= args.warmup and (best is None or st["device_ms"] < best[1]["device_ms"]):
                best = (res, st)
        return best

    pgm = bogus_gpu.ProjectedGradient()
    pgm.setTol(TOL)
    pgm.setMaxIters(MAX_ITERS)
    pgm.setMixedPrecision(True, 50)
    res_m, st_m = timed(pgm)
    pg64 = bogus_gpu.ProjectedGradient()
    pg64.setTol(TOL)
    pg64.setMaxIters(MAX_ITERS)
    res_p, st_p = timed(pg64)
    # the FP64 solve to the residual the mixed solve reached
    pgt = bogus_gpu.ProjectedGradient()
    pgt.setTol(res_m)
    pgt.setMaxIters(4 * MAX_ITERS)
    res_t, st_t = timed(pgt)
    m32 = st_m["fp32_device_ms"]
    print(json.dumps({
        "workload": "fp32_refined_apgd_200k_contacts", "law": "SOC", "contacts": d.n,
        "mixed": {"device_ms": st_m["device_ms"], "fp32_ms": m32, "fp32_iterations":
                  st_m["iterations"] - st_m["refine_iterations"], "fp64_refine_iterations": st_m["refine_iterations"],
                  "fp64_residual": res_m,
                  "fp32_ms_per_iteration": m32 / max(1, st_m["iterations"] - st_m["refine_iterations"]),
                  "algorithmic_gbs": st_m["algorithmic_bytes"] / (st_m["device_ms"] * 1e-3) / 1e9},
        "fp64_same_iterations": {"device_ms": st_p["device_ms"], "iterations": st_p["iterations"],
                                 "residual": res_p, "ms_per_iteration": st_p["device_ms"] / max(1, st_p["iterations"])},
        "fp64_to_mixed_residual": {"device_ms": st_t["device_ms"], "iterations": st_t["iterations"],
                                   "residual": res_t, "reached": bool(res_t <= res_m)},
        "speedup_time_to_residual": st_t["device_ms"] / st_m["device_ms"],
        "timing": f"best of {args.steps} after {args.warmup} warm-up solves, CUDA events on the library stream"}),
        flush=True)


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


def run_adjoint(args) -> None:
    """Gradient workload: 64 problems x 20 000 contacts (bodies = contacts / 3, compliance 0.05 I), forward =
    batched APGD with the SOC law to 1e-10 per problem, loss L = g . r with g ~ N(0, 1); backward = the adjoint
    (dL/db, dL/dmu) over the whole batch, then dL/dH, dL/dw, dL/df. Reports t_adjoint / t_forward."""
    import bogus_gpu
    from bogus_gpu import generator

    d, cptr = generator.adjoint_batch()
    P = bogus_gpu.PrimalFrictionProblem(d.minv, d.objA, d.objB, d.HA, d.HB, d.b.reshape(-1), d.mu)
    D = bogus_gpu.DualFrictionProblem(0)
    D.computeFrom(P)
    D.add_compliance(generator.ADJOINT_COMPLIANCE)
    D.setBatch(cptr)
    pg = bogus_gpu.ProjectedGradient()
    pg.setTol(1e-10)
    pg.setMaxIters(MAX_ADJ_FWD_ITERS)
    g = np.random.default_rng(6).standard_normal(3 * d.n)
    fwd, adj, prim = [], [], []
    for k in range(args.warmup + args.steps):
        r = np.zeros(3 * d.n)
        res, its = D.solveBatchWith(pg, r)
        tf = D.solve_stats()["device_ms"]
        t0 = time.perf_counter()
        db, dmu = D.adjoint(r, g, tol=1e-10)
        ta = D.solve_stats()["device_ms"]
        t1 = time.perf_counter()
        D.adjoint_primal(P)
        t2 = time.perf_counter()
        if k >= args.warmup:
            fwd.append(tf)
            adj.append(ta)
            prim.append((t2 - t1) * 1e3)
    tf, ta = statistics.median(fwd), statistics.median(adj)
    print(json.dumps({
        "workload": "adjoint_64x20000_contacts", "problems": len(cptr) - 1, "contacts": d.n,
        "compliance": generator.ADJOINT_COMPLIANCE, "forward_ms": tf, "forward_iterations_max": int(its.max()),
        "forward_converged_fraction": float(np.mean(res < 1e-10)), "adjoint_ms": ta,
        "adjoint_cg_iterations": D.last_adjoint_iterations, "adjoint_rel_residual": D.last_adjoint_residual,
        "primal_gradients_wall_ms": statistics.median(prim), "t_adjoint_over_t_forward": ta / tf,
        "timing": f"median of {args.steps} after {args.warmup} warm-up; device times (CUDA events) of the batched "
                  "solve kernel and of the adjoint kernel"}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", type=int, default=0,
                    help="run one solve capped at this many iterations and exit (for ncu captures)")
    ap.add_argument("--workload", default="apgd",
                    choices=["apgd", "batch", "gs", "mixed", "admm", "dama", "adjoint"],
                    help="apgd: the benchmark line; batch / gs / mixed / admm / dama / adjoint: secondary measurements")
    ap.add_argument("--profile-mixed", action="store_true",
                    help="with --profile: the FP32-refined solve (FP32 iterations, then 1 FP64 iteration)")
    args = ap.parse_args()
    if args.workload == "mixed":
        run_mixed(args)
        return
    if args.workload == "admm":
        run_admm(args)
        return
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.workload == "dama":
        run_dama(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "gs":
        run_gs(args)
        return
    if args.profile:
        run_profile(args.profile, args.profile_mixed)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl", device_id=torch.device(f"cuda:{local_rank}"))
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
