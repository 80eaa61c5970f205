"""Benchmark of the Galerkin assembly + Krylov solve path on GB300.

Workload (the 3D unit cube): the Kuhn subdivision of a 32^3 grid
(196,608 tets), every vertex coordinate jittered by seeded uniform +-0.1h,
FP64 signed squared edge lengths. A step assembles the k=1 and k=2 Hodge masses
and exterior-derivative stiffnesses (M_1, M_2, dif_both(2), dif_both(3)) from
lengths resident in HBM; the metric is assembled cells/s (cells per step time).
The same run times the mixed k=1 Hodge-Laplace solve by preconditioned MINRES to
1e-10 (solves/s, p50/p99 latency) and the end-to-end assembly through the C ABI
with host buffers.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --workload precision|serve|batch|next|dirac|shapes

The other workloads: the 4D FP32-with-refinement study, the served request
stream, many meshes assembled in one launch set, the rows after the headline
path (matrix-free operator, source load, de Rham map, leapfrog), and the direct
Lorentzian Dirac solves by mesh size.

Multi-GPU: the path does not shard (one mesh per solve), so N > 1 runs N
independent replicas, one per rank, with no collective on the data path.
"""
from __future__ import annotations

import argparse
import collections
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIM, NBOX, JITTER, SEED = 3, 32, 0.1, 20261203
FORMS = [("mass", 1), ("mass", 2), ("dif_both", 2), ("dif_both", 3)]
METRIC = "assembled cells/s"
L2_BYTES = 129 * 2 ** 20


def comb(n, k):
    return math.comb(n, k) if 0 <= k <= n else 0


def local_shape(n, name, k):
    """(rows, cols, symmetric) of the element matrix of a form."""
    tg = k - 1 if name in ("dif_test", "dif_both") else k
    sg = k - 1 if name in ("dif_trial", "dif_both") else k
    return comb(n + 1, tg + 1), comb(n + 1, sg + 1), name in ("mass", "dif_both")


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), int(
        os.environ.get("WORLD_SIZE", "1"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(ms: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's step time (all ranks call it; one all-reduce MAX)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# reference arm / CPU baseline: the oracle's OpenMP assembly
# ---------------------------------------------------------------------------

def cpu_assembly(nbox: int, steps: int = 1):
    """The oracle's C++/OpenMP assembly of the step's four forms on the same
    mesh and lengths; returns the cell count, the per-step times, the host
    threads used and the last step's matrices (the parity reference)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    cx, coords = oracle.cartesian_unit(DIM, nbox)
    coords = oracle.jitter_coords(coords, nbox, SEED, JITTER)
    lengths = cx.edge_lengths_sq(coords)
    wc = oracle.WhitneyComplex(cx, lengths)
    times, mats = [], None
    for _ in range(steps):
        t0 = time.perf_counter()
        mats = [getattr(wc, name)(k) for name, k in FORMS]
        times.append(time.perf_counter() - t0)
    return cx.ncells(), times, oracle.num_threads(), mats


def parity_record(gpu_mats, ref_mats):
    """Parity of the timed step's matrices with the oracle's: CSR row_ptr and
    col_idx bit-exact, values by relative Frobenius norm (bar 1e-12)."""
    import scipy.sparse as sp

    exact, worst, per = True, 0.0, {}
    for (name, k), g, r in zip(FORMS, gpu_mats, ref_mats):
        g = g.to_scipy()
        pat = g.shape == r.shape and np.array_equal(g.indptr.astype(np.int64), r.indptr.astype(np.int64)) and \
            np.array_equal(g.indices.astype(np.int64), r.indices.astype(np.int64))
        if pat:
            err = float(np.linalg.norm(g.data - r.data) / max(np.linalg.norm(r.data), 1e-300))
        else:
            d = (sp.csr_matrix(g) - r).tocsr()
            err = float(sp.linalg.norm(d) / max(sp.linalg.norm(r), 1e-300))
        exact &= bool(pat)
        worst = max(worst, err)
        per[f"{name}({k})"] = {"pattern_exact": bool(pat), "rel_frob": err}
    return {"pattern_exact": exact, "max_rel_frob": worst, "bar_rel_frob": 1e-12, "pass": exact and worst <= 1e-12,
            "against": "oracle C++ restatement of the reference assembly, same mesh and lengths", "forms": per}


def workload_name(ncells: int) -> str:
    """The headline workload, worded identically in both arms."""
    return (f"kuhn {DIM}D {NBOX}^3 ({ncells} tets), jitter 0.1h seed {SEED}; step = M_1, M_2, dif_both(2), "
            f"dif_both(3) assembled from resident lengths")


DTYPE_FP64 = "f64 (float-float compute, 48-bit significand; f64 storage)"


def run_reference(args):
    rank, _, world = env_rank()
    if rank != 0:
        return
    ncells, times, cores, _ = cpu_assembly(NBOX, args.warmup + args.steps)
    t = times[args.warmup:]
    mean = sum(t) / len(t)
    value = ncells / mean
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(ncells),
                   "parallelism": "host threads (OpenMP cell-parallel, rayon-style per-thread triplets)"},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": cores, "kind": "port",
                         "sample": f"full workload, {args.steps} timed steps"},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def timed_assembly(ctx, mats, flush, stream, steps, warmup, world):
    """W untimed steps, then K steps each bracketed by CUDA events on the
    library's stream (L2 flushed before each, outside the events), then a second
    pass of the same steps with CUDA events around every kernel for the element
    / scatter split (events inside the timed steps would perturb them)."""
    import torch

    import formoniq_gb300 as fq

    def step():
        fq.Matrix.reassemble_many(mats)  # the forms queued back to back, one status read

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    launches0 = ctx.kernel_launches
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for i in range(steps):
        flush.fill_(float(i))
        evs[i][0].record(stream)
        step()
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = ctx.kernel_launches - launches0
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / steps, world)
    ctx.profile(reset=True)
    ctx.set_profiling(True)
    for i in range(steps):
        flush.fill_(float(i))
        step()
    torch.cuda.synchronize()
    ctx.set_profiling(False)
    (el_ms, sc_ms), (el_n, sc_n) = ctx.profile(reset=True)
    return dict(ms=ms, wall=wall, launches=launches, el_ms=el_ms, sc_ms=sc_ms, el_n=el_n, sc_n=sc_n)


def run_ours(args):
    import torch

    import formoniq_gb300 as fq

    rank, local_rank, world = env_rank()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream()  # a real stream: the library launches on it and the events time it
    torch.cuda.set_stream(stream)
    ctx = fq.Context(local_rank, stream=stream.cuda_stream)
    mesh = fq.Mesh.kuhn_cube(ctx, DIM, NBOX)
    mesh.kuhn_lengths(jitter=JITTER, seed=SEED + rank)
    ncells = mesh.ncells()
    t0 = time.perf_counter()
    mats = [getattr(fq.WhitneyComplex(mesh), name)(k) for name, k in FORMS]  # patterns and plans built here
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    mats_ieee = [getattr(fq.WhitneyComplex(mesh, precision=fq.FQ_FP64_IEEE), name)(k) for name, k in FORMS]
    torch.cuda.synchronize()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    # the clock sampler starts before the warm-up: its process start-up stays out of the timed steps
    with ClockSampler(local_rank) as clocks:
        time.sleep(0.5)
        main = timed_assembly(ctx, mats, flush, stream, args.steps, args.warmup, world)
        ieee = timed_assembly(ctx, mats_ieee, flush, stream, args.steps, args.warmup, world)
        solve = None if args.no_solve else solve_phase(fq, torch, mesh, stream, args)
    ms = main["ms"]
    value = world * ncells / (ms * 1e-3)
    roofline = roofline_record(ctx, mesh, mats, ncells, ms, main)
    ieee_roof = roofline_record(ctx, mesh, mats_ieee, ncells, ieee["ms"], ieee)
    ieee_rec = {"value": world * ncells / (ieee["ms"] * 1e-3), "unit": "cells/s", "ms_per_step": ieee["ms"],
                "dtype": "f64 (IEEE binary64 throughout)", "element_ms_per_step": ieee_roof["element_ms_per_step"],
                "scatter_ms_per_step": ieee_roof["scatter_ms_per_step"],
                "scatter_frac": ieee_roof["scatter_GBps"] / ieee_roof["peak"],
                "fused_assembly_frac": ieee_roof["fused_assembly_frac"]}
    e2e = None if args.no_e2e else e2e_phase(ctx, mesh, mats, flush, args, ncells, world)
    cpu = parity = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cnc, ct, cores, omats = cpu_assembly(NBOX, 1)
        cpu = {"value": cnc / ct[0], "unit": "cells/s", "cores": cores, "kind": "port",
               "sample": f"one full step ({cnc} tets, 4 forms), oracle C++/OpenMP assembly"}
        fq.Matrix.reassemble_many(mats)
        fq.Matrix.reassemble_many(mats_ieee)
        parity = {"fp64_float_float": parity_record(mats, omats), "fp64_ieee": parity_record(mats_ieee, omats)}
    sub = {}
    if world == 1 and not args.no_sub:
        # compact forms of the batch, precision and serving workloads, in the
        # same run as the headline so that one clock covers them
        for name, fn in (("batch", batch_study), ("precision", precision_study), ("serve", serve_study)):
            t0 = time.perf_counter()
            try:
                sub[name] = fn(args, compact=True)
            except Exception as e:  # reported, not hidden: the line still prints
                sub[name] = {"error": f"{type(e).__name__}: {e}"}
            sub[name]["study_wall_s"] = time.perf_counter() - t0
    line = {
        "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPE_FP64, "precision_mode": "FQ_FP64", "data": "synthetic",
        "config": {"workload": workload_name(ncells),
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{world}",
                   "setup_s_pattern_and_permutation": round(setup_s, 3)},
        "roofline": roofline,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "gpu_launches": main["launches"],
        "clocks": clocks.summary(),
        "wall_s_timed": main["wall"],
        "ieee_fp64": ieee_rec,
        "parity": parity,
        "solve": solve,
        **sub,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


# DRAM bytes (read + write) of the step's four scatter launches in FQ_FP64 on
# the 3D 32^3 workload, from one ncu capture of the current kernels (--metrics
# dram__bytes_read.sum,dram__bytes_write.sum --cache-control none; its summary
# is kept under profiles/): the bench cannot run ncu itself, so the line
# carries the captured figure and says so.
SCATTER_TRAFFIC_3D32_FP64 = 251_345_920 + 116_041_984


def roofline_record(ctx, mesh, mats, ncells, ms, t):
    """Algorithmic bytes per launch of each kernel (per form, summed over the
    step's forms) over its CUDA-event time on the launching stream."""
    n = DIM
    n1 = mesh.nsimplices(1)
    el_bytes = sc_bytes = fused_bytes = 0
    for (name, k), m in zip(FORMS, mats):
        lr, lc, sym = local_shape(n, name, k)
        nent = lr * (lr + 1) // 2 if sym else lr * lc
        _, _, nnz, prec = m.info()
        w = 4 if prec == 1 else 8
        el_bytes += n1 * 8 + ncells * comb(n + 1, 2) * 4 + ncells * nent * w
        # the scatter's compulsory bytes for this plan (the library's count):
        # symmetric plans gather every packed element entry once, read one
        # 16-byte record per upper slot (slot, mirror, first two contributions)
        # and the plan indices of the slots with more than two, and write every
        # slot's value
        sc_bytes += m.scatter_bytes()
        tg = k - 1 if name == "dif_both" else k
        fused_bytes += n1 * 8 + ncells * (n + 1) * 4 + ncells * 2 * comb(n + 1, tg + 1) * 4 + nnz * w
    el_avg = t["el_ms"] / max(t["el_n"], 1) * len(FORMS)  # per step, all forms
    sc_avg = t["sc_ms"] / max(t["sc_n"], 1) * len(FORMS)
    hbm_peak, peak_src = measured_peaks()
    dominant = "element" if el_avg >= sc_avg else "scatter"
    dom_bytes, dom_ms = (el_bytes, el_avg) if dominant == "element" else (sc_bytes, sc_avg)
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    fused_gbps = fused_bytes / (ms * 1e-3) / 1e9
    fp64 = all(m.info()[3] == 0 for m in mats)
    traffic = SCATTER_TRAFFIC_3D32_FP64 if (dominant == "scatter" and fp64 and n == 3 and ncells == 6 * NBOX ** 3) \
        else None
    return {"kernel": dominant, "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "traffic": traffic,
            "traffic_source": "ncu capture of the four scatter launches of one step (per step, like achieved)"
            if traffic else None,
            "traffic_over_algorithmic": traffic / dom_bytes if traffic else None, "peak_source": peak_src,
            "algorithmic_bytes_per_step": dom_bytes, "kernel_ms_per_step": dom_ms,
            "element_ms_per_step": el_avg, "scatter_ms_per_step": sc_avg,
            "element_bytes_per_step": el_bytes, "scatter_bytes_per_step": sc_bytes,
            "scatter_GBps": sc_bytes / (sc_avg * 1e-3) / 1e9,
            "fp64_fma_peak_tflops_measured": ctx.fma_peak_tflops(True),
            "fp32_fma_peak_tflops_measured": ctx.fma_peak_tflops(False),
            "fused_assembly_bytes_per_step": fused_bytes, "fused_assembly_GBps": fused_gbps,
            "fused_assembly_frac": fused_gbps / hbm_peak}


def solve_phase(fq, torch, mesh, stream, args):
    """Mixed k=1 Hodge-Laplace, MINRES to 1e-10 on the resident problem, FP64;
    then the same problem with an FP32 inner MINRES inside FP64 iterative
    refinement, its error stated against the FP64 solution."""
    pc = {"auto": fq.FQ_PC_AUTO, "jacobi": fq.FQ_PC_JACOBI, "hx": fq.FQ_PC_HX}[args.pc]
    rng = np.random.default_rng(SEED)
    src = torch.tensor(rng.standard_normal(mesh.nsimplices(1)), device="cuda")
    out = {}
    ref = None
    for label, prec in (("fp64", fq.FQ_FP64), ("fp32_refined", fq.FQ_FP32)):
        t0 = time.perf_counter()
        prob = fq.MixedProblem(mesh, 1, fq.FQ_ABSOLUTE, prec)
        ns, nu, nh, sys_nnz = prob.info()
        sig = torch.empty(mesh.nsimplices(0), dtype=torch.float64, device="cuda")
        u = torch.empty(mesh.nsimplices(1), dtype=torch.float64, device="cuda")
        if prec == fq.FQ_FP64:
            opts = fq.SolveOpts.default(rtol=1e-10, max_iters=args.max_iters, preconditioner=pc)
        else:
            opts = fq.SolveOpts.default(rtol=1e-5, max_iters=args.max_iters, precision=fq.FQ_FP32,
                                        refine_rtol=1e-10, max_refinements=8, preconditioner=pc)
        torch.cuda.synchronize()
        prob.solve_device(src.data_ptr(), sig.data_ptr(), u.data_ptr(), 0, opts)  # warm-up, builds the preconditioner
        torch.cuda.synchronize()
        setup_ms = (time.perf_counter() - t0) * 1e3
        lat, reps = [], []
        for _ in range(args.solves):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            reps.append(prob.solve_device(src.data_ptr(), sig.data_ptr(), u.data_ptr(), 0, opts))
            b.record(stream)
            torch.cuda.synchronize()
            lat.append(a.elapsed_time(b))
        x = torch.cat([sig, u]).cpu().numpy()
        prob.close()
        if not lat:
            continue
        lat_sorted = sorted(lat)

        def pct(p):
            return lat_sorted[min(len(lat_sorted) - 1, int(math.ceil(p / 100 * len(lat_sorted))) - 1)]

        rec = {"problem": f"mixed k=1 Hodge-Laplace, {ns + nu + nh} DOFs, {sys_nnz} nnz",
               "preconditioner": args.pc, "solves_per_s": 1e3 / (sum(lat) / len(lat)), "p50_ms": pct(50),
               "p99_ms": pct(99), "setup_ms_first_solve": setup_ms, "iters": reps[-1].iters,
               "refinements": reps[-1].refinements,
               "ms_per_iter": (sum(lat) / len(lat)) / max(reps[-1].iters, 1),
               "true_residual": reps[-1].true_residual, "converged": all(r.converged for r in reps), "n": len(lat)}
        if ref is None:
            ref = x
            rec["stop"] = "MINRES preconditioned residual 1e-10"
        else:
            rec["stop"] = "FP64 residual 1e-10 (FP32 inner MINRES to 1e-5)"
            rec["rel_err_vs_fp64_solve"] = float(np.linalg.norm(x - ref) / np.linalg.norm(ref))
        out[label] = rec
    return out or None


def e2e_phase(ctx, mesh, mats, flush, args, ncells, world):
    """The same metric through the C-ABI call with host buffers
    (fq_assemble_host_many): every step uploads the lengths (H2D) once and
    downloads every matrix's values (D2H) into pinned host buffers."""
    import ctypes

    import torch

    lengths_h = torch.from_numpy(mesh.lengths_sq()).pin_memory()
    outs = [torch.empty(m.nnz, dtype=torch.float64).pin_memory() for m in mats]
    lp = ctypes.cast(lengths_h.data_ptr(), ctypes.POINTER(ctypes.c_double))

    mat_arr = (ctypes.c_void_p * len(mats))(*[m.h for m in mats])
    out_arr = (ctypes.c_void_p * len(mats))(*[o.data_ptr() for o in outs])

    def e2e_step():
        ctx.check(ctx.L.fq_assemble_host_many(ctx.h, mesh.h, lp, mat_arr, out_arr, len(mats)),
                  "fq_assemble_host_many")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    torch.cuda.synchronize()
    e_ms = []
    for i in range(args.steps):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t = time.perf_counter()
        e2e_step()
        e_ms.append((time.perf_counter() - t) * 1e3)
    e2e_ms = sum(e_ms) / len(e_ms)
    h2d = lengths_h.numel() * 8
    d2h = sum(o.numel() * 8 for o in outs)
    return {"value": world * ncells / (e2e_ms * 1e-3), "unit": "cells/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
            "link": link_floor(h2d, d2h, e2e_ms)}


def link_floor(h2d: int, d2h: int, e2e_ms: float) -> dict:
    """The host link's bound on the end-to-end step: plain pinned copies of the
    step's byte counts (one copy each way, CUDA events on the current stream).
    Splitting a download over several streams, or storing into the pinned
    buffer from the SMs, moves no more bytes per second than one copy-engine
    copy, so the sum of the two copy times is the step's floor."""
    import torch

    hd = torch.empty(max(h2d // 8, 1), dtype=torch.float64).pin_memory()
    dd = torch.empty(max(h2d // 8, 1), dtype=torch.float64, device="cuda")
    ds = torch.empty(max(d2h // 8, 1), dtype=torch.float64, device="cuda")
    hs = torch.empty(max(d2h // 8, 1), dtype=torch.float64).pin_memory()

    def copy_ms(dst, src, reps=10):
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    up_ms, down_ms = copy_ms(dd, hd), copy_ms(hs, ds)
    floor_ms = up_ms + down_ms
    return {"h2d_GBps": hd.numel() * 8 / up_ms / 1e6, "d2h_GBps": hs.numel() * 8 / down_ms / 1e6,
            "floor_ms": floor_ms, "frac": floor_ms / e2e_ms}


# ---------------------------------------------------------------------------
# precision workload: 4D 12^4 Kuhn, k=2 mixed Hodge-Laplace
# ---------------------------------------------------------------------------

def precision_study(args, compact: bool):
    """4D 12^4 Kuhn, k=2 mixed Hodge-Laplace (1,483,536 DOFs): FP32 element
    matrices and SpMV with FP64 Gram inverse/determinant inside FP64 iterative
    refinement, against the plain FP64 path. Each result's relative error is
    stated against an FP64 solve at rtol 1e-12 on the device and, in the full
    study, against the oracle's CPU MINRES at rtol 1e-12 on the oracle's own
    KKT system. The KKT product's achieved HBM bandwidth (the system, 1.1 GB,
    does not fit L2) is measured with L2 flushed before every product."""
    import torch

    import formoniq_gb300 as fq

    dim, nbox, grade = 4, 12, 2
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = fq.Context(0, stream=stream.cuda_stream)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nbox)
    mesh.kuhn_lengths(jitter=JITTER, seed=SEED)
    rng = np.random.default_rng(SEED + 4)
    src_h = rng.standard_normal(mesh.nsimplices(grade))
    src = torch.tensor(src_h, device="cuda")
    sig = torch.empty(mesh.nsimplices(grade - 1), dtype=torch.float64, device="cuda")
    u = torch.empty(mesh.nsimplices(grade), dtype=torch.float64, device="cuda")
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    nsolves = 3 if compact else args.solves

    def timed_solves(prob, opts, n):
        prob.solve_device(src.data_ptr(), sig.data_ptr(), u.data_ptr(), 0, opts)  # builds the preconditioner
        lat, rep = [], None
        for _ in range(n):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            rep = prob.solve_device(src.data_ptr(), sig.data_ptr(), u.data_ptr(), 0, opts)
            b.record(stream)
            torch.cuda.synchronize()
            lat.append(a.elapsed_time(b))
        return torch.cat([sig, u]).cpu().numpy(), sorted(lat), rep

    def timed(fn, n=3):
        fn()
        torch.cuda.synchronize()
        t = []
        for _ in range(n):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            t.append(a.elapsed_time(b))
        return statistics.median(t)

    out = {"metric": "solves/s @1e-8 rel err vs the FP64 oracle", "workload":
           f"kuhn {dim}D {nbox}^4 ({mesh.ncells()} cells), k={grade} mixed Hodge-Laplace, N(0,1) source seed {SEED + 4}",
           "data": "synthetic", "n_solves": nsolves}
    t0 = time.perf_counter()
    p64 = fq.MixedProblem(mesh, grade, fq.FQ_ABSOLUTE, fq.FQ_FP64)
    out["setup_fp64_s"] = time.perf_counter() - t0
    ns, nu, nh, nnz = p64.info()
    out["dofs"], out["kkt_nnz"] = ns + nu + nh, nnz
    ref, _, rref = timed_solves(p64, fq.SolveOpts.default(rtol=1e-12, max_iters=args.max_iters), 1)
    out["fp64_rtol_1e-12"] = {"iters": rref.iters, "true_residual": rref.true_residual}
    # the KKT product on the device (SpMV roofline: nnz (8 + 4) + (n + 1) 4 + 2 n 8 bytes)
    kkt = p64.system()
    n = ns + nu + nh
    xv = torch.tensor(rng.standard_normal(n), device="cuda")
    yv = torch.empty_like(xv)
    ms_spmv = timed(lambda: ctx.check(ctx.L.fq_spmv(ctx.h, kkt.h, fq._P(xv.data_ptr()), fq._P(yv.data_ptr()))), 5)
    spmv_bytes = nnz * 12 + (n + 1) * 4 + 2 * n * 8
    peak, peak_src = measured_peaks()
    out["spmv"] = {"matrix": f"FP64 KKT, {n} rows, {nnz} nnz ({nnz * 12 / 1e9:.2f} GB of values and columns)",
                   "ms": ms_spmv, "algorithmic_bytes": spmv_bytes, "achieved_GBps": spmv_bytes / (ms_spmv * 1e6),
                   "peak_GBps": peak, "peak_source": peak_src, "frac": spmv_bytes / (ms_spmv * 1e6) / peak,
                   "l2": "flushed before every product (256 MiB write)"}
    variants = [("fp64", p64, fq.SolveOpts.default(rtol=1e-10, max_iters=args.max_iters))]
    t0 = time.perf_counter()
    p32 = fq.MixedProblem(mesh, grade, fq.FQ_ABSOLUTE, fq.FQ_FP32)
    out["setup_fp32_s"] = time.perf_counter() - t0
    variants.append(("fp32_refined", p32, fq.SolveOpts.default(rtol=1e-5, max_iters=args.max_iters,
                                                                precision=fq.FQ_FP32, refine_rtol=1e-10,
                                                                max_refinements=8)))
    sols = {}
    for label, prob, opts in variants:
        x, lat, rep = timed_solves(prob, opts, nsolves)
        sols[label] = x
        mean = sum(lat) / len(lat)
        out[label] = {"solves_per_s": 1e3 / mean, "p50_ms": lat[(len(lat) - 1) // 2], "p99_ms": lat[-1],
                      "iters": rep.iters, "refinements": rep.refinements, "true_residual": rep.true_residual,
                      "rel_err_vs_fp64_rtol_1e-12": float(np.linalg.norm(x - ref) / np.linalg.norm(ref)),
                      "kkt_assembly_ms": timed(prob.reassemble)}
    p32.close()
    p64.close()
    mesh.close()
    ctx.close()
    if not compact:
        # the oracle on the host: its own KKT system of the same mesh, lengths and
        # source, MINRES at rtol 1e-12 (the solution does not depend on the
        # preconditioner; the oracle uses its restatement of the HX blocks)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import hx_oracle
        import oracle

        t0 = time.perf_counter()
        cx, coords = oracle.cartesian_unit(dim, nbox)
        coords = oracle.jitter_coords(coords, nbox, SEED, JITTER)
        lengths = cx.edge_lengths_sq(coords)
        wc = oracle.WhitneyComplex(cx, lengths)
        a, rhs, ons, onu = oracle.assemble_mixed_kkt(wc, src_h, grade, oracle.harmonics(wc, grade))
        hx = hx_oracle.HxPreconditioner(wc, cx, lengths, nbox, False)

        def pc(r):
            return np.concatenate([hx.apply(grade - 1, r[:ons]), hx.apply(grade, r[ons:ons + onu]), r[ons + onu:]])

        xo, orep = oracle.minres(a, pc, rhs, rtol=1e-12)
        out["cpu_oracle"] = {"rtol": 1e-12, "iters": orep.iters, "converged": orep.converged,
                             "seconds": time.perf_counter() - t0, "cores": oracle.num_threads()}
        for label, x in sols.items():
            out[label]["rel_err_vs_cpu_oracle"] = float(np.linalg.norm(x - xo) / np.linalg.norm(xo))
    return out


def run_precision(args):
    print(json.dumps(precision_study(args, compact=False)))


# ---------------------------------------------------------------------------
# serving workload: a Poisson stream of Hodge-Laplace and Minkowski Dirac solves
# ---------------------------------------------------------------------------

def serve_stream(fq, n, seed, rate_per_s, max_cells_hodge=5e5, max_cells_dirac=3e5):
    """Seeded request stream: half (i) Riemannian Kuhn n in {2,3,4}, cells
    log-uniform in [1e3, 5e5], k uniform in 0..n, bc uniform, jittered 0.1h,
    Hodge-Laplace source problem; half (ii) Minkowski 1+2 Kuhn, cells in
    [1e3, 3e5], squared lengths s(1 + U(-0.05, 0.05)), Dirac with m = 1.5."""
    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    for i in range(n):
        t += rng.exponential(1.0 / rate_per_s)
        if rng.random() < 0.5:
            dim = int(rng.integers(2, 5))
            cells = math.exp(rng.uniform(math.log(1e3), math.log(max_cells_hodge)))
            nb = max(1, round((cells / math.factorial(dim)) ** (1.0 / dim)))
            reqs.append(dict(kind=fq.FQ_REQ_HODGE, dim=dim, nbox=nb, grade=int(rng.integers(0, dim + 1)),
                             bc=int(rng.integers(0, 2)), jitter=0.1, seed=seed * 100003 + i, arrival_ms=t * 1e3))
        else:
            cells = math.exp(rng.uniform(math.log(1e3), math.log(max_cells_dirac)))
            nb = max(1, round((cells / 6.0) ** (1.0 / 3.0)))
            reqs.append(dict(kind=fq.FQ_REQ_DIRAC, dim=3, nbox=nb, minkowski=True, jitter=0.05, mass_term=1.5,
                             seed=seed * 100003 + i, arrival_ms=t * 1e3))
    return reqs


def run_stream(fq, reqs, lanes, cache, mixed_precision, dirac_iters, sols=None, inputs=None, tight=False):
    """Submit the whole stream (the server releases each request at its
    arrival time); returns per-request results in stream order. sols[i], when
    given, receives request i's solution; inputs[i] = (lengths, source) pins a
    request's inputs. tight: FP64 solves to rtol 1e-13 (the accuracy reference
    of the sampled requests)."""
    fp64 = fq.SolveOpts.default(rtol=1e-13 if tight else 1e-10, max_iters=40_000 if tight else 10_000)
    fp32 = fq.SolveOpts.default(rtol=1e-5, precision=fq.FQ_FP32, refine_rtol=1e-10, max_refinements=8)
    dirac = fq.SolveOpts.default(rtol=1e-13 if tight else 1e-10, max_iters=dirac_iters)
    with fq.Server(lanes=lanes, cache=cache) as srv:
        t0 = time.perf_counter()
        tickets = []
        for i, r in enumerate(reqs):
            if r["kind"] == fq.FQ_REQ_DIRAC:
                opts = dirac
            else:
                opts = fp32 if mixed_precision else fp64
            extra = {}
            if sols is not None and sols[i] is not None:
                extra["solution"] = sols[i]
            if inputs is not None and inputs.get(i) is not None:
                extra["lengths"], extra["source"] = inputs[i]
            tickets.append(srv.submit(**r, opts=opts, **extra))
        res = [srv.wait(t) for t in tickets]
        wall = time.perf_counter() - t0
        stats = srv.stats()
    return res, wall, stats


def pct(vals, p):
    v = sorted(vals)
    return v[min(len(v) - 1, max(0, int(math.ceil(p / 100 * len(v))) - 1))] if v else None


def stream_summary(reqs, res, wall, kind=None):
    pairs = [(q, r) for q, r in zip(reqs, res) if kind is None or q["kind"] == kind]
    if not pairs:
        return None
    lat = [r["latency_ms"] for _, r in pairs]
    run = [r["run_ms"] for _, r in pairs]
    que = [r["queue_ms"] for _, r in pairs]
    ok = [r for _, r in pairs if r["status"] == 0 and r["report"].converged]
    first = min(q["arrival_ms"] for q in reqs)
    span_ms = max(r["end_ms"] for r in res) - first
    statuses = collections.Counter(int(r["status"]) for _, r in pairs)
    return {"solves_per_s": len(ok) / (span_ms * 1e-3), "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
            "service_p50_ms": pct(run, 50), "service_p99_ms": pct(run, 99), "mean_service_ms": sum(run) / len(run),
            "queue_p50_ms": pct(que, 50), "queue_p99_ms": pct(que, 99), "converged": len(ok), "n": len(pairs),
            "wall_s": wall, "cache_hits": sum(r["cache_hit"] for _, r in pairs),
            "dirac_on_fp64_class_factors": sum(1 for q, r in pairs if q["kind"] == 1 and r["report"].refinements > 0),
            "statuses": {str(k): v for k, v in sorted(statuses.items())},
            "unconverged": [{"dim": q.get("dim"), "nbox": q.get("nbox"), "grade": q.get("grade"),
                             "status": int(r["status"]), "iters": int(r["report"].iters),
                             "true_residual": float(r["report"].true_residual)}
                            for q, r in pairs if not (r["status"] == 0 and r["report"].converged)][:8]}


def solution_sizes(fq, reqs):
    """Length of each request's solution: (sigma, u) for Hodge, every grade for Dirac."""
    ctx = fq.Context(0)
    counts = {}
    out = []
    for q in reqs:
        key = (q["dim"], q["nbox"])
        if key not in counts:
            m = fq.Mesh.kuhn_cube(ctx, *key)
            counts[key] = [m.nsimplices(k) for k in range(key[0] + 1)]
            m.close()
        ns = counts[key]
        if q["kind"] == fq.FQ_REQ_DIRAC:
            out.append(sum(ns))
        else:
            k = q["grade"]
            out.append((ns[k - 1] if k >= 1 else 0) + ns[k])
    ctx.close()
    return out


def oracle_inputs(q):
    """Host lengths and source of a request and its oracle solution
    (solve_source / solve_dirac_source restated on the host)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    dim, nb = q["dim"], q["nbox"]
    rng = np.random.default_rng(q["seed"])
    if q.get("minkowski"):
        cx, coords, signs = oracle.minkowski(dim, nb)
        lengths = cx.edge_lengths_sq(coords, signs)
        lengths = lengths * (1.0 + q["jitter"] * rng.uniform(-1.0, 1.0, len(lengths)))
    else:
        cx, coords = oracle.cartesian_unit(dim, nb)
        lengths = cx.edge_lengths_sq(oracle.jitter_coords(coords, nb, q["seed"], q["jitter"]))
    if q["kind"] == 1:  # Dirac
        load = rng.standard_normal(sum(cx.nsimplices(k) for k in range(dim + 1)))
        want = oracle.dirac_solve_source(cx, lengths, q["mass_term"], load, np.zeros(len(load)))
        return lengths, load, want
    k = q["grade"]
    src = rng.standard_normal(cx.nsimplices(k))
    wc = oracle.WhitneyComplex(cx, lengths, relative=bool(q["bc"]))
    sigma, u, _, _ = oracle.solve_source(wc, src, k, rtol=1e-12)
    return lengths, src, np.concatenate([sigma, u])


def serve_study(args, compact: bool):
    """The served form (lanes, residency, FP32-inner refinement for Hodge
    requests) against the plain one (one lane, no residency, FP64) on the same
    seeded Poisson stream; every sampled request's served solution against its
    plain solution, and a few small requests against the oracle on the host."""
    import formoniq_gb300 as fq

    nreq = 40 if compact else args.requests
    reqs = serve_stream(fq, nreq, SEED, args.rate)
    sizes = solution_sizes(fq, reqs)
    step = max(1, nreq // 100)
    sample = [i for i in range(nreq) if i % step == 0]
    sols_s = [np.zeros(sizes[i]) if i in sample else None for i in range(nreq)]
    sols_p = [np.zeros(sizes[i]) if i in sample else None for i in range(nreq)]
    # the smallest requests of each kind get host inputs, checked against the oracle
    inputs, wants = {}, {}
    if not compact:
        for kind in (fq.FQ_REQ_HODGE, fq.FQ_REQ_DIRAC):
            idx = sorted((i for i in sample if reqs[i]["kind"] == kind), key=lambda i: sizes[i])[:2]
            for i in idx:
                lengths, src, want = oracle_inputs(reqs[i])
                inputs[i], wants[i] = (lengths, src), want
    served, wall_s, st = run_stream(fq, reqs, args.lanes, True, True, args.dirac_iters, sols_s, inputs)
    plain, wall_p, _ = run_stream(fq, reqs, 1, False, False, args.dirac_iters, sols_p, inputs)
    # the sampled requests again, one lane, solved to rtol 1e-13: the accuracy
    # reference both sides are measured against
    sub = [dict(reqs[i], arrival_ms=0.0) for i in sample]
    sols_t = [np.zeros(sizes[i]) for i in sample]
    tight, _, _ = run_stream(fq, sub, 1, False, False, args.dirac_iters, sols_t,
                             {j: inputs[i] for j, i in enumerate(sample) if i in inputs}, tight=True)
    errs = {"hodge": [], "dirac": []}
    acc = {side: {"hodge": [], "dirac": []} for side in ("served", "plain")}
    for j, i in enumerate(sample):
        kind = "hodge" if reqs[i]["kind"] == fq.FQ_REQ_HODGE else "dirac"
        if served[i]["status"] == 0 and plain[i]["status"] == 0:
            errs[kind].append(float(np.linalg.norm(sols_s[i] - sols_p[i]) / max(np.linalg.norm(sols_p[i]), 1e-300)))
        if tight[j]["status"] == 0:
            ref = max(np.linalg.norm(sols_t[j]), 1e-300)
            for side, sol, res in (("served", sols_s[i], served[i]), ("plain", sols_p[i], plain[i])):
                if res["status"] == 0:
                    acc[side][kind].append(float(np.linalg.norm(sol - sols_t[j]) / ref))
    oracle_errs = [{"kind": "hodge" if reqs[i]["kind"] == fq.FQ_REQ_HODGE else "dirac", "dim": reqs[i]["dim"],
                    "nbox": reqs[i]["nbox"], "dofs": sizes[i],
                    "served_rel_err": float(np.linalg.norm(sols_s[i] - w) / np.linalg.norm(w)),
                    "plain_rel_err": float(np.linalg.norm(sols_p[i] - w) / np.linalg.norm(w))}
                   for i, w in wants.items()]
    kinds = collections.Counter("hodge" if q["kind"] == fq.FQ_REQ_HODGE else "dirac" for q in reqs)

    def side(res, wall, **kw):
        return dict(all=stream_summary(reqs, res, wall), hodge=stream_summary(reqs, res, wall, fq.FQ_REQ_HODGE),
                    dirac=stream_summary(reqs, res, wall, fq.FQ_REQ_DIRAC), **kw)

    return {"metric": "solves/s and p50/p99 latency, served vs plain", "requests": len(reqs), "rate_per_s": args.rate,
            "mix": dict(kinds), "data": "synthetic (seeded Poisson stream)", "dirac_max_iters": args.dirac_iters,
            "served": side(served, wall_s, lanes=args.lanes, cache=True,
                           precision="FP32 inner MINRES + FP64 refinement (Hodge), FP64 GMRES on sparse LU (Dirac)",
                           peak_committed_gb=st["peak_committed_bytes"] / 1e9),
            "plain": side(plain, wall_p, lanes=1, cache=False, precision="FP64 (Hodge), FP64 GMRES on sparse LU (Dirac)"),
            "served_vs_plain_rel_err": {k: {"n": len(v), "max": max(v) if v else None,
                                            "median": statistics.median(v) if v else None} for k, v in errs.items()},
            "rel_err_vs_tight_solve": {side: {k: {"n": len(v), "max": max(v) if v else None,
                                                  "median": statistics.median(v) if v else None,
                                                  "over_1e-8": sum(1 for e in v if e > 1e-8)}
                                              for k, v in d.items()} for side, d in acc.items()},
            "tight_solve": "the sampled requests re-solved on one lane in FP64 to rtol 1e-13 (MINRES; GMRES on the "
                           "sparse LU for Dirac, stopping at its backward-error floor)",
            "sampled_requests": len(sample), "vs_cpu_oracle": oracle_errs}


def run_serve(args):
    print(json.dumps(serve_study(args, compact=False)))


# ---------------------------------------------------------------------------
# batching workload: 512 Kuhn meshes of uneven dimension, size and degree
# ---------------------------------------------------------------------------

def batch_specs(n, seed):
    """n in U{2,3,4}, cells log-uniform in [1e3, 2e5], N = max(1, round((cells/n!)^(1/n))),
    k in U{0..n}."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        dim = int(rng.integers(2, 5))
        cells = math.exp(rng.uniform(math.log(1e3), math.log(2e5)))
        nb = max(1, round((cells / math.factorial(dim)) ** (1.0 / dim)))
        specs.append((dim, nb, int(rng.integers(0, dim + 1))))
    return specs


def batch_study(args, compact: bool):
    import torch

    import formoniq_gb300 as fq

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = fq.Context(0, stream=stream.cuda_stream)
    specs = batch_specs(128 if compact else args.meshes, SEED + 3)
    t0 = time.perf_counter()
    meshes = []
    for i, (dim, nb, _) in enumerate(specs):
        m = fq.Mesh.kuhn_cube(ctx, dim, nb)
        m.kuhn_lengths(jitter=JITTER, seed=SEED + 1000 + i)
        meshes.append(m)
    grades = [k for _, _, k in specs]
    mesh_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch = fq.Batch(ctx, meshes, grades, fq.FQ_BATCH_HDIF)
    plan_s = time.perf_counter() - t0
    batch.assemble()
    t0 = time.perf_counter()
    batch.tune(reps=1 if compact else 2)
    tune_s = time.perf_counter() - t0
    info = batch.info()
    batch.assemble()  # validates (status words) once with the tuned shape
    # the drop-in path: one fq_reassemble per mesh (element + scatter + status read per mesh)
    mats = [fq.WhitneyComplex(m).hdif_gram(k) for m, k in zip(meshes, grades)]
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def timed(fn, steps):
        ts = []
        for _ in range(steps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    for _ in range(max(3, args.warmup)):
        batch.assemble(check=False)
        batch.assemble_per_mesh(check=False)
    torch.cuda.synchronize()
    reps = min(args.steps, 10) if compact else args.steps
    ms_batched = timed(lambda: batch.assemble(check=False), reps)
    ms_launches = timed(lambda: batch.assemble_per_mesh(check=False), reps)

    def dropin():
        for m, mat in zip(meshes, mats):
            mat.reassemble(m)

    ms_dropin = timed(dropin, max(1, reps // 2))
    # the element pass as one fused launch over every class (same values), at
    # each grid, against the tuned per-class launches above
    fused = {"registers_per_thread": batch.fused_registers(), "ms_by_grid": {}}
    for per_sm in (0, 2, 4, 8):
        batch.set_element_launch(True, per_sm * 152)
        for _ in range(3):
            batch.assemble(check=False)
        fused["ms_by_grid"][f"{per_sm}_per_sm" if per_sm else "one_thread_per_cell"] = timed(
            lambda: batch.assemble(check=False), reps)
    batch.set_element_launch(False)
    fused["best_ms"] = min(fused["ms_by_grid"].values())
    fused["cells_per_s"] = info["cells"] / (fused["best_ms"] * 1e-3)
    fused["launches"] = 2
    cells = info["cells"]
    out = {"metric": "assembled cells/s (batched vs per-mesh launches)", "meshes": len(meshes),
           "form": "hdif_gram(k) = M_k + dif_both(k+1), FP64 values (float-float compute)",
           "workload": f"{len(meshes)} Kuhn cubes, n in {{2,3,4}}, cells log-uniform [1e3, 2e5], k in 0..n, "
                       f"seed {SEED + 3}", "data": "synthetic",
           "cells": cells, "slots": info["slots"], "classes": info["classes"],
           "launches_batched": info["launches_per_assembly"], "launches_per_mesh": 2 * len(meshes),
           "tuned": {"scatter_threads_per_slot": info["scatter_threads_per_slot"],
                     "scatter_grid": info["scatter_grid"], "element_grids": info["element_grids"]},
           "batched": {"ms": ms_batched, "cells_per_s": cells / (ms_batched * 1e-3)},
           "per_mesh_launches": {"ms": ms_launches, "cells_per_s": cells / (ms_launches * 1e-3)},
           "per_mesh_dropin_reassemble": {"ms": ms_dropin, "cells_per_s": cells / (ms_dropin * 1e-3)},
           "fused_single_element_launch": fused,
           "setup_s": {"meshes": mesh_s, "plans": plan_s, "tune": tune_s},
           "l2": "flushed before every timed assembly (256 MiB write)"}
    for m in mats:
        m.close()
    batch.close()
    for m in meshes:
        m.close()
    ctx.close()
    return out


def run_batch(args):
    print(json.dumps(batch_study(args, compact=False)))


# ---------------------------------------------------------------------------
# scatter launch shapes on the headline step
# ---------------------------------------------------------------------------

def run_shapes(args):
    """The headline step (3D 32^3, the four forms) with every launch shape of
    the symmetric scatter (fq_ctx_set_scatter_shape: slots per thread 0 = one
    thread per upper slot, 1-8 on a persistent grid; CTAs per SM 0 = as many as
    are resident) in each precision mode; --steps timed steps after --warmup,
    L2 flushed before each, per-kernel split from the profiled pass."""
    import torch

    import formoniq_gb300 as fq

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = fq.Context(0, stream=stream.cuda_stream)
    mesh = fq.Mesh.kuhn_cube(ctx, DIM, NBOX)
    mesh.kuhn_lengths(jitter=JITTER, seed=SEED)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    out = {"metric": "ms per assembly step by scatter launch shape", "workload": workload_name(mesh.ncells()),
           "shapes": []}
    for prec, label in ((fq.FQ_FP64, "fp64 float-float"), (fq.FQ_FP64_IEEE, "fp64 ieee"), (fq.FQ_FP32, "fp32")):
        mats = [getattr(fq.WhitneyComplex(mesh, precision=prec), name)(k) for name, k in FORMS]
        for spt in (-1, 0, 1, 2, 4, 8):
            for bps in ((0,) if spt <= 0 else (0, 2, 4, 8)):
                ctx.set_scatter_shape(spt, bps)
                t = timed_assembly(ctx, mats, flush, stream, args.steps, args.warmup, 1)
                out["shapes"].append({"precision": label, "slots_per_thread": spt, "blocks_per_sm": bps,
                                      "ms_per_step": t["ms"], "element_ms": t["el_ms"] / max(t["el_n"], 1) * len(FORMS),
                                      "scatter_ms": t["sc_ms"] / max(t["sc_n"], 1) * len(FORMS)})
        ctx.set_scatter_shape(-1, 0)
        for m in mats:
            m.close()
    mesh.close()
    ctx.close()
    print(json.dumps(out))


# ---------------------------------------------------------------------------
# Dirac workload: direct Lorentzian Dirac solves at the served stream's sizes
# ---------------------------------------------------------------------------

def run_dirac(args):
    """The served stream's Lorentzian requests one size at a time: Minkowski
    1+2 Kuhn boxes (time axis 0.7), squared lengths s (1 + U(-0.05, 0.05)),
    the relative Hodge-Dirac source problem at m = 1.5 and at m = 0 (bordered
    with the top harmonic) through fq.solve_dirac_source with host buffers.
    Per size: the sparse direct solver's analysis, its FP32, float-float
    (FQ_FP64, the default for FP64 factors) and IEEE FP64 factorizations timed
    with CUDA events (TFLOP/s of the factor's flops),
    and the end-to-end solve (wall clock, median of --solves after one
    untimed call that builds the analysis). Sizes up to 8 boxes per axis are
    checked against the oracle's LU solve on the same inputs, which is also
    timed as the CPU baseline. The Lorentzian mixed k = 1 source problem on
    the same box goes through the same solver (its `mixed_k1` record)."""
    import torch

    import formoniq_gb300 as fq

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = fq.Context(0, stream=stream.cuda_stream)
    sizes = [int(a) for a in args.dirac_sizes.split(",")]
    side = np.array([0.7, 1.0, 1.0])
    signs = np.array([-1.0, 1.0, 1.0])
    out = {"metric": "Dirac solves/s (direct route) by mesh size", "data": "synthetic (seeded Minkowski 1+2 boxes)",
           "rtol": 1e-10, "max_iters": args.dirac_iters, "sizes": []}
    for nb in sizes:
        mesh = fq.Mesh.kuhn_cube(ctx, 3, nb)
        mesh.kuhn_lengths(side=side, ambient_signs=signs, jitter=0.0, seed=0)
        rng = np.random.default_rng(SEED + nb)
        lengths = mesh.lengths_sq() * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, mesh.nsimplices(1)))
        mesh.set_lengths_sq(lengths)
        ntot = sum(mesh.nsimplices(k) for k in range(4))
        load = rng.standard_normal(ntot)
        rec = {"nbox": nb, "cells": mesh.ncells(), "unknowns_full": ntot}
        # the factorizations of the m = 1.5 system
        a = fq.dirac_system(mesh, 1.5)
        t0 = time.perf_counter()
        lu = fq.SparseLu(mesh, a)
        torch.cuda.synchronize()
        rec["analyse_s"] = time.perf_counter() - t0
        info = lu.info()
        rec.update(unknowns=int(a.shape[0]), fronts=int(info["fronts"]), levels=int(info["levels"]),
                   factor_gflop=info["flops"] / 1e9, factor_gb=info["factor_bytes"] / 1e9)
        for name, prec in (("fp32", fq.FQ_FP32), ("fp64", fq.FQ_FP64), ("fp64_ieee", fq.FQ_FP64_IEEE)):
            lu.factor(prec)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lu.factor(prec)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            rec[f"factor_{name}_ms"] = ms
            rec[f"factor_{name}_tflops"] = info["flops"] / (ms * 1e9)
            rec[f"perturbed_{name}"] = int(lu.info()["perturbed_pivots"])
        # the FP32 factors alone (no FP64 refactorization), GMRES to rtol or 500 iterations
        # (the FP64 factors are still in place from the loop above; replace them first)
        lu.factor(fq.FQ_FP32)
        bvec = torch.tensor(rng.standard_normal(a.shape[0]), device="cuda")
        xvec = torch.empty_like(bvec)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rep32 = lu.solve_device(bvec.data_ptr(), xvec.data_ptr(),
                                fq.SolveOpts.default(rtol=1e-10, max_iters=500, max_refinements=0))
        e1.record(stream)
        torch.cuda.synchronize()
        rec["fp32_factors_only"] = {"gmres_iters": int(rep32.iters), "converged": bool(rep32.converged),
                                    "true_residual": float(rep32.true_residual), "solve_ms": e0.elapsed_time(e1)}
        lu.close()
        a.close()
        for mass in (1.5, 0.0):
            opts = fq.SolveOpts.default(rtol=1e-10, max_iters=args.dirac_iters)
            x, rep = fq.solve_dirac_source(mesh, mass, load, None, opts)
            ts = []
            for _ in range(max(1, args.solves)):
                t0 = time.perf_counter()
                x, rep = fq.solve_dirac_source(mesh, mass, load, None, opts)
                ts.append((time.perf_counter() - t0) * 1e3)
            key = "m1.5" if mass else "m0"
            r = {"e2e_ms": statistics.median(ts), "solves_per_s": 1e3 / statistics.median(ts),
                 "gmres_iters": int(rep.iters), "fp64_factors": int(rep.refinements),
                 "converged": bool(rep.converged), "true_residual": float(rep.true_residual)}
            if nb <= 8 and not args.no_cpu:
                sys.path.insert(0, os.path.join(ROOT, "oracle"))
                import oracle

                cx, _, _ = oracle.minkowski(3, nb)
                t0 = time.perf_counter()
                want = oracle.dirac_solve_source(cx, lengths, mass, load, np.zeros(ntot))
                cpu_ms = (time.perf_counter() - t0) * 1e3
                r["rel_err_vs_oracle"] = float(np.linalg.norm(x - want) / np.linalg.norm(want))
                r["cpu_baseline"] = {"ms": cpu_ms, "kind": "port", "cores": 1,
                                     "sample": "oracle.dirac_solve_source (SciPy SuperLU), same inputs"}
            rec[key] = r
        # the Lorentzian mixed k = 1 source problem on the same box: no SPD block
        # preconditioner exists (indefinite hdif_gram), so the signature guard
        # sends it to the sparse direct solver (FP32 factors first)
        src = rng.standard_normal(mesh.nsimplices(1))
        prob = fq.MixedProblem(mesh, 1, fq.FQ_ABSOLUTE, fq.FQ_FP64)
        mopts = fq.SolveOpts.default(rtol=1e-10, max_iters=args.dirac_iters)
        t0 = time.perf_counter()
        _, _, _, frep = prob.solve(src, mopts)  # analysis and factorization, then GMRES
        first_ms = (time.perf_counter() - t0) * 1e3
        ts = []
        for _ in range(max(1, args.solves)):
            t0 = time.perf_counter()
            _, _, _, mrep = prob.solve(src, mopts)  # the factors stay resident while the values do
            ts.append((time.perf_counter() - t0) * 1e3)
        rec["mixed_k1"] = {"unknowns": int(prob.info()[0] + prob.info()[1]),
                           "first_solve_ms": first_ms, "first_gmres_iters": int(frep.iters),
                           "first_fp64_factors": int(frep.refinements),
                           "resident_solve_ms": statistics.median(ts), "gmres_iters": int(mrep.iters),
                           "converged": bool(mrep.converged), "true_residual": float(mrep.true_residual)}
        prob.close()
        mesh.close()
        out["sizes"].append(rec)
        print(json.dumps(rec), file=sys.stderr, flush=True)
    ctx.close()
    print(json.dumps(out))


def run_next(args):
    """The rows after the headline path on the 3D 32^3 mesh: the matrix-free
    operator against the assembled SpMV, the right-hand side (the source load
    and the de Rham map) and the Maxwell leapfrog. Each is timed with CUDA
    events on the library's stream around the public call (median of
    --steps, L2 flushed before each), and the host restatement in oracle/ is
    timed once on the same input."""
    import torch

    import formoniq_gb300 as fq

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = fq.Context(0, stream=stream.cuda_stream)
    peak, peak_src = measured_peaks()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    def timed(fn, steps):
        for _ in range(max(1, args.warmup)):
            fn()
        ts = []
        for _ in range(steps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    def host_time(fn):
        t0 = time.perf_counter()
        r = fn()
        return (time.perf_counter() - t0) * 1e3, r

    def lattice(dim, nb, seed):
        """Vertex coordinates of the Kuhn cube (vertex id = sum_a c_a (N+1)^a,
        axis 0 fastest) with a seeded uniform +-0.1h jitter of every coordinate."""
        idx = np.arange((nb + 1) ** dim)
        c = np.stack([(idx // (nb + 1) ** a) % (nb + 1) for a in range(dim)], 1).astype(np.float64) / nb
        return c + JITTER / nb * np.random.default_rng(seed).uniform(-1.0, 1.0, c.shape)

    dim, nb = DIM, NBOX
    coords = lattice(dim, nb, SEED)
    mesh = fq.Mesh.kuhn_cube(ctx, dim, nb)
    mesh.lengths_from_coords(coords)
    lengths = mesh.lengths_sq()
    cx = oracle.Complex.from_cells(oracle.kuhn_cells(dim, nb))  # the host restatement's complex (CPU baseline)
    dcoords = torch.tensor(coords, device="cuda")
    nc, n0, n1 = mesh.ncells(), mesh.nsimplices(0), mesh.nsimplices(1)
    rng = np.random.default_rng(SEED)
    steps = max(3, min(args.steps, 50))
    out = {"metric": "throughput of the rows after the headline path", "workload":
           f"kuhn 3D {nb}^3 ({nc} tets), coordinates jittered 0.1h seed {SEED}", "data": "synthetic",
           "timing": "CUDA events on the library stream around the public call, median, L2 flushed before each",
           "peak_hbm_gbs": peak, "peak_source": peak_src}

    # matrix-free mass (ElementOperator) against the assembled M_1 (SpMV)
    x = torch.tensor(rng.standard_normal(n1), device="cuda")
    y = torch.empty_like(x)
    op = fq.ElementOperator(mesh, fq.FQ_MASS, 1)
    m1 = fq.WhitneyComplex(mesh).mass(1)
    ms_op = timed(lambda: op.apply(x.data_ptr(), y.data_ptr()), steps)
    ms_spmv = timed(lambda: ctx.check(ctx.L.fq_spmv(ctx.h, m1.h, fq._P(x.data_ptr()), fq._P(y.data_ptr()))),
                    steps)
    lf_, lr_ = comb(dim + 1, 2), comb(dim + 1, 2)
    op_bytes = n1 * 8 + nc * (lf_ + lr_) * 4 + n1 * 8 + nc * lr_ * 8 * 2 + nc * lr_ * 4 + (n1 + 1) * 4 + n1 * 8
    spmv_bytes = m1.nnz * 12 + (n1 + 1) * 4 + 2 * n1 * 8
    m1_host = m1.to_scipy()
    xh = x.cpu().numpy()
    cpu_ms, _ = host_time(lambda: m1_host @ xh)
    out["matfree_mass_1"] = {
        "unit": "applies/s", "dofs": n1, "matrix_free": {"ms": ms_op, "per_s": 1e3 / ms_op,
                                                          "algorithmic_bytes": op_bytes,
                                                          "GBps": op_bytes / (ms_op * 1e6)},
        "assembled_spmv": {"ms": ms_spmv, "per_s": 1e3 / ms_spmv, "algorithmic_bytes": spmv_bytes,
                           "GBps": spmv_bytes / (ms_spmv * 1e6), "frac_of_peak": spmv_bytes / (ms_spmv * 1e6) / peak},
        "cpu_baseline": {"ms": cpu_ms, "kind": "port", "cores": 1, "sample": "scipy CSR matvec of the same M_1"}}
    op.close()
    m1.close()

    # source load: SourceForm, k = 1, degree-3 rule, reference-frame values
    for k, degree in ((1, 3), (2, 3)):
        nq = ctx.L.fq_source_npoints(dim, degree)
        vals_h = rng.standard_normal((nc, nq, comb(dim, k)))
        vals = torch.tensor(vals_h, device="cuda")
        ms_src = timed(lambda: fq.source_form(mesh, k, vals, degree), steps)
        nk = mesh.nsimplices(k)
        lf = comb(dim + 1, k + 1)
        src_bytes = vals_h.nbytes + nc * comb(dim + 1, 2) * 4 + n1 * 8 + nc * lf * (8 + 4) + nk * (4 + 8)
        cpu_ms, _ = host_time(lambda: oracle.source_form(cx, lengths, k, vals_h, degree))
        out[f"source_load_{k}"] = {"unit": "cells/s", "quadrature_degree": degree, "nodes": nq, "ms": ms_src,
                                   "per_s": nc / (ms_src * 1e-3), "algorithmic_bytes": src_bytes,
                                   "GBps": src_bytes / (ms_src * 1e6),
                                   "cpu_baseline": {"ms": cpu_ms, "per_s": nc / (cpu_ms * 1e-3), "kind": "port",
                                                    "cores": 1, "sample": "oracle.source_form, numpy, same values"}}

    # de Rham map of a smooth 1-form, degree-3 rule (nodes, field on the device, reduction)
    def field_t(p):
        return torch.stack([torch.sin(p[:, 0]) * p[:, 1], p[:, 2] ** 2, torch.cos(p[:, 1]) - p[:, 0]], 1)

    def field_n(p):
        return np.stack([np.sin(p[:, 0]) * p[:, 1], p[:, 2] ** 2, np.cos(p[:, 1]) - p[:, 0]], 1)

    ms_dr = timed(lambda: fq.derham_map(mesh, dcoords, 1, field_t, 3), steps)
    cpu_ms, _ = host_time(lambda: oracle.derham_map(cx, coords, 1, field_n, 3))
    out["derham_map_1"] = {"unit": "edges/s", "edges": n1, "quadrature_degree": 3, "ms": ms_dr,
                           "per_s": n1 / (ms_dr * 1e-3),
                           "cpu_baseline": {"ms": cpu_ms, "per_s": n1 / (cpu_ms * 1e-3), "kind": "port", "cores": 1,
                                            "sample": "oracle.derham_map, numpy, same field"}}

    # Maxwell leapfrog on the full complex of a 16^3 mesh (all grades, CG mass blocks)
    nbl = 16
    meshl = fq.Mesh.kuhn_cube(ctx, dim, nbl)
    meshl.lengths_from_coords(lattice(dim, nbl, SEED + 1))
    ll = meshl.lengths_sq()
    cxl = oracle.Complex.from_cells(oracle.kuhn_cells(dim, nbl))
    dt = 0.05 / nbl
    lf = fq.Leapfrog(meshl, fq.FQ_ABSOLUTE, dt)
    off = lf.offsets()
    y0 = torch.tensor(rng.standard_normal(int(off[-1])), device="cuda")
    nsteps = 10
    ms_lf = timed(lambda: lf.step(y0, nsteps), max(3, steps // 10))
    owc = oracle.WhitneyComplex(cxl, ll)
    _, _, olf = oracle.leapfrog_for(owc, dt)
    yh = y0.cpu().numpy()

    def cpu_steps():
        y = yh
        for _ in range(2):
            y = olf.step(y)
        return y

    cpu_ms, _ = host_time(cpu_steps)
    out["leapfrog_16"] = {"unit": "steps/s", "mesh": f"kuhn 3D {nbl}^3", "dofs": int(off[-1]), "dt": dt,
                          "ms_per_step": ms_lf / nsteps, "per_s": nsteps / (ms_lf * 1e-3),
                          "inner_cg_iterations_last": lf.inner_iters,
                          "cpu_baseline": {"ms_per_step": cpu_ms / 2, "per_s": 2 / (cpu_ms * 1e-3), "kind": "port",
                                           "cores": 1, "sample": "oracle.Leapfrog (SuperLU mass factors), 2 steps"}}
    lf.close()
    meshl.close()
    mesh.close()
    ctx.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--solves", type=int, default=5)
    ap.add_argument("--max-iters", type=int, default=10000)
    ap.add_argument("--pc", default="auto", choices=["auto", "jacobi", "hx"],
                    help="block preconditioner of the mixed solve")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-solve", action="store_true", help="skip the solve phase (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer phase (profiling runs)")
    ap.add_argument("--no-sub", action="store_true",
                    help="skip the compact batch / precision / serving studies of the default run")
    ap.add_argument("--workload", default="assembly",
                    choices=["assembly", "precision", "serve", "batch", "next", "dirac", "shapes"],
                    help="assembly: the headline line; precision: the 4D FP32-with-refinement study; "
                         "serve: the request stream, served vs plain; batch: many meshes in one launch set; "
                         "next: matrix-free operator, source load, de Rham map, leapfrog; "
                         "dirac: direct Lorentzian Dirac solves by mesh size; "
                         "shapes: the headline step by scatter launch shape")
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--meshes", type=int, default=512, help="batch: number of meshes")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: Poisson arrival rate (requests/s)")
    ap.add_argument("--lanes", type=int, default=4)
    ap.add_argument("--dirac-iters", type=int, default=300,
                    help="serve: iteration cap of the Lorentzian Dirac requests (GMRES on the sparse LU)")
    ap.add_argument("--dirac-sizes", default="6,12,20,28,37",
                    help="dirac: boxes per axis of the Minkowski meshes (6 N^3 cells each)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "next":
        run_next(args)
    elif args.workload == "dirac":
        run_dirac(args)
    elif args.workload == "shapes":
        run_shapes(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
