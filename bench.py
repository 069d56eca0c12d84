"""Benchmark: 256-bit interior-point iterations per second on the graph-partition
workload with n = 500, m = 501 (one dense 500 x 500 block, C = -L of an
Erdos-Renyi graph with edge probability 0.02, diag(X) = 1 and (11^T).X = 0).

A "step" is one predictor-corrector iteration of the solver (Newton predictor,
step length, Newton corrector, Lanczos step length, iterate update with the
X / Z inverse Cholesky, residuals): one pass of the reference's main-loop body.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision 256|512] [--no-e2e] [--no-cpu]

Our arm (default): the multi-limb GPU solver.  Timed with CUDA events on the
solver's stream around exactly K iterations after W warm-up iterations, with a
barrier and device synchronisation on both sides; max over ranks.  With N > 1
each rank solves its own replica (the single solve does not shard): scaling
"weak", value = iterations of all ranks / max time.

Reference arm (--impl reference): the CPU port of the reference solver
(oracle/sdpa_port.cpp, GMP mpf, OpenMP over all host cores in the NN matrix
product exactly where the reference parallelises) running the same iterations
of the same problem; rank 0 only.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import re
import shutil
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# Hardware work queues for the solver's streams (four per solve, 64 and more with
# concurrent batched solves); read by CUDA when the context is created, so set before
# any CUDA call.  The default of 8 makes unrelated streams wait on one another.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = "256-bit IPM iters/s (gpp n=500 m=501)"
UNIT = "iters/s"
RESIDUE_MODULI = 70  # primes of the 256-bit residue GEMM (csrc/crt_tables.h)
# DRAM bytes (read + write) per algorithmic byte (or per launch for the tensor kernel),
# from the ncu captures of a 500^3 product summarised in
# profiles/residue_gemm_gemm500_256bit.md: tc_residue_kernel 20.1 + 16.2 MB against
# 20.0 + 70.0 MB algorithmic; tc_reconstruct_kernel 35.9 MB against 45.0 MB;
# crt_exp_kernel 20.0 MB against 20.0 MB; tc_modgemm_kernel 80.2 MB per launch.
TC_TRAFFIC_BYTES = 80.2e6
TRAFFIC_PER_ALG_BYTE = {"tc_residue_kernel": 36.3 / 90.0, "tc_reconstruct_kernel": 35.9 / 45.0,
                        "crt_exp_kernel": 20.0 / 20.0}
# Kernel families with an algorithmic-work figure (sdpg_kernel_times' work column):
# roofline bound and the unit of that work.
FAMILY_BOUND = {"tc_residue_kernel": "hbm", "crt_exp_kernel": "hbm", "tc_reconstruct_kernel": "hbm",
                "lz_matvec_kernel": "hbm", "tc_modgemm_kernel": "tensor"}


def workload(precision: int):
    problems = importlib.import_module("sdpa-gmp_gb300.problems")
    d = tempfile.mkdtemp(prefix="sdpg_bench_")
    dat = os.path.join(d, "gpp500.dat-s")
    par = os.path.join(d, "gpp500.param")
    problems.gpp(500, 0.02, 0).write(dat)
    with open(par, "w") as f:
        f.write(problems.param_text(precision=precision))
    return d, dat, par


def config(precision: int, ws_mb: float | None = None) -> dict:
    return {"workload": f"gpp n=500 m=501 p=0.02 seed=0, {precision}-bit mantissa, default param.sdpa",
            "n": 500, "m": 501, "precision_bits": precision,
            "l2": f"no flush; per-iteration working set {ws_mb:.0f} MB > 129 MB L2" if ws_mb else "n/a",
            "parallelism": "replicas"}


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.f = open(self.path, "w")
        self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits", "-lms", "100"],
                                     stdout=self.f, stderr=subprocess.DEVNULL)

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return {}


def cpu_port_binary() -> str:
    exe = os.path.join(ROOT, "oracle", "_port", "sdpa_port")
    if not os.path.exists(exe):
        subprocess.run([os.path.join(ROOT, "oracle", "build_port.sh")], check=True, stdout=subprocess.DEVNULL)
    return exe


def run_cpu_port(dat: str, par_dir: str, precision: int, iters: int) -> tuple[list[float], int]:
    """Run the CPU port for `iters` iterations; returns per-iteration seconds and threads."""
    problems = importlib.import_module("sdpa-gmp_gb300.problems")
    par = os.path.join(par_dir, f"cpu{iters}.param")
    with open(par, "w") as f:
        f.write(problems.param_text(precision=precision, max_iteration=iters))
    threads = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([cpu_port_binary(), "-ds", dat, "-p", par, "-times"], env=env, capture_output=True, text=True,
                       check=True)
    times = [float(m.group(2)) for m in re.finditer(r"^ITER (\d+) ([0-9.eE+-]+)$", r.stderr, re.M)]
    return times, threads


def kernel_families(sdpg, new_solver, steps: int, warmup: int, peaks: dict) -> tuple[list, float]:
    """A second pass over the same workload: `steps` iterations after `warmup`, every kernel
    bracketed by CUDA events on its own stream (captured graphs run as plain launches).
    Returns per-kernel rows sorted by time and the summed kernel milliseconds per step."""
    import torch
    s = new_solver()
    for _ in range(warmup):
        if not s.iterate():
            s = new_solver()
    torch.cuda.synchronize()
    sdpg.kernel_times()  # drop anything recorded before
    sdpg.kernel_timing(True)
    try:
        k = 0
        while k < steps:
            if s.iterate():
                k += 1
            else:
                s = new_solver()
        torch.cuda.synchronize()
        times = sdpg.kernel_times()
    finally:
        sdpg.kernel_timing(False)
    s.close()
    total = sum(v[1] for v in times.values())
    hbm = peaks.get("hbm_gbs") or 6800.0
    tflops = peaks.get("bf16_tflops_sustained") or 1700.0
    rows = []
    for name, (launches, ms, work) in sorted(times.items(), key=lambda kv: -kv[1][1]):
        row = {"kernel": name, "launches_per_step": launches / steps, "ms_per_step": ms / steps,
               "share": ms / total if total else None, "avg_launch_us": 1e3 * ms / max(1, launches)}
        bound = FAMILY_BOUND.get(name)
        if bound and work > 0 and ms > 0:
            if bound == "hbm":
                ach = work / (ms * 1e-3) / 1e9
                row.update(bound="hbm", achieved=ach, peak=hbm, unit="GB/s", frac=ach / hbm,
                           algorithmic_bytes_per_launch=work / launches)
            else:
                ach = work / (ms * 1e-3) / 1e12
                row.update(bound="tensor", achieved=ach, peak=tflops, unit="TFLOP/s", frac=ach / tflops,
                           algorithmic_flops_per_launch=work / launches)
        else:
            row["bound"] = "latency"
        rows.append(row)
    return rows, total / steps


def reference_errors(sdpg, solver, name: str) -> dict | None:
    """log2 relative errors against a high-precision golden (tests/golden/<name>.json)."""
    gpath = os.path.join(ROOT, "tests", "golden", name + ".json")
    if not os.path.exists(gpath):
        return None
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    precise = importlib.import_module("precise")
    with open(gpath) as f:
        g = json.load(f)
    info = solver.info()
    out = {"golden": name, "reference_phase": g["phase"], "reference_iterations": g["iteration"],
           "phase": info["phase"], "iterations": info["iteration"]}
    if info["iteration"] != g["iteration"]:
        out["note"] = "different iteration counts: final iterates not comparable"
        return out
    e = precise.errors(sdpg, solver, g)
    out["log2_rel_error"] = {k: round(e[k + "_log2"], 1) for k in ("objValPrimal", "objValDual", "relgap", "xVec",
                                                                  "xMat", "yMat")}
    return out


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def bench_ours(args) -> None:
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    sdpg = importlib.import_module("sdpa-gmp_gb300")
    d, dat, par = workload(args.precision)
    stream = torch.cuda.Stream(device=local)
    param = sdpg.Param.read(par)

    def new_solver():
        s = sdpg.Solver(sdpg.Problem.read(dat), param, device=local, stream=stream.cuda_stream)
        s.initialize()
        return s

    solver = new_solver()
    for _ in range(args.warmup):
        if not solver.iterate():
            solver = new_solver()
    solver.reset_counters()
    solver.gemm_profile(enable=1)
    launches0 = sdpg.launch_count()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    barrier(dist)
    clocks.start()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    done = 0
    restarts = 0
    while done < args.steps:
        if solver.iterate():
            done += 1
        else:  # the solve finished before K steps: start the same solve again
            solver = new_solver()
            solver.gemm_profile(enable=1)
            restarts += 1
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(dist)
    launches = sdpg.launch_count() - launches0
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(dist, ms)
    total_steps = sum_over_ranks(dist, float(args.steps))
    prof = solver.gemm_profile(enable=0)
    timers = solver.timers()

    # roofline of the GEMM kernel (the bulk of the arithmetic): at 256 bits the tcgen05
    # residue GEMM against the measured bf16 tensor peak (fp16 runs at the same rate;
    # sustained figure, the kernel runs inside a long step); at 512 bits the integer
    # digit GEMM against the measured IMAD.WIDE throughput.
    gemm_ms = prof["kernel_ms"]
    mac_rate = prof["macs"] / (gemm_ms * 1e-3) if gemm_ms > 0 else 0.0
    common = {"launches": prof["launches"], "avg_launch_us": 1e3 * gemm_ms / max(1, prof["launches"]),
              "share_of_step": gemm_ms / ms if ms > 0 else None, "mac_rate_gmacs": mac_rate / 1e9}
    if args.precision <= 256:
        peaks = measured_peaks()
        peak = peaks.get("bf16_tflops_sustained")
        src = "bf16_tflops_sustained of measured (MEASURED_PEAKS.json)"
        if not peak:
            peak, src = 1700.0, "sustained bf16 fallback"
        achieved = 2.0 * RESIDUE_MODULI * mac_rate / 1e12
        roofline = {"bound": "tensor", "kernel": "tc_modgemm_kernel", "achieved": achieved, "peak": peak,
                    "unit": "TFLOP/s", "frac": achieved / peak, "traffic": TC_TRAFFIC_BYTES, "peak_source": src,
                    "algorithmic": f"2*M*N*K*{RESIDUE_MODULI} fp16 flops per multi-limb GEMM "
                                   f"({RESIDUE_MODULI} residue GEMMs)", **common}
    else:
        imad_peak = sdpg.probe_imad_wide(local)
        D = 20
        imad_per_mac = D * (D + 1) // 2
        achieved_imad = mac_rate * imad_per_mac
        roofline = {"bound": "int", "kernel": "bfp_gemm_kernel",
                    "achieved": achieved_imad / 1e12, "peak": imad_peak / 1e12, "unit": "TIMAD.WIDE/s",
                    "frac": achieved_imad / imad_peak if imad_peak else None,
                    "peak_source": "measured in-run by sdpg_probe_imad_wide (MEASURED_PEAKS.json has no "
                                   "integer-pipe figure)",
                    "imad_wide_per_mac": imad_per_mac, "traffic": None, **common}

    # the same iterations with every product on the integer digit GEMM (the plain
    # multi-limb path): the tensor-core path's speed-up at equal accuracy, timed right
    # after the tensor-core iterations (before the longer per-kernel pass)
    plain = None
    if args.precision <= 256 and not args.no_plain:
        old_method = sdpg.set_gemm_method(1)
        try:
            sp = new_solver()
            for _ in range(args.warmup):
                if not sp.iterate():
                    sp = new_solver()
            torch.cuda.synchronize()
            p0 = torch.cuda.Event(enable_timing=True)
            p1 = torch.cuda.Event(enable_timing=True)
            p0.record(stream)
            k = 0
            while k < args.steps:
                if sp.iterate():
                    k += 1
                else:
                    sp = new_solver()
            p1.record(stream)
            torch.cuda.synchronize()
            pms = p0.elapsed_time(p1)
            plain = {"value": args.steps / (pms * 1e-3), "unit": UNIT, "ms_per_step": pms / args.steps,
                     "method": "integer digit GEMM on the CUDA cores (sdpg_set_gemm_method(1))",
                     "tensor_speedup": (pms / args.steps) / (ms / args.steps) if ms > 0 else None}
            sp.close()
        finally:
            sdpg.set_gemm_method(old_method)

    # every kernel family of the same iterations, timed per launch in a second pass
    families, kernel_ms_per_step = kernel_families(sdpg, new_solver, args.steps, args.warmup, measured_peaks()) \
        if not args.no_families else ([], None)
    dominant = None
    for fam in families:  # the dominant kernel with a roofline bound (hbm or tensor)
        if fam.get("bound") in ("hbm", "tensor"):
            dominant = fam
            break
    if dominant is not None:
        traffic = None
        if dominant["kernel"] in TRAFFIC_PER_ALG_BYTE:
            traffic = TRAFFIC_PER_ALG_BYTE[dominant["kernel"]] * dominant["algorithmic_bytes_per_launch"]
        elif dominant["kernel"] == "tc_modgemm_kernel":
            traffic = TC_TRAFFIC_BYTES
        roofline_dom = {"bound": dominant["bound"], "kernel": dominant["kernel"], "achieved": dominant["achieved"],
                        "peak": dominant["peak"], "unit": dominant["unit"], "frac": dominant["frac"],
                        "traffic": traffic, "share_of_kernel_time": dominant["share"],
                        "avg_launch_us": dominant["avg_launch_us"],
                        "peak_source": ("hbm_gbs" if dominant["bound"] == "hbm" else "bf16_tflops_sustained")
                                       + " of measured (MEASURED_PEAKS.json)",
                        "timing": "per-launch CUDA events on the launching stream, second pass of the same "
                                  f"{args.steps} iterations after {args.warmup} warm-up"}
    else:
        roofline_dom = None

    # end to end through the public API: host .dat-s -> parse -> upload -> full solve -> xVec back
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prob = sdpg.Problem.read(dat)
        s2 = sdpg.Solver(prob, param, device=local, stream=stream.cuda_stream)
        its = s2.run()
        x = s2.xvec()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        h2d, d2h = s2.io_bytes()
        err_full = reference_errors(sdpg, s2, "gpp500_hp" if args.precision <= 256 else "")
        e2e = {"value": its / (t1 - t0), "unit": UNIT, "iterations": its, "seconds": t1 - t0,
               "h2d_bytes_per_step": int(h2d / max(1, its)), "d2h_bytes_per_step": int((d2h + x.nbytes) / max(1, its)),
               "phase": s2.info()["phase"], "scope": "Problem.read + Solver + run() + xvec(), host file to host result"}
        s2.close()
    # error against the reference's own 80-digit (160 at 512 bits) output: the full solve
    # (above) and the first 10 iterations of the same problem
    errs = {}
    if not args.no_e2e and err_full:
        errs["full_solve"] = err_full
    pref = "gpp500_it10" if args.precision <= 256 else "gpp500_p512_it10"
    par10 = os.path.join(d, "it10.param")
    with open(par10, "w") as f:
        f.write(importlib.import_module("sdpa-gmp_gb300.problems").param_text(precision=args.precision,
                                                                              max_iteration=10))
    s3 = sdpg.Solver(sdpg.Problem.read(dat), sdpg.Param.read(par10), device=local, stream=stream.cuda_stream)
    s3.run()
    e10 = reference_errors(sdpg, s3, pref)
    if e10:
        errs["first_10_iterations"] = e10
    s3.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            times, threads = run_cpu_port(dat, d, args.precision, 2)
            sample = times[-1]
            cpu = {"value": 1.0 / sample, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": f"iteration 1 of gpp500 at {args.precision}-bit on the host CPU "
                             f"({sample:.1f} s; iteration 0 {times[0]:.1f} s)"}
        except Exception as exc:  # the baseline is reported, never required
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "sample": f"failed: {exc}"}

    if rank == 0:
        ws_mb = (15 * 500 * 500 + 501 * 501) * (8 + 4 * (8 if args.precision <= 256 else 16)) / 1e6
        line = {"metric": METRIC if args.precision <= 256 else METRIC.replace("256", str(args.precision)),
                "value": total_steps / (ms_max * 1e-3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": f"u32x{8 if args.precision <= 256 else 16} multi-limb",
                "data": "synthetic (seeded generator standing in for SDPLIB gpp500)",
                "config": config(args.precision, ws_mb),
                "impl": "ours", "e2e": e2e, "gpu_launches": launches, "roofline": roofline_dom or roofline,
                "roofline_gemm": roofline, "kernel_families": families[:12],
                "kernel_ms_per_step": kernel_ms_per_step,
                "dominant_kernel": ({"kernel": families[0]["kernel"], "share": families[0]["share"],
                                     "bound": families[0]["bound"]} if families else None),
                "error_vs_reference": errs or None, "cpu_baseline": cpu,
                "plain_path": plain,
                "clocks": clk, "phase_ms": {k: round(v, 3) for k, v in timers.items()},
                "restarts": restarts, "peaks": {k: measured_peaks().get(k) for k in ("hbm_gbs", "bf16_tflops")}}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    shutil.rmtree(d, ignore_errors=True)


def bench_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    d, dat, par = workload(args.precision)
    try:
        times, threads = run_cpu_port(dat, d, args.precision, args.warmup + args.steps)
        timed = times[args.warmup: args.warmup + args.steps]
        if len(timed) < args.steps:
            raise RuntimeError("the CPU run stopped early")
        total = sum(timed)
        value = len(timed) / total
        line = {"metric": METRIC if args.precision <= 256 else METRIC.replace("256", str(args.precision)),
                "value": value, "unit": UNIT, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(timed),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "GMP mpf",
                "data": "synthetic (seeded generator standing in for SDPLIB gpp500)", "config": config(args.precision),
                "impl": "reference",
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                                 "sample": f"iterations {args.warmup}..{args.warmup + args.steps - 1} of gpp500, "
                                           f"CPU port of the reference (GMP mpf, OpenMP NN product)"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    except Exception as exc:
        line = {"impl": "reference", "unavailable": f"CPU port failed: {exc}"}
    print(json.dumps(line))
    shutil.rmtree(d, ignore_errors=True)


def bench_batch(args) -> None:
    """Batched mode: control/LMI instances with m ~ U[20, 350] and two
    blocks of sizes ~ U[15, 90] (seeds 0 .. batch-1) solved by sdpg_solve_batch with
    --concurrency solvers in flight, against the same solver run one problem at a time
    on the first --serial instances; prints solves/s for both."""
    import numpy as np
    import torch
    world, rank, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    sdpg = importlib.import_module("sdpa-gmp_gb300")
    problems = importlib.import_module("sdpa-gmp_gb300.problems")
    shard = importlib.import_module("sdpa-gmp_gb300.shard")
    # instances are partitioned over the ranks by estimated cost (sum n_b^3 + m^3); each
    # rank builds and solves only its own, and rank 0 gathers the per-instance results
    sizes = [problems.batch_instance_size(seed) for seed in range(args.batch)]
    costs = [shard.instance_cost(m, bl) for m, bl in sizes]
    mine = shard.partition(costs, world)[rank]
    t0 = time.perf_counter()
    probs = {seed: sdpg.Problem.from_dense(*problems.batch_instance(seed)) for seed in mine}
    gen_s = time.perf_counter() - t0
    param = sdpg.Param.default()
    param.precision = args.precision
    sdpg.set_gemm_method(args.gemm_method)
    # warm-up: one small solve (library set-up, tensor-core tables)
    if mine:
        sdpg.solve_batch([probs[mine[0]]], param, device=local, concurrency=1)
    torch.cuda.synchronize()
    barrier(dist)
    t0 = time.perf_counter()

    def solve_mine(seeds):
        if not seeds:
            return []
        its_, info_ = sdpg.solve_batch([probs[s] for s in seeds], param, device=local,
                                       concurrency=args.concurrency)
        torch.cuda.synchronize()
        return [(int(a), [float(v) for v in b]) for a, b in zip(its_, info_)]

    gathered = shard.solve_sharded(list(range(args.batch)), costs, solve_mine, rank, world, dist)
    batched_s = max_over_ranks(dist, time.perf_counter() - t0)
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    its = np.array([g[0] for g in gathered])
    info = np.array([g[1] for g in gathered])
    ns = min(args.serial, args.batch)
    serial_probs = [probs[s] if s in probs else sdpg.Problem.from_dense(*problems.batch_instance(s))
                    for s in range(ns)]
    t0 = time.perf_counter()
    its_s, info_s = sdpg.solve_batch(serial_probs, param, device=local, concurrency=1)
    torch.cuda.synchronize()
    serial_s = time.perf_counter() - t0
    phases = [sdpg.PHASES[int(x)] for x in info[:, 0]]
    line = {"metric": f"batched solves/s ({args.precision}-bit control/LMI SDPs, m~U[20,350], two blocks ~U[15,90])",
            "value": args.batch / batched_s, "unit": "solves/s", "n_gpus": world, "higher_is_better": True,
            "scaling": "strong",
            "config": {"workload": f"{args.batch} instances, seeds 0..{args.batch - 1}",
                       "concurrency": args.concurrency, "precision_bits": args.precision,
                       "sharding": f"instances partitioned over {world} rank(s) by sum n_b^3 + m^3, "
                                   "results gathered on rank 0"},
            "serial": {"value": ns / serial_s, "unit": "solves/s", "instances": ns},
            "speedup_vs_serial": (args.batch / batched_s) / (ns / serial_s),
            "iterations_mean": float(np.mean(its)), "pdOPT": sum(p == "pdOPT" for p in phases),
            "failed": int(np.sum(its < 0)),
            "identical_to_serial": bool(np.array_equal(info[:ns], info_s)),
            "generation_s": gen_s, "data": "synthetic (seeded generator)"}
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def bench_learned(args) -> None:
    """Learned mode (signed MaxCut, n = 124): the committed lambdaStar / beta policy against the
    default parameters on held-out MaxCut instances (n = 124, p ~ U[0.02, 0.2], edge
    weights +-1); prints mean iterations of both and the largest objective difference
    from the default solve, which judges the learned path's error."""
    learned = importlib.import_module("sdpa-gmp_gb300.learned")
    sdpg = importlib.import_module("sdpa-gmp_gb300")
    pol = sdpg.Policy.load(learned.POLICY_FILE)
    seeds = range(learned.HOLDOUT_BASE, learned.HOLDOUT_BASE + args.batch)
    t0 = time.perf_counter()
    ev = learned.evaluate(pol, seeds, workers=args.concurrency, constant=learned.BEST_CONSTANT)
    secs = time.perf_counter() - t0
    line = {"metric": "mean IPM iterations to pdOPT, learned lambdaStar/beta vs default (MaxCut n=124, +-1)",
            "value": ev["mean_iterations_learned"], "unit": "iterations", "n_gpus": 1, "higher_is_better": False,
            "config": {"workload": f"{args.batch} held-out seeds from {learned.HOLDOUT_BASE}",
                       "precision_bits": learned.PRECISION, "policy": os.path.basename(learned.POLICY_FILE)},
            "default_iterations": ev["mean_iterations_default"], "iteration_reduction": ev["iteration_reduction"],
            "ablation": {"default": ev["mean_iterations_default"], "best_constant": ev["mean_iterations_constant"],
                         "policy": ev["mean_iterations_learned"], "constant": ev["constant"],
                         "constant_reduction_vs_default": ev["constant_reduction"],
                         "policy_reduction_vs_constant": ev["learned_vs_constant"],
                         "seeds_policy_better": ev["seeds_learned_better"],
                         "seeds_constant_better": ev["seeds_constant_better"],
                         "max_constant_objective_rel_error": ev["max_constant_objective_rel_error"]},
            "fallback_solves": ev["fallback_solves"], "beta_fallback_rate": ev["beta_fallback_rate"],
            "mean_lambda_star": ev["mean_lambda"], "max_objective_rel_error": ev["max_objective_rel_error"],
            "seconds": secs, "data": "synthetic (seeded generator)"}
    print(json.dumps(line))


def bench_gemm(args) -> None:
    """Kernel mode: repeated n x n x n multi-limb GEMMs through sdpg_rgemm_device
    (the profiling target of the digit-GEMM kernel); prints GMAC/s."""
    import numpy as np
    import torch
    sdpg = importlib.import_module("sdpa-gmp_gb300")
    lib = sdpg.lib()
    n = args.gemm_n
    limbs = 8 if args.precision <= 256 else 16
    rng = np.random.default_rng(0)

    def rnd(cnt):
        h = rng.integers(0, 2**32, size=(cnt, limbs + 2), dtype=np.uint64).astype(np.uint32)
        h[:, 0] = rng.integers(-5, 5, size=cnt).astype(np.int32).view(np.uint32)
        h[:, 1] = rng.integers(0, 2, size=cnt).astype(np.uint32)
        h[:, -1] |= np.uint32(0x80000000)
        return torch.from_numpy(h.view(np.int32)).cuda()

    A, B, C = rnd(n * n), rnd(n * n), rnd(n * n)
    sdpg.set_gemm_method(args.gemm_method)
    one = sdpg.ml_parse(["1"], limbs)
    zero = sdpg.ml_parse(["0"], limbs)
    st = torch.cuda.current_stream().cuda_stream

    def run():
        sdpg.check(lib.sdpg_rgemm_device(limbs, b"N", b"N", n, n, n, one.ctypes.data, A.data_ptr(), n,
                                         B.data_ptr(), n, zero.ctypes.data, C.data_ptr(), n, st))

    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    print(json.dumps({"kernel": "gemm", "n": n, "limbs": limbs, "method": args.gemm_method, "ms_per_gemm": ms,
                      "gmacs": n ** 3 / (ms * 1e-3) / 1e9}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["gemm"], default=None,
                    help="kernel mode: time repeated multi-limb GEMMs instead of IPM iterations")
    ap.add_argument("--gemm-n", type=int, default=500)
    ap.add_argument("--gemm-method", type=int, default=0, choices=[0, 1, 2],
                    help="GEMM method (kernel and batch modes): 0 tensor-core residue path where it applies "
                         "(default), 1 integer digit GEMM, 2 residue path for every 256-bit product")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", type=int, default=256)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the digit-GEMM (plain path) comparison")
    ap.add_argument("--no-families", action="store_true", help="skip the per-kernel timing pass")
    ap.add_argument("--workload", choices=["ipm", "batch", "learned"], default="ipm",
                    help="batch: many small control/LMI solves at once (solves/s); learned: the committed "
                         "lambdaStar/beta policy against the defaults (mean iterations) on --batch held-out seeds")
    ap.add_argument("--batch", type=int, default=64, help="batch mode: instances")
    ap.add_argument("--concurrency", type=int, default=16, help="batch mode: solvers in flight")
    ap.add_argument("--serial", type=int, default=8, help="batch mode: instances timed one at a time")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.kernel == "gemm":
        bench_gemm(args)
    elif args.workload == "batch" and args.impl != "reference":
        bench_batch(args)
    elif args.workload == "learned" and args.impl != "reference":
        bench_learned(args)
    elif args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
