#!/usr/bin/env python3
"""Benchmark of the periodic REPEAT charge fit on GB300.

Workload (default): the batched configuration — 256 independent seeded cubes
(20-300 atoms, cubic or orthorhombic 12-30 Bohr cells, 40^3-96^3 grids at
0.2-0.3 Bohr, neutral charges N(0, 0.5), ESP = Ewald potential + N(0, 1e-4),
half with symmetry groups, half with RESP), fitted by one ``rp_fit_batch`` call
per step: every filter, the normal equations of every cube and one launch of
all bordered solves.  A step is one batch; ``value`` is fits/s with the grids
resident in HBM, ``e2e`` the same through the public API from pinned host
memory (H2D of every grid and D2H of the charges inside the timed region).

Beside it, in the same run: the plain FP64 GPU fit of a subset of the cubes
(fits/s and max|dq| of the mixed path against it), single-fit p50/p99 latency,
the dominant kernel's roofline from live CUDA-event stage timings, SM clocks
sampled during the timed region, and the CPU oracle timed on a bounded sample.

``--impl reference`` times the reference algorithm on the host cores (the C
oracle restatement of repeat.py / repeat_cpu_omp.cpp; the reference's own
compiled program cannot be built where its sources are absent).

Multi-GPU (torchrun): every rank fits its own 256 cubes (weak scaling, no
data-path collective); the step time is the max over ranks.
"""
from __future__ import annotations

import argparse
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

METRIC = "fits/s & p50/p99 latency vs plain FP64 GPU fit at max|dq|<=1e-5 e"

# ncu figures of phi_chunk_kernel: DRAM bytes and thread instructions per point-atom pair
# of the captured launch (the file holds the command and the raw figures)
PHI_CAPTURE = "profiles/phi_chunk_kernel_batch8.txt"
PHI_DRAM_PER_PAIR = 10.15
PHI_INST_PER_PAIR = 344.4


# ----------------------------------------------------------------------------- distributed helpers

def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            backend = os.environ.get("REPEAT_BENCH_BACKEND", "nccl")
            if backend == "nccl":
                import torch
                torch.cuda.set_device(local)
            dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value: float, world: int, device=None) -> float:
    """Largest value over all ranks (the step time of a weak-scaled job)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ----------------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def mark(self):
        """Samples before this call (the sampler's start-up) are left out of stop()'s figures."""
        self.first = len(self.rows)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows[getattr(self, "first", 0):]:
            try:
                sm.append(float(r[0]))
                smax.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------- workloads

def make_workload(name: str, n_cubes: int, seed0: int, ctx, host_esp: bool = True):
    """(cubes, description) of the workload.  With ctx the ESP is evaluated on the GPU
    (rp_potential); without, on the host, or, for the single large cubes when host_esp is
    False, left as noise (the same geometry and fit work, for host-side timing)."""
    from pyrepeat_gb300 import synth
    esp = host_esp or ctx is not None
    if name == "batch":
        cubes = [synth.make_batch_item(seed0 + i, ctx=ctx) for i in range(n_cubes)]
    elif name == "mof":
        cubes = [synth.make_mof(seed0, ctx=ctx, esp=esp)]
    elif name == "water":
        cubes = [synth.make_water(seed0, ctx=ctx)]
    elif name == "tric":
        cubes = [synth.make_tric(seed0, ctx=ctx, esp=esp)]
    else:
        raise SystemExit(f"unknown workload {name}")
    return cubes, _workload_desc(name, n_cubes)


def _workload_desc(name: str, n_cubes: int) -> str:
    return {"batch": f"batch-{n_cubes}: {n_cubes} independent cubes, 20-300 atoms, cubic/orthorhombic 12-30 Bohr, "
                     f"40^3-96^3 grids at 0.2-0.3 Bohr, KMAX 7 (K=754), Rc 20, half symmetry groups, half RESP",
            "mof": "mof: cubic 25.8 Bohr, 128^3 grid, 424 atoms, KMAX 12 (K=3779)",
            "water": "water: cubic 18 Bohr, 72^3 grid, 9 atoms, K=754",
            "tric": "tric: triclinic 40 x 42 x 45 Bohr (85/95/100 deg), 200 x 210 x 225 grid (9.45 M points), "
                    "2000 atoms C/H/N/O, 150 symmetry groups, RESP on C/N/O, KMAX 7 (K=754), Rc 20"}[name]


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["bf16_tflops"]), float(d["hbm_gbs"]), "measured"
    except Exception:
        return 1900.0, 6800.0, "fallback"


# ----------------------------------------------------------------------------- CPU oracle timing

def cpu_oracle_sample(cube, sample: int, threads: int):
    """Time the C oracle (restatement of the reference fit) on `sample` kept points
    of one cube; returns (seconds, sample, kept count of the cube)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cube.host_V()
    of = oracle.OracleFit(cube, threads=threads, sample=sample, seed=0)
    t0 = time.perf_counter()
    of.fit()
    dt = time.perf_counter() - t0
    return dt, min(sample, of.M_total), of.M_total


def reference_arm(args, world, rank):
    """Reference CPU implementation of the path on the host cores (rank 0 only): the C
    oracle (restatement of repeat.py's FP64 fit) on the first cubes of the same seeded
    workload the GPU arm fits, generated on the host with no GPU context.  Each step fits a
    seeded sample of one cube's kept points, extrapolated linearly to the whole cube."""
    if rank != 0:
        return
    if args.workload == "serve":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving mode (repeat.py is a "
                                                               "one-shot program); its per-fit CPU time is the batch arm"}),
              flush=True)
        return
    if args.workload == "qeq":
        reference_qeq_arm(args, world)
        return
    threads = max(1, os.cpu_count() or 1)
    k = min(args.n_cubes, args.ref_cubes)
    t0 = time.time()
    cubes, _ = make_workload(args.workload, k, 1000, None, host_esp=False)
    desc = _workload_desc(args.workload, args.n_cubes)
    gen_s = time.time() - t0
    sample = args.ref_sample
    times = []
    for step in range(args.warmup + args.steps):
        c = cubes[step % len(cubes)]
        dt, s, M = cpu_oracle_sample(c, sample, threads)
        if step >= args.warmup:
            times.append(dt * M / s)   # seconds for the whole cube, linear in kept points
    per_fit = statistics.mean(times)
    value = 1.0 / per_fit
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "fits/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_fit * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": desc, "seeds": "the GPU arm's rank-0 seeds (cubes 0..%d of its list)" % (k - 1),
                   "generation_s": round(gen_s, 1)},
        "cpu_baseline": {"value": value, "unit": "fits/s", "cores": threads, "kind": "port",
                         "sample": f"one cube per step, cycling over the first {k} cubes of the workload "
                                   f"(host-generated, no GPU context); {sample} seeded kept points per step, "
                                   f"extrapolated linearly to the cube's kept count; fits/s = 1 / mean per-fit "
                                   f"seconds over the timed steps"},
        "e2e": {"value": value, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm

def reference_qeq_arm(args, world):
    """QEq charges on the host: the oracle's NumPy restatement of compute_qeq_charges
    (Coulomb matrix by pairs, the reference's difference-form solve), one core; each step
    times the matrix rows of a bounded block of atoms and the full solve, extrapolated in
    pairs."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from pyrepeat_gb300 import qeq as Q
    N = args.qeq_atoms
    atoms, Z, ngrid, axis = qeq_cell(N, 7)
    chi, js, _, _ = Q.charge_parameters(Z)
    box = np.eye(3) * (axis[0, 0] * ngrid[0])
    rows = min(N, 64)
    times = []
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.qeq_matrix(atoms[:rows], box, 20.0, 7, js[:rows])
        t_rows = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.qeq_charges(np.eye(N) + 0.01, chi, 0.0)   # LU time does not depend on the values
        t_solve = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(t_rows * (N * (N - 1) / 2) / (rows * (rows - 1) / 2) + t_solve)
    per = statistics.mean(times)
    line = {
        "impl": "reference", "metric": "QEq charge sets/s (periodic Ewald Coulomb matrix + equalisation solve, "
                                      "host in/out)",
        "value": 1.0 / per, "unit": "charge sets/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": f"qeq: {N} atoms, Rc 20, KMAX 7"},
        "cpu_baseline": {"value": 1.0 / per, "unit": "charge sets/s", "cores": 1, "kind": "port",
                         "sample": f"Coulomb matrix rows of {rows} atoms per step, extrapolated to {N} atoms' pairs, "
                                   f"plus the {N}-atom solve"},
        "e2e": {"value": 1.0 / per, "unit": "charge sets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def served_stream(ctx, args, rank: int) -> dict:
    """The served workload on one GPU: Poisson arrivals at args.serve_rate from a pool of
    seeded cubes of the batch distribution plus a share of large cubes (800-1500 atoms,
    160^3), through a continuous-batching FitServer (size classes, HBM admission across
    the batches in flight, up to three batches on the device at once).  Latency is from a
    request's arrival to its charges on the host.  Beside it, the plain FP64 fit's service
    time of the same request mix (each class's cubes fitted alone in FP64, no queueing: a
    lower bound of an FP64 server's latency), and its sustainable rate."""
    import torch
    from pyrepeat_gb300 import _lib, synth
    from pyrepeat_gb300.serve import FitServer
    t0 = time.time()
    small = [synth.make_batch_item(20000 + 1000 * rank + i, ctx=ctx) for i in range(args.serve_pool)]
    large = [synth.make_batch_item(90000 + 1000 * rank + i, large=True, ctx=ctx) for i in range(args.serve_large)]
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    budget = args.serve_budget_gb * 1e9
    large_bytes = 8e9

    def stream(n_req, rate, seed):
        rng = np.random.default_rng(seed)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n_req))
        pick_large = rng.random(n_req) < args.serve_large_share
        picks = [large[int(rng.integers(len(large)))] if (pl and large) else small[int(rng.integers(len(small)))]
                 for pl in pick_large]
        srv = FitServer(ctx, max_batch=args.serve_batch, max_wait_s=args.serve_wait_ms / 1e3, hbm_budget=budget,
                        large_bytes=large_bytes)
        start = time.perf_counter()
        futs = []
        for k in range(n_req):
            delay = start + arrivals[k] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(srv.submit(picks[k], V_dev=picks[k].V_dev))
        for f in futs:
            f.result()
        wall = time.perf_counter() - start
        srv.close()
        return srv, wall, pick_large

    # warm-up at a high rate: every slot's buffers are sized before the clock starts
    stream(max(200, 4 * len(small)), 400.0, 5 + rank)
    srv, wall, pick_large = stream(args.serve_requests, args.serve_rate, 11 + rank)
    lat = np.array(srv.latencies) * 1e3
    lat_large = np.array(srv.large_latencies) * 1e3
    lat_small = np.array(srv.small_latencies) * 1e3
    # plain FP64 service time per class (cubes alone, no queueing), on a sample of the pool
    fp64 = {"small": [], "large": []}
    for name, cubes, k in (("small", small, args.serve_fp64_small), ("large", large, args.serve_fp64_large)):
        for c in cubes[:k]:
            ctx.fit_batch([c], _lib.PREC_FP64, V_dev=[c.V_dev])  # warm
            torch.cuda.synchronize()
            t = time.perf_counter()
            ctx.fit_batch([c], _lib.PREC_FP64, V_dev=[c.V_dev])
            torch.cuda.synchronize()
            fp64[name].append((time.perf_counter() - t) * 1e3)
    rng = np.random.default_rng(17)
    mix = np.array([rng.choice(fp64["large"] if (pl and fp64["large"]) else fp64["small"]) for pl in pick_large])
    nl = int(np.sum(pick_large))
    return {
        "fits_per_s": len(lat) / wall, "requests": len(lat), "wall_s": wall,
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "small_p50_ms": float(np.percentile(lat_small, 50)) if len(lat_small) else None,
        "small_p99_ms": float(np.percentile(lat_small, 99)) if len(lat_small) else None,
        "large_p50_ms": float(np.percentile(lat_large, 50)) if len(lat_large) else None,
        "large_p99_ms": float(np.percentile(lat_large, 99)) if len(lat_large) else None,
        "mean_batch": float(np.mean(srv.batch_sizes)), "batches": len(srv.batch_sizes),
        "max_batches_in_flight": srv.max_in_flight,
        "fp64": {"service_p50_ms": float(np.percentile(mix, 50)), "service_p99_ms": float(np.percentile(mix, 99)),
                 "sustainable_fits_per_s": 1e3 / float(np.mean(mix)),
                 "how": f"each request's plain FP64 fit time alone (no queueing), from {len(fp64['small'])} "
                        f"small and {len(fp64['large'])} large pool cubes fitted in FP64; at "
                        f"{args.serve_rate:.0f} req/s an FP64 server is stable only if its sustainable rate "
                        f"exceeds the arrival rate"},
        "config": f"{len(lat)} requests, Poisson {args.serve_rate:.0f}/s, {nl} large; pool of {len(small)} "
                  f"batch-distribution cubes and {len(large)} large cubes (800-1500 atoms at 160^3), max batch "
                  f"{args.serve_batch}, max wait {args.serve_wait_ms} ms, large requests (> {large_bytes / 1e9:.0f} "
                  f"GB estimated) batched alone, admission budget {args.serve_budget_gb} GB across the batches "
                  f"in flight",
        "generation_s": round(gen_s, 1),
    }


def serve_arm(args, world, rank, local):
    """The served workload alone (--workload serve): its own JSON line."""
    import torch
    from pyrepeat_gb300.fit import Context
    torch.cuda.set_device(local)
    ctx = Context(local)
    barrier(world)
    sv = served_stream(ctx, args, rank)
    wall = max_over_ranks(sv["wall_s"], world, "cuda")
    if rank != 0:
        return
    line = {
        "metric": "served fits/s & p50/p99 latency (arrival to charges on the host)",
        "value": sv["requests"] * world / wall, "unit": "fits/s", "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": wall * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+double-float+exact-int+f64", "data": "synthetic", "served": sv,
        "config": {"workload": "serve: " + sv["config"]},
    }
    print(json.dumps(line), flush=True)


def qeq_cell(n_atoms: int, seed: int):
    """A periodic cell of n_atoms on a jittered 5 Bohr lattice (H, C, O, Zn at random), the
    well-conditioned QEq system of a MOF-like density.  Returns (atoms, Z, n_grid, axis)."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil((1.2 * n_atoms) ** (1.0 / 3.0)))
    L = 5.0 * side
    site = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)
    site = site[rng.choice(len(site), size=n_atoms, replace=False)]
    atoms = (site + 0.5 + rng.uniform(-0.15, 0.15, size=(n_atoms, 3))) * 5.0
    Z = rng.choice([1, 6, 8, 30], size=n_atoms)
    ng = 2 * side * 5
    return atoms, Z, np.array([ng, ng, ng]), np.eye(3) * (L / ng)


def qeq_arm(args, world, rank, local):
    """QEq charges (repeat.py:2539-2634) of one periodic cell per step through rp_qeq, from
    host atoms and parameters to host charges: the Coulomb matrix (per-atom k tables, one
    FP64 DGEMM, the real-space pair kernel over all 27+ images) and the equalisation solve.
    CPU baseline: the oracle's NumPy Coulomb matrix on a bounded block of rows,
    extrapolated in pairs, plus its full solve."""
    import torch
    from pyrepeat_gb300 import qeq as Q
    from pyrepeat_gb300.fit import Context
    torch.cuda.set_device(local)
    ctx = Context(local)
    N = args.qeq_atoms
    atoms, Z, ngrid, axis = qeq_cell(N, 7 + rank)
    chi, js, _, _ = Q.charge_parameters(Z)
    for _ in range(max(args.warmup, 3)):
        ctx.qeq(ngrid, axis, atoms, chi, js, 0.0, 20.0, 7)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        q, _, info = ctx.qeq(ngrid, axis, atoms, chi, js, 0.0, 20.0, 7)
    torch.cuda.synchronize()
    wall = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    ctx.set_timing(True)
    ctx.stage_times()
    ctx.qeq(ngrid, axis, atoms, chi, js, 0.0, 20.0, 7)
    st = {k: round(v[0], 3) for k, v in ctx.stage_times().items()}
    ctx.set_timing(False)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        rows = min(N, 64)
        t1 = time.perf_counter()
        O.qeq_matrix(atoms[:rows], np.eye(3) * (axis[0, 0] * ngrid[0]), 20.0, 7, js[:rows])
        t_rows = time.perf_counter() - t1
        t1 = time.perf_counter()
        O.qeq_charges(np.eye(N) + 0.01, chi, 0.0)   # LU time does not depend on the values
        t_solve = time.perf_counter() - t1
        pairs_sample = rows * (rows - 1) / 2
        t_cpu = t_rows * (N * (N - 1) / 2) / pairs_sample + t_solve
        cpu = {"value": 1.0 / t_cpu, "unit": "charge sets/s", "cores": 1, "kind": "port",
               "sample": f"oracle Coulomb matrix of the first {rows} atoms ({int(pairs_sample)} pairs, "
                         f"{t_rows:.2f} s) extrapolated to {N * (N - 1) // 2} pairs, plus its {N}-atom solve "
                         f"({t_solve:.2f} s)"}
    per = wall / args.steps
    K = 754
    line = {
        "metric": "QEq charge sets/s (periodic Ewald Coulomb matrix + equalisation solve, host in/out)",
        "value": args.steps * world / wall, "unit": "charge sets/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "pairs_per_s": N * (N - 1) / 2 / per, "stage_ms_one_step": st, "residual": info["residual"],
        "e2e": {"value": args.steps * world / wall, "unit": "charge sets/s",
                "h2d_bytes_per_step": 8 * (3 * N + 2 * N), "d2h_bytes_per_step": 8 * N},
        "config": {"workload": f"qeq: {N} atoms on a jittered 5 Bohr lattice (H/C/O/Zn), cubic cell "
                               f"{axis[0, 0] * ngrid[0]:.0f} Bohr, Rc 20 (27 images), KMAX 7 (K={K})"},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "mof", "water", "tric", "serve", "qeq"])
    ap.add_argument("--qeq-atoms", type=int, default=2000)
    ap.add_argument("--serve-requests", type=int, default=10000,
                    help="requests of the served stream (10,000 at 50/s: about 200 s); 0 leaves it out of the "
                         "default line")
    ap.add_argument("--serve-fp64-small", type=int, default=12, help="small pool cubes timed in plain FP64")
    ap.add_argument("--serve-fp64-large", type=int, default=2, help="large pool cubes timed in plain FP64")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="Poisson arrival rate, requests/s")
    ap.add_argument("--serve-pool", type=int, default=128, help="distinct batch-distribution cubes")
    ap.add_argument("--serve-large", type=int, default=8, help="distinct large cubes (800-1500 atoms, 160^3)")
    ap.add_argument("--serve-large-share", type=float, default=0.05)
    ap.add_argument("--serve-batch", type=int, default=64)
    ap.add_argument("--serve-wait-ms", type=float, default=4.0)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--n-cubes", type=int, default=256)
    ap.add_argument("--fp64-cubes", type=int, default=8, help="cubes of the plain FP64 comparator")
    ap.add_argument("--fp64-repeats", type=int, default=3, help="timed batches of the FP64 comparator")
    ap.add_argument("--latency-fits", type=int, default=32, help="single fits timed for p50/p99")
    ap.add_argument("--cpu-sample", type=int, default=120000,
                    help="kept points of the CPU baseline sample (capped at the cube's kept count; ~5-10 s of CPU)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tile shapes")
    ap.add_argument("--ref-cubes", type=int, default=8, help="cubes the reference arm cycles over")
    ap.add_argument("--ref-sample", type=int, default=40000,
                    help="kept points per reference-arm step (~2-4 s of host work on 16 cores)")
    args = ap.parse_args()

    world, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
        return
    if args.workload == "serve":
        serve_arm(args, world, rank, local)
        return
    if args.workload == "qeq":
        qeq_arm(args, world, rank, local)
        return

    import torch
    from pyrepeat_gb300 import _lib
    from pyrepeat_gb300.fit import Context
    torch.cuda.set_device(local)
    ctx = Context(local)
    dev = torch.device(f"cuda:{local}")

    t0 = time.time()
    cubes, desc = make_workload(args.workload, args.n_cubes, 1000 + 100000 * rank, ctx)
    gen_s = time.time() - t0
    n = len(cubes)
    V_dev = [c.V_dev for c in cubes]
    grid_bytes = sum(c.n_points * 8 for c in cubes)

    def step(prec=_lib.PREC_MIXED, sel=None):
        cs = cubes if sel is None else [cubes[i] for i in sel]
        vs = V_dev if sel is None else [V_dev[i] for i in sel]
        return ctx.fit_batch(cs, prec, V_dev=vs)

    # tile shapes: the autotuner times each (atoms, kept points, KMAX) bucket of the batch once
    tune = None
    if not args.no_autotune:
        import tempfile
        t_tune = time.time()
        table = ctx.autotune(cubes, os.path.join(tempfile.gettempdir(), f"repeat_gb300_tiles_{rank}.txt"))
        tune = {"buckets": len(table), "seconds": round(time.time() - t_tune, 2),
                "table": {str(k): {"phi_atoms": v[0], "gram_points_per_cta": 64 * v[1], "best_ms": round(v[2], 4),
                                   "default_ms": round(v[3], 4), "N": v[4], "M": v[5]} for k, v in table.items()}}

    # warm-up (the clock sampler starts here, so that its own start-up, which holds the
    # driver for a moment, falls outside the timed region)
    clock = ClockSampler(local)
    clock.start()
    for _ in range(max(args.warmup, 1)):
        q_mixed, M, info = step()
    torch.cuda.synchronize()

    # timed region: K batched steps, events on the stream the library runs on
    clock.mark()
    launches0 = _lib.launch_count()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        q_mixed, M, info = step()
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    launches = _lib.launch_count() - launches0
    clocks = clock.stop()
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, world, dev)
    value = n * args.steps * world / (ms / 1e3)
    q_mixed = [q.copy() for q in q_mixed]

    # end to end: grids from pinned host memory, charges back to the host
    pinned = [c.V_dev.cpu().pin_memory() for c in cubes]
    host_cubes = []
    for c, p in zip(cubes, pinned):
        hc = type(c)(**{k: getattr(c, k) for k in c.__dataclass_fields__})
        hc.V = p.numpy()
        hc.V_dev = None
        host_cubes.append(hc)
    qbuf = torch.zeros(sum(c.n_atoms for c in cubes), dtype=torch.float64).pin_memory().numpy()
    ctx.fit_batch(host_cubes, _lib.PREC_MIXED, out=qbuf)
    torch.cuda.synchronize()
    barrier(world)
    t_e2e = time.perf_counter()
    e2e_steps = []
    for _ in range(args.steps):
        ts = time.perf_counter()
        ctx.fit_batch(host_cubes, _lib.PREC_MIXED, out=qbuf)  # synchronous: charges are on the host
        e2e_steps.append(round(1e3 * (time.perf_counter() - ts), 2))
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t_e2e, world, dev)
    e2e_value = n * args.steps * world / e2e_s

    # plain FP64 GPU fit of a subset: speed and the accuracy of the mixed path against it
    nf = min(args.fp64_cubes, n)
    sel = list(range(nf))
    fp64_value = dq = mixed_sub_value = None
    fp64_reps = []
    if nf > 0:
        step(_lib.PREC_FP64, sel)   # warm-up over every cube of the subset
        torch.cuda.synchronize()
        for _ in range(args.fp64_repeats):
            tf = time.perf_counter()
            q64, _, _ = step(_lib.PREC_FP64, sel)
            torch.cuda.synchronize()
            fp64_reps.append(time.perf_counter() - tf)
        fp64_value = nf / statistics.median(fp64_reps)
        mixed_sub = [q_mixed[i] for i in sel]
        dq = max(float(np.abs(a - b).max()) for a, b in zip(mixed_sub, q64))
        mreps = []
        for _ in range(args.fp64_repeats):
            tm = time.perf_counter()
            step(_lib.PREC_MIXED, sel)
            torch.cuda.synchronize()
            mreps.append(time.perf_counter() - tm)
        mixed_sub_value = nf / statistics.median(mreps)

    # relative RMS of the fitted ESP over the kept points, both centred
    # (sqrt(sum (V_fit - V)^2 / sum V^2)), from rp_potential at the mixed charges
    rrms = []
    for i in range(min(8, n)):
        c = cubes[i]
        kept, Vc, _, _ = ctx.filter(c.n_grid, c.axis_vector, c.atom_pos, c.atom_index, c.V_dev, c.vdw_factor,
                                    c.vdw_max)
        ew = ctx.ewald(c.n_grid, c.axis_vector, c.cutoff, c.kmax)
        try:
            vfit = ctx.potential(ew, c.atom_pos, q_mixed[i], kept)
        finally:
            ew.close()
        d = (vfit - vfit.mean()) - (Vc - Vc.mean())
        rrms.append(float(torch.sqrt((d * d).sum() / (Vc * Vc).sum())))

    # single-fit latency (each cube alone through the batch entry point)
    lat = []
    for i in range(min(args.latency_fits, n)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        step(_lib.PREC_MIXED, [i])
        b.record()
        torch.cuda.synchronize()
        lat.append(a.elapsed_time(b))
    lat.sort()
    p50 = lat[len(lat) // 2]
    p99 = lat[min(len(lat) - 1, int(math.ceil(0.99 * len(lat))) - 1)]

    # roofline of the dominant stage from live CUDA-event stage timings of one more step
    # (with timing on, the library runs the batch's fits on one stream, so every stage is
    # timed alone; the timed steps above overlap fits on four streams)
    ctx.set_timing(True)
    ctx.stage_times()
    step()
    stages = ctx.stage_times()
    ctx.set_timing(False)
    bf16_peak, hbm_peak, peak_kind = peaks()
    Ms = [int(m) for m in M]
    # algorithmic work per stage over the whole batch (one step)
    flops_gram, b_phi, b_slice, b_rows, b_filter, pairs = 0.0, 0.0, 0.0, 0.0, 0.0, 0.0
    for c, m in zip(cubes, Ms):
        na = c.n_atoms
        nx, ny, nz = c.n_grid
        pairs += float(m) * na
        flops_gram += 2.0 * m * (na + 1) ** 2                   # X X^T over the atoms + the ESP row
        b_phi += 8.0 * m * na + 4.0 * m                         # Phi written once, kept index read
        b_slice += 8.0 * m * na + 8.0 * m * (na + 1) + 8.0 * m  # Phi read, 4 FP16 digits written, Vc read
        b_rows += 8.0 * ny * nz * na * c.kmax                   # E rows written (FP32 complex, KMAX per row)
        b_filter += 9.0 * nx * ny * nz + 12.0 * m            # V read + mask, kept index + Vc written
    algo = {"gram_exact": ("tensor", flops_gram / 1e12, "TFLOP/s", bf16_peak, "bf16 dense burst"),
            "phi": ("hbm", b_phi / 1e9, "GB/s", hbm_peak, "copy"),
            "center_slice": ("hbm", b_slice / 1e9, "GB/s", hbm_peak, "copy"),
            "recip_rows": ("hbm", b_rows / 1e9, "GB/s", hbm_peak, "copy"),
            "filter": ("hbm", b_filter / 1e9, "GB/s", hbm_peak, "copy")}
    rooflines = {}
    for name, (bound, work, unit, peak, pk) in algo.items():
        if name in stages and stages[name][0] > 0:
            ms_, n_ = stages[name]
            ach = work / (ms_ / 1e3)
            rooflines[name] = {"bound": bound, "achieved": ach, "peak": peak, "unit": unit, "frac": ach / peak,
                               "launches": n_, "avg_launch_ms": ms_ / max(n_, 1),
                               "peak_kind": f"{pk}, {peak_kind}"}
    dom_name = max(stages.items(), key=lambda kv: kv[1][0])[0] if stages else "none"
    roof = dict(rooflines.get(dom_name, {"bound": None, "achieved": None, "peak": None, "unit": None, "frac": None}))
    roof["kernel"] = dom_name
    roof["traffic"] = None
    if dom_name == "phi":
        # phi_chunk_kernel: one ncu capture (PHI_CAPTURE) measured
        # PHI_DRAM_PER_PAIR DRAM bytes and PHI_INST_PER_PAIR thread instructions per point-atom
        # pair; traffic is that times the pairs of an average launch.  The kernel is bound by
        # instruction issue (FP32/ALU pipes), not by HBM: "issue" relates its live instruction
        # rate to the nominal issue peak (4 warp instructions per clock per SM at the SM clock).
        n_l = max(stages["phi"][1], 1)
        roof["kernel"] = "phi_chunk_kernel"
        roof["traffic"] = PHI_DRAM_PER_PAIR * pairs / n_l
        roof["traffic_source"] = (f"{PHI_DRAM_PER_PAIR} DRAM bytes per point-atom pair from the ncu capture in "
                                  f"{PHI_CAPTURE}, times this step's pairs per launch; not re-measured in this run")
        roof["point_atom_evals_per_s"] = pairs / (stages["phi"][0] / 1e3)
        sm_mhz = clocks.get("sm_mhz") or 2070.0
        peak_inst = 152 * 4 * 32 * sm_mhz * 1e6
        ach_inst = PHI_INST_PER_PAIR * pairs / (stages["phi"][0] / 1e3)
        roof["issue"] = {"achieved_thread_inst_per_s": ach_inst, "peak_thread_inst_per_s": peak_inst,
                         "frac": ach_inst / peak_inst, "peak_kind": "nominal issue rate at the sampled SM clock",
                         "inst_per_pair": PHI_INST_PER_PAIR, "inst_source": PHI_CAPTURE}
    stage_share = {k: round(v[0], 3) for k, v in sorted(stages.items(), key=lambda kv: -kv[1][0])}

    # the served stream (one GPU): continuous batching of Poisson arrivals beside plain FP64
    served = None
    if world == 1 and args.serve_requests > 0 and args.workload == "batch":
        try:
            served = served_stream(ctx, args, rank)
        except Exception as e:  # noqa: BLE001 - reported in the line, the batch figures stand
            served = {"error": f"{type(e).__name__}: {e}"}

    # CPU oracle on a bounded sample (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = max(1, os.cpu_count() or 1)
        c0 = cubes[0]
        dt, s, Mc = cpu_oracle_sample(c0, args.cpu_sample, threads)
        per_cube = dt * Mc / s
        mean_M = statistics.mean(Ms)
        cpu_value = 1.0 / (per_cube * mean_M / Mc)
        cpu = {"value": cpu_value, "unit": "fits/s", "cores": threads, "kind": "port",
               "sample": f"cube 0 (N={c0.n_atoms}, M={Mc}), {s} seeded kept points, {dt:.2f} s; extrapolated "
                         f"linearly to the batch's mean kept count {mean_M:.0f}"}

    if rank != 0:
        return
    h2d = grid_bytes
    d2h = sum(c.n_atoms for c in cubes) * 8
    line = {
        "metric": METRIC, "value": value, "unit": "fits/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+double-float+exact-int+f64",
        "data": "synthetic: seeded cubes, ESP = Ewald potential of planted charges + N(0,1e-4) (rp_potential)",
        "config": {"workload": desc, "n_cubes": n, "grid_bytes": grid_bytes,
                   "l2": "inputs larger than L2 (%.2f GB of grids per step)" % (grid_bytes / 1e9),
                   "generation_s": round(gen_s, 1)},
        "p50_ms": p50, "p99_ms": p99, "latency": "single-fit, each cube alone through rp_fit_batch",
        "fp64": {"fits_per_s": fp64_value, "cubes": nf, "mixed_fits_per_s_same_cubes": mixed_sub_value,
                 "speedup": (mixed_sub_value / fp64_value) if nf else None, "max_dq_mixed_vs_fp64_e": dq,
                 "timing": f"median of {args.fp64_repeats} host-timed batches of the {nf} cubes after a warm-up "
                           f"batch of the same cubes; both arms fit the same cubes through rp_fit_batch",
                 "fp64_batch_s": fp64_reps},
        "rrms": {"median": float(np.median(rrms)), "max": float(np.max(rrms)), "cubes": len(rrms),
                 "definition": "sqrt(sum (V_fit - V)^2 / sum V^2) over kept points, both centred"},
        "e2e": {"value": e2e_value, "unit": "fits/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "step_ms": e2e_steps,
                "inputs": "each step's grids (h2d_bytes_per_step) from page-locked host memory; the filter reads "
                          "them in place over the host link at the kept points only (kept_bytes_read_per_step), "
                          "charges back to page-locked host memory",
                "kept_bytes_read_per_step": 8 * int(sum(Ms))},
        "gpu_launches": launches,
        "roofline": roof,
        "stage_rooflines": rooflines,
        "stage_ms_one_step": stage_share,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "served": served,
        "autotune": tune,
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
