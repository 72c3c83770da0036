"""Benchmark of the DMR restart cycle on GB300: solves/s and p50/p99 latency at
1e-10 FP64 relative residual, batched mixed precision vs plain FP64.

Workload (one GPU): 3D 7-point shifted Helmholtz on a 96^3 grid (kappa 24,
damping 0.1, n = 884,736, 6.14M non-zeros, CSR -> SELL-32), 64 right-hand
sides (unit Gaussian sources of sigma 3 cells at seeded positions plus 1%
complex noise), basis m = 48 with k = 24 recycled deflation vectors shared by
all 64, tolerance 1e-10 on the true FP64 residual.  One step = one batched
solve of all 64 right-hand sides from x = 0 and a cold deflation space,
through the C ABI (gdmr_solve_batch): complex64 inner DMR cycles, FP64
residual and solution.  The working set (~27 GB) is far larger than L2, so no
flush is needed between steps.

Also reported: `e2e` (the same step with the right-hand sides and solutions
in pinned host memory, copies inside the timed region), timed samples of
the plain forms (reference algorithm, one right-hand side at a time with
recycling) in native complex128 (the drop-in) and in fp64e (the same
iteration in double-float arithmetic on the FP32 pipes) with the HBM
fraction of their kernel classes, the roofline of the dominant kernel class
from CUDA events recorded by the library on its own stream, the SM clocks
during the timed region, and the host oracle as CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun each rank solves its own 64 right-hand sides (seeds offset by
rank): independent systems, no collective on the data path ("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gdmr-solver_gb300"))

import problems  # noqa: E402

METRIC = "solves/s + p50/p99 latency at 1e-10 rel. residual: mixed batched vs plain FP64"
SHAPE = (96, 96, 96)
KAPPA, DAMPING, M, K, TOL = 24.0, 0.1, 48, 24, 1e-10


# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic byte, per kernel
# class, measured by ncu over three batched cycles of this same workload with the tensor-core
# shared-basis kernels in use.
TRAFFIC_PER_ALGORITHMIC_BYTE = {"projection": 1.027, "update": 1.043, "operator": 0.938, "combine": 1.000,
                                "deflation_update": 1.303, "residual64": 1.478, "other": 0.949}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl != "reference" else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(value, world):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
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
        os.remove(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def build_workload(nrhs: int, rank: int, shape=SHAPE):
    A = problems.helmholtz(shape, KAPPA, DAMPING)
    B = np.stack([problems.gaussian_source_rhs(shape, seed) for seed in problems.shard_seeds(nrhs, rank)])
    return A, B


def class_table(prof: dict, hbm_peak: float) -> dict:
    """Per kernel class: algorithmic GB/s, fraction of the HBM peak, share of kernel time."""
    tot = sum(v["ms"] for v in prof.values()) or 1.0
    out = {}
    for k, v in prof.items():
        if not v["launches"]:
            continue
        gbs = v["bytes"] / (v["ms"] / 1e3) / 1e9 if v["ms"] > 0 else None
        out[k] = {"GB/s": gbs, "frac": (gbs / hbm_peak) if gbs else None, "share": v["ms"] / tot,
                  "launches": v["launches"]}
    return out


def workload_config(A, nrhs: int, shape=SHAPE, m_basis: int = M) -> dict:
    """The workload as both arms name it (the same dict in the reference arm's line)."""
    return {"workload": f"helmholtz{shape[0]}_{nrhs}rhs", "grid": list(shape), "n": int(A.n), "nnz": int(A.nnz),
            "kappa": KAPPA, "damping": DAMPING, "nrhs_per_gpu": nrhs, "m": m_basis, "k": K, "tol": TOL,
            "form": "mixed batched (complex64 inner DMR, FP64 true residual each cycle)",
            "l2": "working set ~27 GB >> 129 MB L2; no flush"}


def oracle_deflated_cycles(o, b, cycles: int, warm: bool):
    """`cycles` deflated restart cycles of the host oracle on one right-hand side, each timed by
    the oracle itself.  warm: the oracle already holds a deflation space (every cycle of a mode-1
    solve is deflated); otherwise one undeflated cycle builds it first and is not counted."""
    if warm:
        r = o.solve(b, mode=1, tol=TOL, mat_rank=cycles - 1)
        ms = r["cycle_ms"]
    else:
        r = o.solve(b, mode=0, tol=TOL, mat_rank=cycles)
        ms = r["cycle_ms"][1:]
    return float(np.mean(ms)) / 1e3, len(ms)


def cpu_baseline(A, b, cycles: int, cycles_per_solve: int, rhs_seed: int):
    """The host oracle (complex128 DMR, all host threads) on `cycles` deflated restart cycles of
    one right-hand side of the same workload; solves/s = 1 / (seconds per deflated cycle x the
    cycles the plain FP64 GPU form took to solve that right-hand side in this run)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    o = oracle.Oracle(A, M, K, threads=threads, fuse_deflation=True)
    t = time.perf_counter()
    per_cycle, timed = oracle_deflated_cycles(o, b, cycles, warm=False)
    el = time.perf_counter() - t
    return {"value": 1.0 / (per_cycle * cycles_per_solve), "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": f"right-hand side seed {rhs_seed} of the full workload: one undeflated restart cycle, "
                      f"then {timed} deflated cycles timed one by one ({per_cycle:.3f} s each; {el:.1f} s in all); "
                      f"x {cycles_per_solve} cycles, the plain FP64 GPU form's count for this right-hand side"}


def run_reference(args, world, rank):
    """Reference arm: the host oracle (the reference has no CPU implementation of this path) on
    the same workload.  Calibration, untimed: one full solve of right-hand side seed 100, whose
    cycle count converts seconds per cycle into solves/s.  Each step: `ref_cycles` deflated
    restart cycles of the same right-hand side (a mode-1 solve on the calibration's deflation
    space), timed cycle by cycle by the oracle."""
    if rank != 0:
        return
    shape = (args.grid,) * 3
    A = problems.helmholtz(shape, KAPPA, DAMPING)
    seed = problems.shard_seeds(1, 0)[0]
    b = problems.gaussian_source_rhs(shape, seed)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    threads = os.cpu_count() or 1
    o = oracle.Oracle(A, M, K, threads=threads, fuse_deflation=True)
    t = time.perf_counter()
    full = o.solve(b, mode=0, tol=TOL, mat_rank=args.max_cycles)
    full_s = time.perf_counter() - t
    cycles_per_solve = int(full["cycles"])
    per = []
    step_s = []
    for step in range(args.warmup + args.steps):
        t = time.perf_counter()
        pc, _ = oracle_deflated_cycles(o, b, args.ref_cycles, warm=True)
        el = time.perf_counter() - t
        if step >= args.warmup:
            per.append(pc)
            step_s.append(el)
    per_cycle = float(np.mean(per))
    value = 1.0 / (per_cycle * cycles_per_solve)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(step_s)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic", "config": workload_config(A, args.nrhs, shape),
            "calibration": {"rhs_seed": seed, "cycles": cycles_per_solve, "status": int(full["status"]),
                            "relative_residual": float(full["ret"]), "full_solve_s": full_s,
                            "full_solve_solves_s": 1.0 / full_s},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"{args.ref_cycles} deflated restart cycles of right-hand side seed {seed} per "
                                       f"step ({per_cycle:.3f} s each), x {cycles_per_solve} cycles, the count of "
                                       f"one full oracle solve of it ({full_s:.1f} s, untimed calibration)"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_serve(args, rank):
    """Serving workload: six resident operators (7-point Helmholtz 64^3 /
    96^3 / 128^3 with kappa 16 / 24 / 32, each at damping 0.05 and 0.2), m = 48, k = 24 per
    operator, device memory bounded by a 150 GB budget split evenly across the operators; each
    request picks an operator uniformly and brings one Gaussian-source right-hand side with a
    tolerance drawn from {1e-6, 1e-8, 1e-10}.  Two phases per precision: capacity (a burst of
    requests submitted at once; solves/s while the queues stay full), then Poisson arrivals at
    `--load` times that capacity for `--duration` seconds, so that the p50/p99 latencies measure
    service and the queueing a stated load brings, not an unbounded queue."""
    import gdmr
    gdmr.load()
    specs = [((64,) * 3, 16.0), ((96,) * 3, 24.0), ((128,) * 3, 32.0)]
    mats = [problems.helmholtz(shape, kappa, damping) for shape, kappa in specs for damping in (0.05, 0.2)]
    shapes = [shape for shape, _ in specs for _ in (0.05, 0.2)]
    pools = [[problems.gaussian_source_rhs(shapes[i], 7000 + 97 * (i + 1) + j) for j in range(args.serve_pool)]
             for i in range(len(mats))]
    budget = int(args.budget_gb * (1 << 30))
    forms = ["mixed", "fp64"] if args.serve_precision == "both" else [args.serve_precision]
    out = {}
    for form in forms:
        rng = np.random.default_rng(4)
        srv = gdmr.Server(budget_bytes=budget, device=0)
        share = budget // len(mats)
        ops = []
        for A in mats:
            per = gdmr.load().gdmr_server_slot_bytes(A.n, M, 1 if form == "mixed" else 0)
            fixed = A.nnz * 40 + A.n * 16 * (3 * K + 1) + (64 << 20)
            cap = int(max(1, min(args.serve_slots, (share - fixed) // per)))
            ops.append(srv.add_operator(A, M, K, capacity=cap, precision=form))
        srv.start()

        def run_requests(nreq, gaps):
            choice = rng.integers(0, len(ops), nreq)
            tols = rng.choice([1e-6, 1e-8, 1e-10], nreq)
            tickets = []
            t0 = time.perf_counter()
            t_next = t0
            for i in range(nreq):
                if gaps is not None:
                    t_next += gaps[i]
                    delay = t_next - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                j = int(choice[i])
                tickets.append((float(tols[i]), srv.submit(ops[j], pools[j][i % args.serve_pool], tol=float(tols[i]))))
            lat, ok = [], True
            for tol, t in tickets:
                x, st = srv.wait(t, timeout=3600)
                lat.append(st["latency_ms"])
                ok &= st["status"] == 0 and st["true_rel_res"] <= tol
            wall = time.perf_counter() - t0
            return {"solves_s": nreq / wall, "requests": nreq, "wall_s": wall,
                    "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                    "verified": bool(ok)}

        burst = run_requests(args.serve_burst, None)
        rate = args.load * burst["solves_s"]
        nreq = max(1, int(rate * args.duration))
        poisson = run_requests(nreq, rng.exponential(1.0 / rate, nreq))
        poisson.update({"rate_req_s": rate, "load": args.load, "arrival_window_s": args.duration})
        out[form] = {"capacity": burst, "poisson": poisson, "slots": [srv.capacity(o) for o in ops],
                     "device_bytes": srv.device_bytes}
        srv.close()
    head = out[forms[0]]["poisson"]
    line = {"mode": "serve", "metric": METRIC, "value": head["solves_s"], "unit": "solves/s",
            "latency_ms": head["latency_ms"], "forms": out,
            "config": {"workload": "serve6_helmholtz", "budget_gb": args.budget_gb, "m": M, "k": K,
                       "operators": "64^3/96^3/128^3 x damping 0.05/0.2", "tolerances": [1e-6, 1e-8, 1e-10]}}
    if len(forms) == 2:
        line["mixed_over_plain"] = out["mixed"]["capacity"]["solves_s"] / out["fp64"]["capacity"]["solves_s"]
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_sequence(args, rank):
    """Drifting-sequence workload: 3D 7-point Helmholtz 128^3 (kappa 30, damping 0.1,
    n = 2,097,152), right-hand sides b_1 a unit complex Gaussian and b_(j+1) = b_j + 0.05 ||b_j||
    g_j / ||g_j||, solved one after another with the recycled deflation space (m = 60, k = 20,
    tol 1e-10): plain complex128 (the drop-in, gdmr_solve mode 0 then 1), fp64e, and the
    complex64-inner / FP64-refined form (gdmr_solve_batch one right-hand side at a time, the
    system's deflation space carried from call to call), on the first --seq-count of the 32.
    Each form first solves b_1 once untimed (kernel tuning), then drops its deflation space."""
    import gdmr
    gdmr.load()
    A, seq, cfg = problems.config_3d128()
    B = seq(args.seq_count)
    tol = cfg["tol"]
    S = A.to_scipy()
    out = {}
    for form in ("mixed", "fp64e", "fp64"):
        s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision=form)
        if form == "mixed":
            s.solve_batch(B[:1], tol=tol, max_cycles=args.max_cycles)
        else:
            s.solve(B[0], mode=0, tol=tol, mat_rank=args.max_cycles)
        s.drop_deflation()
        cyc, lat, worst, ok = [], [], 0.0, True
        t0 = time.perf_counter()
        for i, b in enumerate(B):
            t = time.perf_counter()
            if form == "mixed":
                X, st = s.solve_batch(b[None], tol=tol, max_cycles=args.max_cycles)
                x, st = X[0], st[0]
            else:
                x, st = s.solve(b, mode=0 if i == 0 else 1, tol=tol, mat_rank=args.max_cycles)
            lat.append(time.perf_counter() - t)
            cyc.append(int(st["cycles"]))
            ok &= st["status"] == 0
            worst = max(worst, float(np.linalg.norm(b - S @ x) / np.linalg.norm(b)))
        el = time.perf_counter() - t0
        out[form] = {"solves_s": len(B) / el, "cycles": cyc, "latency_s_each": lat, "verified": bool(ok),
                     "host_worst_true_rel_res": worst}
        s.close()
    line = {"mode": "sequence", "metric": METRIC, "value": out["mixed"]["solves_s"], "unit": "solves/s",
            "forms": out, "mixed_over_plain": out["mixed"]["solves_s"] / out["fp64"]["solves_s"],
            "mixed_over_fp64e": out["mixed"]["solves_s"] / out["fp64e"]["solves_s"],
            "config": {"workload": "helmholtz128_drifting_sequence", "n": int(A.n), "nnz": int(A.nnz),
                       "kappa": 30.0, "damping": 0.1, "m": cfg["m"], "k": cfg["k"], "tol": tol,
                       "rhs": len(B), "of": 32}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_multi_operator(args, rank):
    """Many-operator workload: 48 independent operators, 3D 7-point -div(a grad u) - kappa^2 (1+0.1i) u
    with per-axis edge lengths log-uniform in [32, 128] (seeded), a piecewise constant on 8^3
    blocks (Re U[1,4], Im U[0,0.2]), kappa 16; 4 complex Gaussian right-hand sides each;
    m = 40, k = 16, tolerance 1e-9.  Two forms over the same operators and right-hand sides:
      * lockstep: gdmr_multi_solve, the restart cycles of all 48 in lockstep and the Krylov loops of
        every right-hand side in flight in one cooperative launch a cycle (the headline value);
      * streams: the serving layer, one engine, stream and worker thread per operator, their
        cycles overlapping on the device.
    The metric is solves/s over the whole set (192 solves) and p50/p99 latency."""
    import gdmr
    gdmr.load()
    u = problems.uniform01(31, 3 * args.operators)
    shapes = [tuple(int(round(math.exp(math.log(32) + (math.log(128) - math.log(32)) * u[3 * i + a])))
                    for a in range(3)) for i in range(args.operators)]
    mats = [problems.variable_helmholtz(sh, 16.0, 0.1, seed=500 + i) for i, sh in enumerate(shapes)]
    per_op = args.rhs_per_operator
    rhs = [np.array([problems.unit_gaussian_rhs(A.n, 9000 + 10 * i + j) for j in range(per_op)])
           for i, A in enumerate(mats)]
    forms = {}
    if args.multi_tail >= 0:
        gdmr.multi_tail(args.multi_tail)
    tail = gdmr.multi_tail()
    # lockstep: warm-up of the per-operator kernels' tuning on a first solve, then the timed one
    systems = [gdmr.System(A, 40, 16, capacity=per_op, precision=args.serve_precision if
                           args.serve_precision != "both" else "mixed") for A in mats]
    gdmr.multi_solve(systems, [B[:1] for B in rhs], tol=1e-9, max_cycles=3)
    for s in systems:
        s.drop_deflation()
    t0 = time.perf_counter()
    out = gdmr.multi_solve(systems, rhs, tol=1e-9, max_cycles=5000)
    wall = time.perf_counter() - t0
    lat = [st["latency_ms"] for _, stats in out for st in stats]
    cyc = [st["cycles"] for _, stats in out for st in stats]
    ok = all(st["status"] == 0 and st["true_rel_res"] <= 1e-9 for _, stats in out for st in stats)
    host = max(float(np.linalg.norm(B[i] - A.to_scipy() @ X[i]) / np.linalg.norm(B[i]))
               for A, B, (X, _) in zip(mats, rhs, out) for i in range(B.shape[0]))
    forms["lockstep"] = {"solves_s": len(lat) / wall, "wall_s": wall,
                         "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                         "cycles": {"mean": float(np.mean(cyc)), "max": int(np.max(cyc))}, "verified": bool(ok),
                         "host_worst_true_rel_res": host, "tail": tail}
    for s in systems:
        s.close()
    # streams: the serving layer
    srv = gdmr.Server(budget_bytes=int(args.budget_gb * (1 << 30)), device=0)
    ops = [srv.add_operator(A, 40, 16, capacity=per_op, precision="mixed") for A in mats]
    srv.start()
    t0 = time.perf_counter()
    tickets = [(i, srv.submit(ops[i], rhs[i][j], tol=1e-9)) for i in range(len(mats)) for j in range(per_op)]
    lat, ok, cyc = [], True, []
    for i, t in tickets:
        x, st = srv.wait(t, timeout=3600)
        lat.append(st["latency_ms"])
        cyc.append(st["cycles"])
        ok &= st["status"] == 0 and st["true_rel_res"] <= 1e-9
    wall = time.perf_counter() - t0
    srv.close()
    forms["streams"] = {"solves_s": len(tickets) / wall, "wall_s": wall,
                        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                        "cycles": {"mean": float(np.mean(cyc)), "max": int(np.max(cyc))}, "verified": bool(ok)}
    head = forms["lockstep"]
    line = {"mode": "multi-operator", "metric": METRIC, "value": head["solves_s"], "unit": "solves/s",
            "latency_ms": head["latency_ms"], "solves": len(tickets), "forms": forms,
            "n_range": [min(A.n for A in mats), max(A.n for A in mats)],
            "config": {"workload": "variable_helmholtz_48ops", "operators": len(mats), "rhs_per_operator": per_op,
                       "m": 40, "k": 16, "tol": 1e-9, "precision": "mixed"}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_small(args, rank):
    """The reference-parity case: 2D 5-point Helmholtz 64x64, kappa 20,
    damping 0.05; 8 unit Gaussian right-hand sides solved in sequence with the recycled
    deflation space (mode 0 then 1); m = 40, k = 10, tol 1e-10; the plain FP64 drop-in
    (reference algorithm in complex128) through gdmr_solve, with and without CUDA graphs,
    beside the host oracle on all host cores."""
    import gdmr
    gdmr.load()
    A, rhs, cfg = problems.config_2d64()
    out = {}
    for graphs in (False, True):
        s = gdmr.System(A, cfg["m"], cfg["k"], capacity=1, precision="fp64")
        s.set_graphs(graphs)
        s.solve(rhs[0], mode=0, tol=cfg["tol"], mat_rank=2000)      # warm-up (tuning, first capture)
        s.drop_deflation()
        t = time.perf_counter()
        cyc, ok = [], True
        for i, b in enumerate(rhs):
            x, st = s.solve(b, mode=0 if i == 0 else 1, tol=cfg["tol"], mat_rank=2000)
            cyc.append(st["cycles"])
            ok &= st["status"] == 0 and st["true_rel_res"] <= 2 * cfg["tol"]
        el = time.perf_counter() - t
        out["graphs" if graphs else "eager"] = {"solves_s": len(rhs) / el, "ms_per_solve": el / len(rhs) * 1e3,
                                                "cycles": cyc, "verified": bool(ok)}
        if not graphs:
            gdmr.profile_reset()
            gdmr.profile(True)
            s.solve(rhs[0], mode=1, tol=cfg["tol"], mat_rank=2000)
            gdmr.profile(False)
            pp = gdmr.profile_read()
            pt = sum(v["ms"] for v in pp.values())
            out["eager"]["classes_ms_share"] = {k: round(v["ms"] / pt, 4) for k, v in pp.items() if v["launches"]}
            out["eager"]["kernel_ms_per_cycle"] = pt / max(1, st["cycles"])
        s.close()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    o = oracle.Oracle(A, cfg["m"], cfg["k"], threads=os.cpu_count() or 1, fuse_deflation=True)
    t = time.perf_counter()
    ocyc = [o.solve(b, mode=0 if i == 0 else 1, tol=cfg["tol"], mat_rank=2000)["cycles"] for i, b in enumerate(rhs)]
    el = time.perf_counter() - t
    line = {"mode": "small", "metric": METRIC, "value": out["graphs"]["solves_s"], "unit": "solves/s",
            "plain_fp64": out, "cpu_oracle": {"solves_s": len(rhs) / el, "cycles": ocyc, "cores": os.cpu_count()},
            "config": {"workload": "helmholtz2d64_8rhs", "n": A.n, "nnz": A.nnz, "m": cfg["m"], "k": cfg["k"],
                       "tol": cfg["tol"]}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nrhs", type=int, default=64)
    ap.add_argument("--plain-sample", type=int, default=2, help="right-hand sides timed in the plain FP64 form")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--cpu-cycles", type=int, default=12, help="deflated oracle cycles timed for cpu_baseline")
    ap.add_argument("--ref-cycles", type=int, default=2, help="deflated oracle cycles per reference-arm step")
    ap.add_argument("--max-cycles", type=int, default=3000)
    ap.add_argument("--serve", action="store_true", help="serving workload instead of the batched bench")
    ap.add_argument("--multi-operator", action="store_true", help="48-operator workload instead of the batched bench")
    ap.add_argument("--small", action="store_true", help="64x64 reference-parity case (plain FP64 drop-in)")
    ap.add_argument("--sequence", action="store_true",
                    help="128^3 drifting sequence of right-hand sides: plain complex128, fp64e and mixed")
    ap.add_argument("--seq-count", type=int, default=4, help="right-hand sides of the sequence timed (of 32)")
    ap.add_argument("--operators", type=int, default=48)
    ap.add_argument("--multi-tail", type=int, default=-1,
                    help="multi-operator: systems in flight at which the lockstep hands over (-1: library default)")
    ap.add_argument("--rhs-per-operator", type=int, default=4)
    ap.add_argument("--serve-precision", default="both", choices=["mixed", "fp64", "both"])
    ap.add_argument("--load", type=float, default=0.7,
                    help="serving: Poisson arrival rate as a fraction of the measured capacity")
    ap.add_argument("--serve-burst", type=int, default=48, help="serving: requests of the capacity phase")
    ap.add_argument("--duration", type=float, default=60.0, help="serving: Poisson arrival window in seconds")
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-slots", type=int, default=64)
    ap.add_argument("--serve-pool", type=int, default=4)
    ap.add_argument("--solve-only", action="store_true",
                    help="only the timed batched solves (for profiler captures); prints a short line")
    ap.add_argument("--grid", type=int, default=SHAPE[0],
                    help="edge of the cubic grid (profiling captures of the batched kernels use a smaller one)")
    ap.add_argument("--m", type=int, default=M, help="basis size m (profiling captures)")
    ap.add_argument("--stencil", action="store_true",
                    help="matrix-free 7-point operator for the inner cycles (default: the CSR operator)")
    ap.add_argument("--grid-batch", type=int, default=0, choices=[0, 1, 2, 4],
                    help="batched operator products on the structured-grid kernel with this many systems a "
                         "thread (0: the SELL-32 kernel, the library's default for batches)")
    ap.add_argument("--sell", action="store_true",
                    help="CSR operator products on the SELL-32 kernels (default: the structured-grid kernel, "
                         "which the 7-point CSR operator qualifies for)")
    ap.add_argument("--force-variants", default=None, metavar="P,U",
                    help="pin the Gram-Schmidt projection and update variants (gdmrTuneForce)")
    ap.add_argument("--plain", default=None, choices=["fp64", "fp64e"],
                    help="only the plain-form sample in this precision (for profiler captures); short line")
    ap.add_argument("--profile-classes", action="store_true",
                    help="with --solve-only: record the library's per-class algorithmic bytes and CUDA-event "
                         "times over the timed steps (tuning off) and print them")
    args = ap.parse_args()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    if args.serve:
        run_serve(args, rank)
        return
    if args.multi_operator:
        run_multi_operator(args, rank)
        return
    if args.small:
        run_small(args, rank)
        return
    if args.sequence:
        run_sequence(args, rank)
        return

    import torch
    torch.cuda.set_device(local)
    import gdmr
    gdmr.load()
    hbm_peak, peak_kind = peaks()

    if args.force_variants:
        gdmr.tune_force(*(int(v) for v in args.force_variants.split(",")))
    if args.sell:
        gdmr.grid_operator(False)
    if args.grid_batch:
        gdmr.grid_batch(args.grid_batch)
    shape = (args.grid,) * 3
    A, B = build_workload(args.nrhs, rank, shape)
    nrhs, n = B.shape
    m_basis = args.m
    if args.plain:
        # plain-form sample only: one right-hand side at a time, no batched engine
        res = plain_form_only(args, A, B, m_basis, local, hbm_peak)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return
    sysm = gdmr.System(A, m_basis, K, capacity=nrhs, precision="mixed", device=local)
    if args.stencil:
        sysm.set_stencil(shape, *problems.helmholtz_stencil(shape, KAPPA, DAMPING))
    op_kernel = ("matrix-free stencil (k_stencil)" if args.stencil else
                 f"structured grid (k_grid_spmm, {args.grid_batch} systems a thread)"
                 if sysm.grid_shape() and not args.sell and args.grid_batch else
                 "SELL-32 (k_spmm) for the batch, structured grid (k_grid_spmm) for single vectors"
                 if sysm.grid_shape() and not args.sell else "SELL-32 (k_spmm, k_spmv2)")
    Bd = torch.from_numpy(B).to(f"cuda:{local}")
    Xd = torch.zeros_like(Bd)
    tols = [TOL] * nrhs

    def step():
        sysm.drop_deflation()
        Xd.zero_()
        torch.cuda.synchronize()
        return sysm.solve_batch_device(Bd.data_ptr(), Xd.data_ptr(), nrhs, tols, max_cycles=args.max_cycles)

    for _ in range(args.warmup):
        step()
    if args.profile_classes:
        gdmr.profile_reset()
        gdmr.profile(True)
    # timed region: device-resident inputs
    lat, cycles, verified, worst_res = [], [], True, 0.0
    barrier(world)
    torch.cuda.synchronize()
    l0 = gdmr.kernel_launches()
    with ClockSampler(local) as clk:
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(args.steps):
            stats = step()
            lat.extend(s["latency_ms"] for s in stats)
            cycles.extend(s["cycles"] for s in stats)
            for s in stats:
                verified &= s["status"] == 0 and s["true_rel_res"] <= TOL
                worst_res = max(worst_res, s["true_rel_res"])
        ev1.record()
        torch.cuda.synchronize()
    barrier(world)
    launches = gdmr.kernel_launches() - l0
    elapsed_ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    value = world * nrhs * args.steps / (elapsed_ms / 1e3)
    clocks = clk.summary()
    # the last timed step's solutions, checked on the host in FP64 (SciPy CSR), independently of
    # the library's own residual kernel
    host_worst, host_check = host_residuals(A, B, Xd.cpu().numpy())
    if args.solve_only:
        out = {"mode": "solve-only", "operator": "stencil" if args.stencil else "csr", "operator_kernel": op_kernel,
               "value": value,
               "unit": "solves/s", "nrhs": nrhs,
               "ms_per_step": elapsed_ms / args.steps, "verified": bool(verified),
               "gpu_launches": int(launches), "svd_sweeps": sysm.svd_sweeps(),
               "tuning": gdmr.tune_report().strip().splitlines()}
        if args.profile_classes:
            gdmr.profile(False)
            out["classes"] = {k: v for k, v in gdmr.profile_read().items() if v["launches"]}
        if rank == 0:
            print(json.dumps(out), flush=True)
        return

    # roofline: one more step with library-side CUDA events per kernel class
    gdmr.profile_reset()
    gdmr.profile(True)
    step()
    gdmr.profile(False)
    prof = gdmr.profile_read()
    dom = max((k for k in prof if prof[k]["ms"] > 0), key=lambda k: prof[k]["ms"])
    tot_ms = sum(v["ms"] for v in prof.values())
    d = prof[dom]
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    ratio = TRAFFIC_PER_ALGORITHMIC_BYTE.get(dom)
    per_launch = d["bytes"] / max(1, d["launches"])
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": per_launch,
                "traffic": ratio * per_launch if ratio is not None else None,
                "traffic_basis": (f"ncu DRAM bytes = {ratio} x algorithmic bytes for this class "
                                  "(every launch of 3 cycles of this workload), times this run's mean "
                                  "algorithmic bytes per launch") if ratio is not None else None,
                "share": d["ms"] / tot_ms, "classes": class_table(prof, hbm_peak)}

    # e2e: host buffers (pinned), copies inside the timed region, through the C ABI
    # (the zero initial guesses are the caller's data: written before the clock starts)
    Bh = torch.from_numpy(B).pin_memory()
    Bh_np = Bh.numpy()
    Xhs = [torch.zeros_like(Bh).pin_memory().numpy() for _ in range(args.e2e_steps)]
    torch.cuda.synchronize()
    t = time.perf_counter()
    for Xh_np in Xhs:
        sysm.drop_deflation()
        X, st_e2e = _solve_host(sysm, Bh_np, Xh_np, args.max_cycles)
    e2e_s = max_over_ranks(time.perf_counter() - t, world)
    e2e = {"value": world * nrhs * args.e2e_steps / e2e_s, "unit": "solves/s",
           "h2d_bytes_per_step": int(2 * B.nbytes), "d2h_bytes_per_step": int(B.nbytes)}
    e2e_ok = all(s["status"] == 0 and s["true_rel_res"] <= TOL for s in st_e2e)

    # the same step with the matrix-free stencil as the inner operator (gdmr_system_set_stencil)
    matrix_free = None
    if not args.stencil:
        sysm.set_stencil(shape, *problems.helmholtz_stencil(shape, KAPPA, DAMPING))
        torch.cuda.synchronize()
        ev0.record()
        st_mf = step()
        ev1.record()
        torch.cuda.synchronize()
        mf_ms = max_over_ranks(ev0.elapsed_time(ev1), world)
        sysm.clear_stencil()
        matrix_free = {"value": world * nrhs / (mf_ms / 1e3), "unit": "solves/s", "steps": 1,
                       "verified": all(x["status"] == 0 and x["true_rel_res"] <= TOL for x in st_mf),
                       "operator": "matrix-free 7-point stencil (k_stencil); FP64 residual on the CSR operator"}

    # plain forms, one right-hand side at a time (reference algorithm): native complex128
    # (the drop-in) and fp64e (the same iteration in double-float arithmetic on the FP32 pipes)
    def plain_form(precision, max_cycles):
        sysp = gdmr.System(A, m_basis, K, capacity=1, precision=precision, device=local)
        cyc, ok = [], True
        torch.cuda.synchronize()
        t = time.perf_counter()
        for i in range(args.plain_sample):
            x, st = sysp.solve(B[i], mode=0 if i == 0 else 1, tol=TOL, mat_rank=max_cycles)
            cyc.append(st["cycles"])
            ok &= st["status"] == 0 and st["true_rel_res"] <= 2 * TOL
        el = time.perf_counter() - t
        out = {"value": args.plain_sample / el, "unit": "solves/s", "cycles": cyc,
               "latency_ms_each": el / args.plain_sample * 1e3, "verified": bool(ok),
               "sample": f"{args.plain_sample} right-hand sides solved in sequence (recycled deflation space)"}
        # kernel classes of the plain form: 10 more cycles with library-side CUDA events
        gdmr.profile_reset()
        gdmr.profile(True)
        sysp.solve(B[0], mode=1, tol=TOL, mat_rank=9)
        gdmr.profile(False)
        out["classes"] = class_table(gdmr.profile_read(), hbm_peak)
        sysp.close()
        return out

    plain = plain_form("fp64", args.max_cycles)
    plain_e = plain_form("fp64e", args.max_cycles)

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64-inner/f64-refine", "data": "synthetic",
        "config": workload_config(A, nrhs, shape, m_basis),
        "operator": "stencil" if args.stencil else "csr", "operator_kernel": op_kernel,
        "host_worst_true_rel_res": host_worst, "host_check": host_check,
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "cycles": {"mean": float(np.mean(cycles)), "max": int(np.max(cycles))},
        "verified": bool(verified), "worst_true_rel_res": worst_res,
        "plain_fp64": plain, "mixed_over_plain": value / world / plain["value"],
        "plain_fp64e": plain_e, "mixed_over_plain_fp64e": value / world / plain_e["value"],
        "e2e": e2e, "e2e_verified": bool(e2e_ok), "matrix_free": matrix_free,
        "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline,
        "tuning": gdmr.tune_report().strip().splitlines(),
    }
    if rank == 0 and args.cpu_cycles > 0:
        line["cpu_baseline"] = cpu_baseline(A, B[0], args.cpu_cycles, int(plain["cycles"][0]),
                                            problems.shard_seeds(nrhs, rank)[0])
    if rank == 0:
        print(json.dumps(line), flush=True)


def host_residuals(A, B, X):
    """max over right-hand sides of ||b - A x|| / ||b||, in FP64 on the host (SciPy CSR)."""
    S = A.to_scipy()
    rel = [float(np.linalg.norm(b - S @ x) / np.linalg.norm(b)) for b, x in zip(B, X)]
    return max(rel), {"how": "SciPy CSR FP64 product on the host, every right-hand side of the last timed step",
                      "count": len(rel), "median": float(np.median(rel))}


def plain_form_only(args, A, B, m_basis, device, hbm_peak):
    """--plain: the plain-form sample of bench's main line, alone (profiling captures)."""
    import gdmr
    s = gdmr.System(A, m_basis, K, capacity=1, precision=args.plain, device=device)
    cyc = []
    t = time.perf_counter()
    for i in range(args.plain_sample):
        x, st = s.solve(B[i], mode=0 if i == 0 else 1, tol=TOL, mat_rank=args.max_cycles)
        cyc.append(st["cycles"])
    el = time.perf_counter() - t
    s.close()
    return {"mode": "plain", "precision": args.plain, "value": args.plain_sample / el, "unit": "solves/s",
            "cycles": cyc, "tuning": gdmr.tune_report().strip().splitlines()}


def _solve_host(sysm, Bh_np, Xh_np, max_cycles):
    """gdmr_solve_batch on host buffers (on_device = 0): the copies run inside the call."""
    import ctypes
    import gdmr
    nrhs = Bh_np.shape[0]
    tols = np.full(nrhs, TOL)
    stats = (gdmr.Stats * nrhs)()
    rc = sysm.L.gdmr_solve_batch(sysm._h, nrhs, Bh_np.ctypes.data_as(ctypes.c_void_p),
                                 Xh_np.ctypes.data_as(ctypes.c_void_p), tols.ctypes.data_as(ctypes.c_void_p),
                                 int(max_cycles), 0, stats)
    if rc not in (0, 3, 4):
        raise RuntimeError(gdmr.last_error())
    return Xh_np, [s.as_dict() for s in stats]


if __name__ == "__main__":
    main()
