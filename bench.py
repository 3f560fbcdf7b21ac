"""Benchmark: steady MG-PCG solves per second on the 800 x 800 x 10 stack.

Workload (a "step"): one steady solve from T = 0 to ||r|| / ||P|| < 1e-10 of
the 800 x 800 x 10 two-tier stack (the reference's default_stack: 25 W per Si
tier + a seeded 3 W, 1 mm hotspot in the bottom tier), FP32 V-cycle inside a
flexible PCG whose outer iteration - residual and iterate updates, dot
products, alpha and beta - is FP64 (CT_MG_FP32_FLEX), with the operator and
multigrid hierarchy resident in HBM (built once, outside the timed region, as
in a power-map sweep). Inputs are larger than L2 (the fine level alone moves
> 1 GB per iteration), so no L2 flush is needed between steps.

Reported beside it, on the same GPU and the same model: the plain FP64
MG-PCG (FP64 V-cycle); the same FP32 V-cycle with the outer iteration in
double-word arithmetic on the FP32 pipes (CT_MG_FP32_FLEX_DW); the
reference's own GPU solver (src/pcg3d_gpu.cu, compiled for sm_103a from an
unmodified copy, in its default and -DMG_DOUBLE builds; a child process);
max|dT| and the FP64 true residual of each; the end-to-end rate through the
C ABI with the power map copied in and the temperatures copied out every
step; the per-kernel roofline; the 1024 x 1024 x 16 four-tier stack; the
batched 256-instance floorplan sweep; the 800 x 800 and batched 64 x 256 x
256 backward-Euler runs; and the reference CPU solver on the host cores.

--impl reference times the UNMODIFIED reference CPU solver (src/pcg3d_cpu.cpp,
default build, model built by the reference's own stack3d.h functions) on
every host core, one steady solve of the same workload per core and step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cuda-thermal_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "steady solves/s + % HBM roofline: FP32-MG & batched vs FP64 MG-PCG, <=5e-4 K"
N_GRID = 800
TOL = 1e-10
MAXIT = 1000
SEED = 2
BATCH_N = 256   # instances of the batched floorplan sweep
BATCH_SEED = 4
TR_N, TR_GRID, TR_SEED = 64, 256, 5   # batched transient: instances, lateral size, seed
TR_DT0, TR_GROWTH, TR_DT_MAX, TR_TOL = 1e-5, 1.1, 0.05, 1e-9
TR_CHECK = 4   # instances re-run with the plain FP64 solver for max|dT| and its rate
FALLBACK_HBM_GBS = 6800.0
# the workload as both arms name it
WORKLOAD = (f"steady solve {N_GRID}x{N_GRID}x10 two-tier stack (default_stack), 25 W per Si tier "
            f"+ 3 W 1 mm hotspot at a seeded position (seed {SEED}), tol {TOL:g}, from T = 0")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the timed region starts once the sampler is producing samples
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0:
            try:
                if os.path.getsize(self.file.name) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.02)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for k, name in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    """One process per GPU (RANK / LOCAL_RANK / WORLD_SIZE from the launcher):
    NCCL between GPU ranks, gloo when there is no GPU (the host-side logic
    of the multi-rank path is tested that way)."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if torch.cuda.is_available():
        torch.cuda.set_device(local if world > 1 else 0)
    if world > 1:
        import torch.distributed as td
        td.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as td
        td.barrier()


def _reduce(v, world, op):
    """v reduced over the ranks (a plain float; on the GPU under NCCL)."""
    if world == 1:
        return v
    import torch
    import torch.distributed as td
    dev = "cuda" if td.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    td.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(v, world):
    import torch.distributed as td
    return _reduce(v, world, td.ReduceOp.MAX)


def sum_over_ranks(v, world):
    import torch.distributed as td
    return _reduce(v, world, td.ReduceOp.SUM)


def partition_instances(costs, world):
    """A cost-balanced share of the batched instances for each rank: the
    largest remaining instance goes to the rank with the least cost so far
    (longest-processing-time first). Instances are independent, so ranks
    exchange nothing but their timing. Returns one sorted index list per
    rank; every instance is in exactly one."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def timed_solves(ct, solver, k, world):
    """k steady solves, timed with CUDA events on the solver's stream. The
    solves are queued one after another (ct_solve_async) and waited for once
    (ct_solve_wait), as a power-map sweep would run them, so the device time
    does not include host pauses between solves (a driver call held up by the
    clock sampler's nvidia-smi queries once stalled a blocking loop by about
    0.1 s)."""
    import torch
    stream = torch.cuda.ExternalStream(solver.stream())
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(k):
        solver.set_x_zero()
        solver.set_rhs_steady()
        solver.solve_async(TOL, MAXIT)
    e1.record(stream)
    st = solver.solve_wait()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    return ms, [st]


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class RefCpu:
    """The reference CPU solver on `threads` host threads, one CpuPcg per
    thread solving the workload's model from T = 0 (the unmodified reference,
    kind "reference", when its sources are staged and its build succeeds;
    otherwise the C oracle, a restatement of the same arithmetic, kind
    "port"). Set-up (model, levels, factors) happens once, outside timing."""

    def __init__(self, threads):
        self.threads = threads
        self.kind = "port"
        self.why = ""
        self.model = self.solvers = None
        try:
            from oracle import ref
            if ref.available() or ref.stage():
                ref.build()
                self.kind = "reference"
        except Exception as e:  # noqa: BLE001 - reported in the JSON line
            self.why = f"reference build unavailable ({e}); C oracle port timed instead"
        if self.kind == "port":
            import oracle
            import workloads
            oracle.build()
            m = workloads.steady_hotspot(N_GRID, seed=SEED)
            self.port = [oracle.Solver(m, "multigrid", mg_double=False) for _ in range(threads)]

    def step(self):
        """One timed step: every thread solves once. (solves/s, seconds, iterations)"""
        if self.kind == "reference":
            from oracle import ref_bench
            rate, sec, it, self.model, self.solvers = ref_bench.cpu_rate(
                N_GRID, SEED, self.threads, TOL, MAXIT, model=self.model, solvers=self.solvers)
            return rate, sec, it
        go = threading.Barrier(self.threads + 1)
        iters = [0] * self.threads

        def work(k):
            s = self.port[k]
            go.wait()
            s.set_x_zero()
            s.set_rhs_steady()
            iters[k] = s.solve(TOL, MAXIT)[0]

        th = [threading.Thread(target=work, args=(k,)) for k in range(self.threads)]
        for t in th:
            t.start()
        go.wait()
        t0 = time.perf_counter()
        for t in th:
            t.join()
        sec = time.perf_counter() - t0
        return self.threads / sec, sec, iters[0]

    def close(self):
        if self.kind == "reference" and self.solvers:
            from oracle import ref_bench
            ref_bench.free_cpu_solvers(self.solvers)
            self.solvers = None

    def describe(self, sec, it, steps):
        what = ("unmodified reference src/pcg3d_cpu.cpp (default build: float V-cycle, FP64 PCG), "
                "model from the reference's stack3d.h" if self.kind == "reference" else
                "C oracle port of src/pcg3d_cpu.cpp (float V-cycle)")
        d = (f"{self.threads} threads x {steps} step(s) x 1 steady {N_GRID}x{N_GRID}x10 solve each "
             f"({sec:.1f} s, {it} iterations); {what}")
        return d + (f"; {self.why}" if self.why else "")


def run_reference(args):
    """Reference arm: the unmodified reference CPU solver (CpuPcg of
    src/pcg3d_cpu.cpp, default build) on every host core, each core solving
    its own copy of the workload once per step. Nothing of this library is
    loaded. Under torchrun only rank 0 runs."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = host_threads()
    rc = RefCpu(threads)
    for _ in range(args.warmup):
        rc.step()
    secs, it = [], 0
    for _ in range(args.steps):
        _, sec, it = rc.step()
        secs.append(sec)
    rc.close()
    total = sum(secs)
    value = threads * args.steps / total
    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32",
        "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "cells": N_GRID * N_GRID * 10,
                   "precision": "reference default build (float V-cycle in FP64 PCG)",
                   "iters": it, "cpu_threads": threads},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": rc.kind,
                         "sample": rc.describe(total, it, args.steps)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def reference_gpu(np, T, steps, warmup):
    """The reference's own GPU solver (src/pcg3d_gpu.cu for sm_103a, from an
    unmodified copy; default and -DMG_DOUBLE builds) on the same model, in a
    child process: solves/s, iterations, set-up, and max|dT| against this
    library's solves T[name]."""
    try:
        from oracle import ref
        if not (ref.available() or ref.stage()):
            return {"unavailable": "reference sources not staged"}
        ref.build(gpu=True)
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"reference GPU build failed: {e}"}
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, flag in (("default", []), ("mg_double", ["--mg-double"])):
            f = os.path.join(td, f"T_{name}.npy")
            cmd = [sys.executable, "-m", "oracle.ref_bench", "gpu", "--n", str(N_GRID), "--seed",
                   str(SEED), "--steps", str(steps), "--warmup", str(warmup), "--tol", str(TOL),
                   "--maxit", str(MAXIT), "--out", f] + flag
            try:
                r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
                res = json.loads(r.stdout.strip().splitlines()[-1])
            except Exception as e:  # noqa: BLE001
                out[name] = {"unavailable": f"reference GPU run failed: {e}"}
                continue
            if os.path.exists(f):
                Tr = np.load(f)
                for k, v in T.items():
                    res[f"max_dT_K_vs_{k}"] = float(np.abs(Tr - v).max())
            out[name] = res
    return out


def traffic_from_profiles(kernel_name):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/*.md), when one lists it."""
    pdir = os.path.join(ROOT, "profiles")
    if not os.path.isdir(pdir):
        return None
    for f in sorted(os.listdir(pdir)):
        if not f.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(pdir, f)):
            if line.startswith("traffic_per_launch") and kernel_name in line:
                try:
                    return float(line.split("=")[1].split()[0])
                except Exception:
                    pass
    return None


def bench_batched(ct, np, torch, args, hbm_peak, peak_kind, rank=0, world=1):
    """The batched form on the 256-instance floorplan sweep: uneven stacks
    (nx, ny in 64..512, 6-16 planes), all solved to 1e-10 together with the
    FP32 V-cycle in FP64 flexible PCG (and, beside it, with the outer
    iteration in double words), against the plain FP64 MG-PCG solving the
    same instances one after another. With
    several ranks each solves a cost-balanced share (cells per instance; the
    iteration counts hardly vary) and the rate is all instances over the
    slowest rank's time."""
    import workloads
    specs_all = workloads.batch_instance_specs(BATCH_N, seed=BATCH_SEED)
    costs = [nx * ny * sum(l.ncells for l in cs.layers) for cs, nx, ny in specs_all]
    mine = partition_instances(costs, world)[rank]
    specs = [specs_all[i] for i in mine]
    kb = max(3, args.steps // 3)

    def make(prec):
        # every instance's model is built on the device from its description
        return ct.GpuBatch.from_specs([q[0] for q in specs], [q[1] for q in specs], [q[2] for q in specs],
                                      False, precision=prec)

    def timed(bt):
        for _ in range(args.warmup):
            bt.set_x_zero()
            bt.set_rhs_steady()
            bt.solve(TOL, MAXIT)
        stream = torch.cuda.ExternalStream(bt.stream())
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(kb):
            bt.set_x_zero()
            bt.set_rhs_steady()
            stats = bt.solve(TOL, MAXIT)
        e1.record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / kb, world), stats

    # the same instances with the outer iteration in double words
    bdw = make(ct.Precision.MG_FP32_FLEX_DW)
    ms_dw, st_dw = timed(bdw)
    Tdw = [bdw.get_x(i) for i in range(len(specs))]
    bdw.close()
    t0 = time.perf_counter()
    b = make(ct.Precision.MG_FP32_FLEX)
    models = b.models
    cells = sum(m.ncells() for m in models)
    setup_s = time.perf_counter() - t0
    ms, st = timed(b)
    iters = [s.iters for s in st]
    conv = sum(1 for s in st if s.converged)
    Tb = [b.get_x(i) for i in range(len(models))]
    true_max = max(b.true_relres(i) for i in range(len(models)))
    # per-kernel profile of one batched solve (direct launches, buckets in turn)
    b.set_x_zero()
    b.set_rhs_steady()
    _, rows = b.profile_solve(TOL, MAXIT)
    rows.sort(key=lambda r: -r["total_ms"])
    top = rows[0]
    achieved = top["bytes"] / (top["total_ms"] / 1e3) / 1e9
    buckets = b.buckets()
    b.close()
    # the same instances, one FP64 MG-PCG solve each, back to back
    ms64 = 0.0
    it64 = []
    max_dT = 0.0
    for i, (cs, nx, ny) in enumerate(specs):
        with ct.GpuPcg.from_spec(cs, nx, ny, False, ct.Precond.Multigrid, ct.Precision.MG_FP64) as s:
            s.set_x_zero()
            s.set_rhs_steady()
            s.solve(TOL, MAXIT)
            ev = torch.cuda.ExternalStream(s.stream())
            torch.cuda.synchronize()
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a0.record(ev)
            s.set_x_zero()
            s.set_rhs_steady()
            r = s.solve(TOL, MAXIT)
            a1.record(ev)
            torch.cuda.synchronize()
            ms64 += a0.elapsed_time(a1)
            it64.append(r.iters)
            max_dT = max(max_dT, float(np.abs(s.get_x() - Tb[i]).max()))
    ms64 = max_over_ranks(ms64, world)
    max_dT = max_over_ranks(max_dT, world)
    max_dT_dw = max_over_ranks(max(float(np.abs(a - c).max()) for a, c in zip(Tdw, Tb)), world)
    value = len(specs_all) / (ms / 1e3)
    value64 = len(specs_all) / (ms64 / 1e3)
    return {
        "value": value, "unit": "instance solves/s", "precision": "CT_MG_FP32_FLEX",
        "workload": f"{len(specs_all)} seeded stacks, nx, ny in 64..512 step 32, 6-16 planes, "
                    f"12 log-normal floorplan blocks per tier, tol {TOL:g} per instance",
        "instances": len(specs_all), "instances_rank0": len(models), "cells_rank0": cells,
        "ms_per_batch_solve": ms, "batch_solves": kb,
        "iters_min": min(iters), "iters_max": max(iters), "converged": conv,
        "true_relres_max": true_max, "max_dT_K_vs_fp64": max_dT,
        "fp64_mg_pcg_sequential": {"value": value64, "unit": "instance solves/s",
                                   "ms_total": ms64, "iters_max": max(it64)},
        "speedup_vs_fp64": value / value64,
        "double_word": {"value": len(specs_all) / (ms_dw / 1e3), "unit": "instance solves/s",
                        "precision": "CT_MG_FP32_FLEX_DW", "ms_per_batch_solve": ms_dw,
                        "iters_max": max(s.iters for s in st_dw), "max_dT_K_vs_flex": max_dT_dw},
        "setup_s": setup_s,
        "setup": "models described on the host, built on the device (ct_batch_create_cases)",
        "sharding": f"{world} rank(s), cost-balanced by cells, no collective",
        "buckets": [{"instances": k["instances"], "depth": k["depth"], "staged": k["staged"],
                     "sweep_tiles": k["sweep_tiles"]} for k in buckets],
        "roofline": {"bound": "hbm", "kernel": top["name"], "achieved": achieved,
                     "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "peak_kind": peak_kind, "share": top["total_ms"] / sum(r["total_ms"] for r in rows)},
        "kernels": [{"name": r["name"], "launches": r["launches"], "ms": round(r["total_ms"], 3),
                     "GBs": round(r["bytes"] / (r["total_ms"] / 1e3) / 1e9, 1)} for r in rows[:8]],
        "gpu_launches_per_batch_solve": sum(r["launches"] for r in rows),
    }


def bench_four_tier(ct, np, torch, args):
    """The 1024 x 1024 x 16 four-tier stack (TSV blocks, log-normal
    floorplans, 80 W): FLEX (the value), DW and plain FP64 steady solves/s
    on the same GPU, max|dT| against FP64, FP64 true residuals."""
    import workloads
    m = workloads.four_tier(1024, seed=3)
    out = {"workload": "steady solve 1024x1024x16 four-tier stack (Si/bond x4, TIM, Cu), 2 % Cu "
                       "TSV 8x8 blocks in bond layers, 12 log-normal blocks per tier, 20 W per tier, "
                       f"tol {TOL:g}", "cells": m.ncells()}
    T = {}
    for key, prec in (("dw", ct.Precision.MG_FP32_FLEX_DW), ("flex", ct.Precision.MG_FP32_FLEX),
                      ("fp64", ct.Precision.MG_FP64)):
        s = ct.GpuPcg(m, ct.Precond.Multigrid, prec)
        for _ in range(2):
            s.set_x_zero()
            s.set_rhs_steady()
            s.solve(TOL, MAXIT)
        k = 3
        ms, st = timed_solves(ct, s, k, 1)
        T[key] = s.get_x()
        out[key] = {"value": k / (ms / 1e3), "unit": "solves/s", "iters": st[-1].iters,
                    "ms_per_solve": ms / k, "true_relres": s.true_relres()}
        s.close()
    out["value"] = out["flex"]["value"]
    out["unit"] = "solves/s"
    out["precision"] = "CT_MG_FP32_FLEX"
    out["speedup_vs_fp64"] = out["flex"]["value"] / out["fp64"]["value"]
    out["dw_speedup_vs_fp64"] = out["dw"]["value"] / out["fp64"]["value"]
    out["max_dT_K"] = float(np.abs(T["flex"] - T["fp64"]).max())
    out["max_dT_K_dw"] = float(np.abs(T["dw"] - T["fp64"]).max())
    return out


def bench_transient_batched(ct, np, args, steps):
    """The batched transient (FP32 V-cycle in FP64 flexible PCG; the
    double-word form beside it): 64 instances of the 256 x 256 x 10 stack, each
    with 9 blocks switching at Poisson times (mean 5 ms), backward-Euler steps
    with per-instance dt (10 us growing 10 % per step, capped at 50 ms, reset
    to 10 us on a switch), warm-started from the steady field of the initial
    power, tol 1e-9 per step. Timed end to end on the host clock: switching
    (power maps uploaded), set_dt, b = P + C/dt T, the batched solve and the
    batched step records of every step."""
    import workloads

    def run(prec):
        ws = workloads.switching_instances(TR_N, TR_GRID, seed=TR_SEED)
        n = len(ws)
        b = ct.GpuBatch([w.model for w in ws], precision=prec)
        for i, w in enumerate(ws):
            b.set_power(i, w.power())
        b.set_x_zero()
        b.set_rhs_steady()
        b.solve(TOL, MAXIT)
        dt = np.full(n, TR_DT0)
        t = np.zeros(n)
        ptot = np.array([w.power().sum() for w in ws])
        eb, its, switches = [], [], 0
        dts, eb_inst = [], []
        t0 = time.perf_counter()
        for k in range(steps):
            for i, w in enumerate(ws):
                if w.advance(t[i]):
                    P = w.power()
                    b.set_power(i, P)
                    ptot[i] = P.sum()
                    dt[i] = TR_DT0
                    switches += 1
            st = b.step_transient(dt, TR_TOL, MAXIT)
            rec = b.step_records(dt)
            on = ptot > 0
            ebk = np.where(on, np.abs(rec[:, 1] + rec[:, 2] - ptot) / np.where(on, ptot, 1.0), np.nan)
            eb_inst.append(ebk[:TR_CHECK].copy())
            if on.any():
                eb.append(float(np.nanmax(ebk)))
            its.append(max(s.iters for s in st))
            dts.append(dt.copy())
            t += dt
            dt = np.minimum(dt * TR_GROWTH, TR_DT_MAX)
        sec = time.perf_counter() - t0
        Tb = [b.get_x(i) for i in range(TR_CHECK)]
        b.close()
        return n, sec, eb, its, switches, dts, eb_inst, Tb

    n, sec_dw, eb_dw, _, _, _, _, Tb_dw = run(ct.Precision.MG_FP32_FLEX_DW)
    n, sec, eb, its, switches, dts, eb_inst, Tb = run(ct.Precision.MG_FP32_FLEX)
    # the same steps for the first instances with the plain FP64 MG-PCG, one by one
    ref = workloads.switching_instances(TR_CHECK, TR_GRID, seed=TR_SEED)
    sec64, max_dT = 0.0, 0.0
    eb64, eb_same = [], []  # the FP64 solver's balance per step; the batch's on the same instances
    for i, w in enumerate(ref):
        s = ct.GpuPcg(w.model, ct.Precond.Multigrid, ct.Precision.MG_FP64)
        s.set_power(w.power())
        s.set_x_zero()
        s.set_rhs_steady()
        s.solve(TOL, MAXIT)
        tt = 0.0
        sec_i = 0.0  # this instance's solving time
        pt = float(w.power().sum())
        for k in range(steps):
            a0 = time.perf_counter()
            if w.advance(tt):
                P = w.power()
                s.set_power(P)
                pt = float(P.sum())
            s.set_dt(float(dts[k][i]))
            s.set_rhs_transient()
            s.solve(TR_TOL, MAXIT)
            sec_i += time.perf_counter() - a0
            if pt > 0:  # bookkeeping outside the timed part
                r = s.step_record(float(dts[k][i]))
                eb64.append(abs(r.q_out + r.q_stored - pt) / pt)
                eb_same.append(eb_inst[k][i])
            tt += float(dts[k][i])
        sec64 += sec_i
        max_dT = max(max_dT, float(np.abs(s.get_x() - Tb[i]).max()))
        s.close()
    value = n * steps / sec
    value64 = TR_CHECK * steps / sec64
    return {
        "value": value, "unit": "instance steps/s", "precision": "CT_MG_FP32_FLEX",
        "double_word": {"value": n * steps / sec_dw, "unit": "instance steps/s",
                        "precision": "CT_MG_FP32_FLEX_DW",
                        "energy_balance_err_max": max(eb_dw) if eb_dw else None,
                        "max_dT_K_vs_flex": max(float(np.abs(a - c).max()) for a, c in zip(Tb_dw, Tb))},
        "workload": f"{n} x {TR_GRID}x{TR_GRID}x10 default stack, 9 blocks per instance toggled at "
                    f"Poisson times (mean 5 ms), {steps} backward-Euler steps, per-instance dt "
                    f"{TR_DT0:g} s x {TR_GROWTH} per step (max {TR_DT_MAX:g}), reset on a switch, "
                    f"tol {TR_TOL:g}",
        "steps": steps, "batch_steps_per_s": steps / sec, "switches": switches,
        "iters_max_per_step_median": float(np.median(its)), "iters_max_per_step_max": int(max(its)),
        "energy_balance_err_max": max(eb) if eb else None,
        "energy_balance_err_median": float(np.median(eb)) if eb else None,
        "fp64_mg_pcg_sequential": {"value": value64, "unit": "instance steps/s",
                                   "instances": TR_CHECK,
                                   "energy_balance_err_max": max(eb64) if eb64 else None,
                                   "energy_balance_err_median": float(np.median(eb64)) if eb64 else None},
        "energy_balance_same_instances": {"batch_max": float(np.nanmax(eb_same)) if eb_same else None,
                                          "fp64_max": max(eb64) if eb64 else None,
                                          "note": "tol is relative to ||b|| = ||P + C/dt T_old||"},
        "speedup_vs_fp64": value / value64,
        "max_dT_K_vs_fp64": max_dT,
    }


def bench_transient_800(ct, np, solvers, m, steps):
    """The 800 x 800 x 10 stack's transient: backward-Euler steps from T = 0
    with the power on at t = 0 (run_transient, src/transient3d.h:48-90), dt
    10 us growing 10 % per step up to 50 ms, tol 1e-9, each step warm-started
    from the last; per step set_dt, b = P + C/dt T, the solve and the step
    record (T_max, heat out, heat stored reduced on the device), all queued
    on the solver's stream with one wait at the end. The FP32
    V-cycle in FP64 flexible PCG (and the double-word form) against the plain
    FP64 MG-PCG on the same steps; the solvers already hold the operator and
    hierarchy."""
    ptot = float(np.sum(m.P))
    res = {}
    for name, s in solvers.items():
        s.set_x_zero()
        dt, last = TR_DT0, -1.0
        # every step queued on the solver's stream (ct_solve_async and the
        # step record into the device table), one wait at the end
        t0 = time.perf_counter()
        for k in range(steps):
            if dt != last:
                s.set_dt(dt)
                last = dt
            s.set_rhs_transient()
            s.solve_async(TR_TOL, MAXIT)
            s.step_record_async(dt, k)
            dt = min(dt * TR_GROWTH, TR_DT_MAX)
        recs, sts = s.step_records(0, steps)
        sec = time.perf_counter() - t0
        its = sum(st.iters for st in sts)
        eb = max(abs(r.q_out + r.q_stored - ptot) / ptot for r in recs)
        assert all(st.converged for st in sts)
        res[name] = dict(sec=sec, iters=its, eb=eb, T=s.get_x(), T_max=recs[-1].T_max)
        s.set_dt(0.0)
    # the same FLEX steps with blocking calls (ct_solve, ct_solver_step_record)
    s = solvers["flex"]
    s.set_x_zero()
    dt, last, its_b = TR_DT0, -1.0, 0
    t0 = time.perf_counter()
    for k in range(steps):
        if dt != last:
            s.set_dt(dt)
            last = dt
        s.set_rhs_transient()
        its_b += s.solve(TR_TOL, MAXIT).iters
        s.step_record(dt)
        dt = min(dt * TR_GROWTH, TR_DT_MAX)
    sec_b = time.perf_counter() - t0
    same_b = bool(np.array_equal(s.get_x(), res["flex"]["T"])) and its_b == res["flex"]["iters"]
    s.set_dt(0.0)
    fx, f64 = res["flex"], res["fp64"]
    out = {
        "value": steps / fx["sec"], "unit": "steps/s", "precision": "CT_MG_FP32_FLEX",
        "workload": f"{N_GRID}x{N_GRID}x10 stack, {steps} backward-Euler steps from T = 0, dt "
                    f"{TR_DT0:g} s x {TR_GROWTH} per step (max {TR_DT_MAX:g}), tol {TR_TOL:g}, "
                    f"device step records",
        "steps": steps, "iters_total": fx["iters"], "energy_balance_err_max": fx["eb"],
        "T_max_end_K": fx["T_max"],
        "fp64_mg_pcg": {"value": steps / f64["sec"], "unit": "steps/s", "iters_total": f64["iters"],
                        "energy_balance_err_max": f64["eb"]},
        "speedup_vs_fp64": f64["sec"] / fx["sec"],
        "max_dT_K_vs_fp64": float(np.abs(fx["T"] - f64["T"]).max()),
        "blocking": {"value": steps / sec_b, "unit": "steps/s", "same_bits": same_b,
                     "calls": "ct_solve and ct_solver_step_record per step (the host waits twice a step)"},
    }
    if "dw" in res:
        dw = res["dw"]
        out["double_word"] = {"value": steps / dw["sec"], "unit": "steps/s", "iters_total": dw["iters"],
                              "energy_balance_err_max": dw["eb"],
                              "max_dT_K_vs_fp64": float(np.abs(dw["T"] - f64["T"]).max())}
    return out


def profile_rows(solver):
    """Per-kernel CUDA-event times of one solve launched kernel by kernel."""
    solver.set_x_zero()
    solver.set_rhs_steady()
    _, rows = solver.profile_solve(TOL, MAXIT)
    rows.sort(key=lambda r: -r["total_ms"])
    return rows


# FP64 instructions per cell of the FP64 outer kernels (CT_MG_FP32_FLEX;
# k_fp64.cu): 7 DFMA for (A + C/dt) p and 1 for p.Ap; r and ||r||^2 (x
# += alpha p runs beside the next V-cycle: pcg_update_x); r.z and z.Ap; p = z
# + beta p; ||b||^2 of a start from x = 0. Conversions are integer operations.
FP64_OPS = {"pcg_apply": 8, "pcg_update_xr": 2, "pcg_update_x": 1, "pcg_dot": 2, "pcg_update_p": 1,
            "pcg_residual": 1}


def kernel_table(rows, n=10, cells=None, dfma=None):
    out = []
    for r in rows[:n]:
        e = {"name": r["name"], "launches": r["launches"], "ms": round(r["total_ms"], 4),
             "GBs": round(r["bytes"] / (r["total_ms"] / 1e3) / 1e9, 1)}
        if cells and dfma and r["name"] in FP64_OPS:
            rate = FP64_OPS[r["name"]] * cells * r["launches"] / (r["total_ms"] / 1e3)
            e["fp64_ops_per_cell"] = FP64_OPS[r["name"]]
            e["fp64_frac"] = round(rate / dfma, 3)
        out.append(e)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 256-instance run")
    ap.add_argument("--no-four-tier", action="store_true", help="skip the 1024x1024x16 stack")
    ap.add_argument("--transient-steps", type=int, default=500,
                    help="backward-Euler steps of the batched transient (0: skip)")
    ap.add_argument("--transient-800-steps", type=int, default=300,
                    help="backward-Euler steps of the 800x800x10 transient (0: skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import cthermal as ct
    import workloads

    rank, world, local = dist_setup(args.gpus)
    ct.lib()
    hbm_peak, peak_kind = peaks()
    m = workloads.steady_hotspot(N_GRID, seed=SEED)
    ncells = m.ncells()

    sfx = ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX)
    sdw = ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX_DW)
    s64 = ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP64)
    for _ in range(args.warmup):
        for s in (sfx, sdw, s64):
            s.set_x_zero()
            s.set_rhs_steady()
            s.solve(TOL, MAXIT)

    # ---- headline: FP32 V-cycle in FP64 flexible PCG, device-resident -------
    clocks = ClockSampler(local)
    clocks.start()
    msfx, stfx = timed_solves(ct, sfx, args.steps, world)
    Tfx = sfx.get_x()
    truefx = sfx.true_relres()
    msfx = max_over_ranks(msfx, world)
    value = sum_over_ranks(args.steps, world) / (msfx / 1e3)

    # ---- the same with the outer iteration in double words (FP32 pipes) -----
    kdw = max(3, args.steps // 2)
    msdw, stdw = timed_solves(ct, sdw, kdw, world)
    Tdw = sdw.get_x()
    truedw = sdw.true_relres()
    msdw = max_over_ranks(msdw, world)
    valuedw = sum_over_ranks(kdw, world) / (msdw / 1e3)

    # ---- plain FP64 MG-PCG on the same GPU ---------------------------------
    k64 = max(3, args.steps // 2)
    ms64, st64 = timed_solves(ct, s64, k64, world)
    T64 = s64.get_x()
    true64 = s64.true_relres()
    ms64 = max_over_ranks(ms64, world)
    value64 = sum_over_ranks(k64, world) / (ms64 / 1e3)

    # ---- end to end through the C ABI: host P in, host T out -------------
    P_host = torch.empty(ncells, dtype=torch.float64, pin_memory=True)
    T_host = torch.empty(ncells, dtype=torch.float64, pin_memory=True)
    P_np, T_np = P_host.numpy(), T_host.numpy()
    P_np[:] = m.P
    stream = torch.cuda.ExternalStream(sfx.stream())
    # Each step through the public calls a power-map sweep makes: P copied in
    # from pinned host memory, x = 0, b = P, solve, T copied out to pinned
    # host memory. Queued (ct_set_power_async, ct_solve_async,
    # ct_get_x_async): the copy in of step k + 1 and the copy out of step k -
    # 1 run on copy streams while step k solves; the timed region ends after
    # the last copy out. One untimed step first warms the copy queues.
    def e2e_step():
        sfx.set_power_async(P_np)
        sfx.set_x_zero()
        sfx.set_rhs_steady()
        sfx.solve_async(TOL, MAXIT)
        sfx.get_x_async(T_np)

    e2e_step()
    sfx.solve_wait()
    sfx.copies_wait()
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    sfx.copies_wait()  # the solver's stream waits for the last copy out, then the host
    e1.record(stream)
    torch.cuda.synchronize()
    wall_e2e = time.perf_counter() - t0
    st_e2e = sfx.solve_wait()
    ms_e2e = max_over_ranks(e0.elapsed_time(e1), world)
    e2e_value = sum_over_ranks(args.steps, world) / (ms_e2e / 1e3)
    e2e_same_bits = bool(np.array_equal(T_np, Tfx)) and st_e2e.converged
    # the same steps with blocking calls (each step's copies and solve in
    # turn, the host waiting on each)
    T_np[:] = 0.0
    torch.cuda.synchronize()
    barrier(world)
    e0b, e1b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0b.record(stream)
    for _ in range(args.steps):
        sfx.set_power(P_np)
        sfx.set_x_zero()
        sfx.set_rhs_steady()
        sfx.solve(TOL, MAXIT)
        sfx.get_x(T_np)
    e1b.record(stream)
    torch.cuda.synchronize()
    ms_e2e_blocking = max_over_ranks(e0b.elapsed_time(e1b), world)
    e2e_blocking = sum_over_ranks(args.steps, world) / (ms_e2e_blocking / 1e3)
    e2e_same_bits = e2e_same_bits and bool(np.array_equal(T_np, Tfx))

    # ---- roofline: per-kernel CUDA-event times of one solve ------------------
    rows = profile_rows(sfx)
    dfma = ct.probe_fp64_rate()
    tot_ms = sum(r["total_ms"] for r in rows)
    top = rows[0]
    achieved = top["bytes"] / top["launches"] / (top["total_ms"] / top["launches"] / 1e3) / 1e9
    traffic = traffic_from_profiles(top["name"])
    alg_bytes_solve = sum(r["bytes"] for r in rows)
    # the profiled solve's launches, plus those a queued solve adds around its
    # graph: the control-block set and the no-heat check (ct_solve_async) and
    # the last iteration's x update after the loop
    launches_per_solve = sum(r["launches"] for r in rows) + 3
    rows_dw = profile_rows(sdw)

    batched = None
    if not args.no_batch:
        batched = bench_batched(ct, np, torch, args, hbm_peak, peak_kind, rank, world)
        # what separates the batched iteration's stages: a grid-wide barrier in
        # one persistent kernel against a dependent launch in a graph
        batched["stage_separation_probe"] = {
            "per_phase_us": [ct.probe_sync_costs(2000, bps) for bps in (1, 4, 8)],
            "note": "dependent phases over SMs x blocks/SM blocks of 256 threads: grid barrier in one "
                    "cooperative kernel vs one PDL launch per phase in a CUDA graph"}
    four = None
    if not args.no_four_tier:
        four = bench_four_tier(ct, np, torch, args)
    transient = None
    if args.transient_steps > 0:
        transient = bench_transient_batched(ct, np, args, args.transient_steps)
    transient800 = None
    if args.transient_800_steps > 0:
        transient800 = bench_transient_800(ct, np, {"flex": sfx, "dw": sdw, "fp64": s64}, m,
                                           args.transient_800_steps)
    # clocks sampled over every timed region above
    clk = clocks.stop()

    ref_gpu = None
    if rank == 0 and not args.no_reference_gpu:
        ref_gpu = reference_gpu(np, {"flex": Tfx, "fp64": T64}, max(3, args.steps // 2),
                                args.warmup)
        for k in ("default", "mg_double"):
            if isinstance(ref_gpu.get(k), dict) and ref_gpu[k].get("value"):
                ref_gpu[k]["flex_speedup"] = value / ref_gpu[k]["value"]

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rc = RefCpu(host_threads())
        rate, sec, it = rc.step()
        rc.close()
        cpu = {"value": rate, "unit": "solves/s", "cores": rc.threads, "kind": rc.kind,
               "sample": rc.describe(sec, it, 1)}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": msfx / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64+f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": ncells,
                       "precision": "CT_MG_FP32_FLEX",
                       "precision_note": "FP32 V-cycle in flexible PCG; FP64 residual and iterate "
                                         "updates, dot products, alpha, beta",
                       "levels": sfx.num_levels(), "iters": stfx[-1].iters,
                       "l2": "inputs larger than L2 (fine level ~1.7 GB moved per iteration)",
                       "parallelism": f"replicas x{world}"},
            "gpu_launches": launches_per_solve * args.steps,
            "kernels": kernel_table(rows, 16, ncells, dfma),
            "double_word_kernels": kernel_table(rows_dw, 6),
        }
        if batched:
            out["batched"] = batched
        if transient:
            out["batched_transient"] = transient
        if transient800:
            out["transient_800"] = transient800
        if four:
            out["four_tier"] = four
        out["e2e"] = {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": ncells * 8,
                      "d2h_bytes_per_step": ncells * 8, "wall_s": wall_e2e,
                      "same_bits_as_device_run": e2e_same_bits,
                      "calls": "ct_set_power_async, ct_set_x_zero, ct_set_rhs_steady, ct_solve_async, "
                               "ct_get_x_async per step; ct_copies_wait after the last",
                      "blocking": {"value": e2e_blocking, "unit": "solves/s",
                                   "calls": "ct_set_power, ct_set_x_zero, ct_set_rhs_steady, ct_solve, "
                                            "ct_get_x per step"}}
        out["roofline"] = {"bound": "hbm", "kernel": top["name"], "achieved": achieved,
                           "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                           "peak_kind": peak_kind, "traffic": traffic,
                           "alg_bytes_per_launch": top["bytes"] / top["launches"],
                           "launch_ms": top["total_ms"] / top["launches"],
                           "share": top["total_ms"] / tot_ms,
                           "solve_frac": alg_bytes_solve / (msfx / args.steps / 1e3) / 1e9 / hbm_peak}
        out["roofline"]["note"] = ("the dominant kernel, the FP64 operator apply, is bound by the FP64 pipe "
                                   "(8 DFMA a cell), not by HBM: fp64_pipe.frac; the smoother's HBM "
                                   "roofline is smoother.frac")
        sw = next((r for r in rows if r["name"] == "mg_sweep_l0"), None)
        if sw:
            sw_rate = sw["bytes"] / (sw["total_ms"] / 1e3) / 1e9
            out["roofline"]["smoother"] = {
                "kernel": "mg_sweep_l0", "bound": "hbm", "achieved": sw_rate, "peak": hbm_peak, "unit": "GB/s",
                "frac": sw_rate / hbm_peak, "peak_kind": peak_kind,
                "traffic": traffic_from_profiles("mg_sweep_l0"),
                "alg_bytes_per_launch": sw["bytes"] / sw["launches"],
                "launch_ms": sw["total_ms"] / sw["launches"],
                "timing": "CUDA events around each launch of a solve launched kernel by kernel (the "
                          "launch's own latency included)"}
        ap = next((r for r in rows if r["name"] == "pcg_apply"), None)
        if ap:
            rate = FP64_OPS["pcg_apply"] * ncells * ap["launches"] / (ap["total_ms"] / 1e3)
            out["roofline"]["fp64_pipe"] = {
                "kernel": "pcg_apply", "bound": "fp64", "achieved": rate, "peak": dfma,
                "unit": "DFMA/s", "frac": rate / dfma,
                "peak_kind": "measured (ct_probe_fp64_rate: independent DFMA chains on every SM)",
                "hbm_frac": ap["bytes"] / (ap["total_ms"] / 1e3) / 1e9 / hbm_peak}
        out["true_relres"] = truefx
        out["double_word"] = {"value": valuedw, "unit": "solves/s", "precision": "CT_MG_FP32_FLEX_DW",
                              "iters": stdw[-1].iters, "ms_per_solve": msdw / kdw,
                              "true_relres": truedw, "max_dT_K_vs_fp64": float(np.abs(Tdw - T64).max()),
                              "speedup_vs_fp64": valuedw / value64}
        out["fp64_mg_pcg"] = {"value": value64, "unit": "solves/s", "iters": st64[-1].iters,
                              "ms_per_solve": ms64 / k64, "true_relres": true64}
        out["max_dT_K"] = float(np.abs(Tfx - T64).max())
        out["speedup_vs_fp64"] = value / value64
        if ref_gpu is not None:
            out["reference_gpu"] = ref_gpu
        if cpu:
            out["cpu_baseline"] = cpu
        out["clocks"] = clk
        print(json.dumps(out), flush=True)
    sfx.close()
    sdw.close()
    s64.close()
    if world > 1:
        import torch.distributed as td
        td.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
