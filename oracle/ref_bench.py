"""Timed runs of the UNMODIFIED reference solvers on the benchmark workload.

COMPARISON INFRASTRUCTURE ONLY: bench.py's reference arm (the reference CPU
solver on every host core) and its reference-GPU leg (the reference GPU
solver, src/pcg3d_gpu.cu compiled for sm_103a, on the same model) run
through here. Models are built by the reference's own stack3d.h functions
(oracle/ref_harness.cpp); nothing here loads this repository's library.

The workload is the 800 x 800 x 10 two-tier stack of default_model
(src/stack3d.h:153-168): 25 W uniform in each Si tier plus a 3 W, 1 x 1 mm
hotspot in the bottom tier whose centre is drawn from a seeded generator
(numpy default_rng(seed), uniform in [0.5, 9.5] mm on each axis).

    python -m oracle.ref_bench gpu --n 800 --seed 2 --steps 5 --warmup 3 \
        [--mg-double] [--out T.npy]
prints one JSON line (solves/s, iterations, set-up time) and writes T.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import threading
import time

import numpy as np

if __package__ in (None, ""):
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    __package__ = "oracle"

from . import ref  # noqa: E402


def hotspot_power(seed: int):
    """The workload's power operations, in the order they are applied."""
    xc, yc = np.random.default_rng(seed).uniform(0.5e-3, 9.5e-3, size=2)
    return [("uniform", 0, 0.0, 0.0, 0.0, 0.0, 25.0),
            ("hotspot", 0, float(xc), float(yc), 1e-3, 0.0, 3.0),
            ("uniform", 2, 0.0, 0.0, 0.0, 0.0, 25.0)]


def known_answer_power():
    """hotspot_model (src/main3d.cu:60-67): 22 W uniform + 3 W in a 1 mm
    hotspot at (3, 3) mm in the bottom tier, 25 W in the top tier."""
    return [("uniform", 0, 0.0, 0.0, 0.0, 0.0, 22.0),
            ("hotspot", 0, 3e-3, 3e-3, 1e-3, 0.0, 3.0),
            ("uniform", 2, 0.0, 0.0, 0.0, 0.0, 25.0)]


def cpu_rate(n: int, seed: int, threads: int, tol: float, maxit: int, mg_double: bool = False,
             solves_per_thread: int = 1, model=None, solvers=None):
    """Steady solves/s of the reference CPU solver (CpuPcg, one per thread,
    each solving the shared model from T = 0) on `threads` host threads.
    Returns (rate, seconds, iterations, model, solvers); pass model and
    solvers back in to time again without their set-up."""
    L = ref.lib(mg_double)
    if model is None:
        model = ref.default_model(n, n, hotspot_power(seed), mg_double)
    if solvers is None:
        solvers = [None] * threads

        def make(k):
            solvers[k] = L.ref_cpu_solver_new(model.handle, 1)

        th = [threading.Thread(target=make, args=(k,)) for k in range(threads)]
        for t in th:
            t.start()
        for t in th:
            t.join()
    go = threading.Barrier(threads + 1)
    iters = [0] * threads

    def work(k):
        import ctypes as C
        it, rel = C.c_int(0), C.c_double(0.0)
        go.wait()
        for _ in range(solves_per_thread):
            L.ref_cpu_solver_steady(solvers[k], tol, maxit, C.byref(it), C.byref(rel))
        iters[k] = it.value

    th = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    for t in th:
        t.start()
    go.wait()
    t0 = time.perf_counter()
    for t in th:
        t.join()
    sec = time.perf_counter() - t0
    return threads * solves_per_thread / sec, sec, iters[0], model, solvers


def free_cpu_solvers(solvers, mg_double: bool = False) -> None:
    L = ref.lib(mg_double)
    for s in solvers:
        if s:
            L.ref_cpu_solver_free(s)


def gpu_run(n: int, seed: int, steps: int, warmup: int, tol: float, maxit: int,
            mg_double: bool, out: str | None, graphs: bool = True) -> dict:
    """The reference GPU solver (GpuPcg, multigrid) on the workload: set-up
    time, then `steps` steady solves from T = 0 timed on the host clock (the
    reference's solve blocks until it has converged)."""
    import ctypes as C
    L = ref.gpu_lib(mg_double)
    if L.refg_device_count() < 1:
        return {"unavailable": "no CUDA device"}
    L.refg_use_graphs(1 if graphs else 0)
    m = ref.default_model(n, n, hotspot_power(seed), mg_double, gpu=True)
    setup = C.c_double(0.0)
    s = L.refg_solver_new(m.handle, 1, C.byref(setup))
    it, rel = C.c_int(0), C.c_double(0.0)
    for _ in range(warmup):
        L.refg_solve_steady(s, tol, maxit, C.byref(it), C.byref(rel))
    t0 = time.perf_counter()
    conv = True
    for _ in range(steps):
        conv = L.refg_solve_steady(s, tol, maxit, C.byref(it), C.byref(rel)) == 1 and conv
    sec = time.perf_counter() - t0
    T = np.empty(n * n * m.nz)
    L.refg_get_x(s, T.ctypes.data)
    L.refg_solver_free(s)
    true = L.ref_true_relres(m.handle, T.ctypes.data)
    if out:
        np.save(out, T)
    return {"value": steps / sec, "unit": "solves/s", "ms_per_solve": 1e3 * sec / steps,
            "iters": it.value, "relres": rel.value, "converged": conv, "true_relres": true,
            "setup_ms": setup.value, "solves": steps,
            "build": "-DMG_DOUBLE (FP64 V-cycle)" if mg_double else "default (float V-cycle)",
            "graphs": graphs}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["gpu"])
    ap.add_argument("--n", type=int, default=800)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--maxit", type=int, default=1000)
    ap.add_argument("--mg-double", action="store_true")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    res = gpu_run(a.n, a.seed, a.steps, a.warmup, a.tol, a.maxit, a.mg_double, a.out)
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
