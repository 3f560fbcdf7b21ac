"""CPU oracle for the MG-PCG thermal solve (ctypes bindings to liboracle.so).

TEST INFRASTRUCTURE ONLY. Only the tests, ``__graft_entry__.smoke()`` and the
CPU baseline leg of ``bench.py`` import this package, to check results and
to time the CPU reference arithmetic. The product library never loads it.

``liboracle.so`` is a plain-C restatement of the reference CPU solver
(cuda-thermal ``src/pcg3d_cpu.cpp``, ``src/mg3d.h``, ``src/operator3d.h``,
``src/transient3d.h``); see ``oracle.h`` for the exact correspondence. A model
is any object with the finalized ``Model3D`` arrays as attributes: ``nx, ny,
nz, dx, dy`` and ``gE, gN, gU, gB, cap`` (float32) and ``P`` (float64), in the
natural layout (x fastest, then y, then z).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class OracleModelC(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double),
        ("gE", C.c_void_p), ("gN", C.c_void_p), ("gU", C.c_void_p),
        ("gB", C.c_void_p), ("cap", C.c_void_p), ("P", C.c_void_p),
    ]


def build(force: bool = False) -> str:
    """Compiles liboracle.so with the committed Makefile (gcc, no reference
    sources needed)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(LIB_PATH)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    mp = C.POINTER(OracleModelC)
    L.oracle_create.restype = vp
    L.oracle_create.argtypes = [mp, C.c_int, C.c_int, C.c_int]
    L.oracle_destroy.argtypes = [vp]
    L.oracle_set_dt.argtypes = [vp, C.c_double]
    L.oracle_set_x_zero.argtypes = [vp]
    L.oracle_set_x.argtypes = [vp, _f64p]
    L.oracle_set_rhs_steady.argtypes = [vp]
    L.oracle_set_rhs_transient.argtypes = [vp]
    L.oracle_set_power.argtypes = [vp, _f64p]
    L.oracle_solve.restype = C.c_int
    L.oracle_solve.argtypes = [vp, C.c_double, C.c_int, ip, dp]
    L.oracle_get_x.argtypes = [vp, _f64p]
    L.oracle_set_outer_df.argtypes = [vp, C.c_int]
    L.oracle_num_levels.restype = C.c_int
    L.oracle_num_levels.argtypes = [vp]
    L.oracle_level_dims.argtypes = [vp, C.c_int, ip, ip, ip]
    L.oracle_level_operator.argtypes = [vp, C.c_int, _f32p, _f32p, _f32p, _f32p, _f32p]
    L.oracle_level_factors.argtypes = [vp, C.c_int, _f64p, _f64p]
    L.oracle_true_relres.restype = C.c_double
    L.oracle_true_relres.argtypes = [mp, _f64p]
    L.oracle_heat_out.restype = C.c_double
    L.oracle_heat_out.argtypes = [mp, _f64p]
    L.oracle_heat_stored.restype = C.c_double
    L.oracle_heat_stored.argtypes = [mp, _f64p, _f64p, C.c_double]
    L.oracle_apply.argtypes = [mp, C.c_double, _f64p, _f64p]
    L.oracle_run_transient.restype = C.c_int
    L.oracle_run_transient.argtypes = [
        mp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
        C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_int, _f64p, C.POINTER(C.c_long), ip]
    _lib = L
    return L


class _ModelRef:
    """Keeps the arrays alive while the C struct points at them."""

    def __init__(self, m):
        self.arrays = [np.ascontiguousarray(getattr(m, k), dtype=np.float32)
                       for k in ("gE", "gN", "gU", "gB", "cap")]
        self.P = np.ascontiguousarray(m.P, dtype=np.float64)
        self.n = int(m.nx) * int(m.ny) * int(m.nz)
        gE, gN, gU, gB, cap = (a.ctypes.data for a in self.arrays)
        self.c = OracleModelC(int(m.nx), int(m.ny), int(m.nz), float(m.dx), float(m.dy),
                              gE, gN, gU, gB, cap, self.P.ctypes.data)

    def ref(self):
        return C.byref(self.c)


@dataclass
class SolveResult:
    T: np.ndarray
    iters: int
    relres: float
    converged: bool


class Solver:
    """CpuPcg (src/pcg3d.h:71-99) over the oracle. precond: "jacobi" or
    "multigrid"; mg_double selects the -DMG_DOUBLE arithmetic; flexible the
    flexible (Polak-Ribiere) beta."""

    def __init__(self, m, precond="multigrid", mg_double=True, flexible=False, outer_df=False):
        self._m = _ModelRef(m)
        self.n = self._m.n
        self._h = lib().oracle_create(self._m.ref(), 1 if precond == "multigrid" else 0,
                                      int(bool(mg_double)), int(bool(flexible)))
        if not self._h:
            raise ValueError("oracle_create rejected the model")
        if outer_df:
            lib().oracle_set_outer_df(self._h, 1)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle_destroy(h)
            self._h = None

    def set_dt(self, dt):
        lib().oracle_set_dt(self._h, float(dt))

    def set_x_zero(self):
        lib().oracle_set_x_zero(self._h)

    def set_x(self, x):
        lib().oracle_set_x(self._h, np.ascontiguousarray(x, dtype=np.float64).ravel())

    def set_rhs_steady(self):
        lib().oracle_set_rhs_steady(self._h)

    def set_rhs_transient(self):
        lib().oracle_set_rhs_transient(self._h)

    def set_power(self, P):
        lib().oracle_set_power(self._h, np.ascontiguousarray(P, dtype=np.float64).ravel())

    def solve(self, tol, maxit):
        it, rel = C.c_int(0), C.c_double(0)
        conv = lib().oracle_solve(self._h, float(tol), int(maxit), C.byref(it), C.byref(rel))
        return it.value, rel.value, bool(conv)

    def get_x(self):
        T = np.empty(self.n, dtype=np.float64)
        lib().oracle_get_x(self._h, T)
        return T

    def num_levels(self):
        return lib().oracle_num_levels(self._h)

    def level_dims(self, k):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        lib().oracle_level_dims(self._h, k, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def level_operator(self, k):
        nx, ny, nz = self.level_dims(k)
        n, nxy = nx * ny * nz, nx * ny
        out = [np.empty(n, np.float32) for _ in range(3)] + [np.empty(nxy, np.float32),
                                                             np.empty(n, np.float32)]
        lib().oracle_level_operator(self._h, k, *out)
        return dict(zip(("gE", "gN", "gU", "gB", "cap"), out))

    def level_factors(self, k):
        nx, ny, nz = self.level_dims(k)
        fcp, finv = np.empty(nx * ny * nz), np.empty(nx * ny * nz)
        lib().oracle_level_factors(self._h, k, fcp, finv)
        return fcp, finv


def solve_steady(m, tol=1e-10, maxit=50000, precond="multigrid", mg_double=True,
                 flexible=False, outer_df=False) -> SolveResult:
    """cpu_pcg (src/pcg3d_cpu.cpp:187-205): steady solve from T = 0."""
    s = Solver(m, precond, mg_double, flexible, outer_df)
    s.set_x_zero()
    s.set_rhs_steady()
    it, rel, conv = s.solve(tol, maxit)
    return SolveResult(s.get_x(), it, rel, conv)


def true_relres(m, T) -> float:
    r = _ModelRef(m)
    return lib().oracle_true_relres(r.ref(), np.ascontiguousarray(T, np.float64).ravel())


def heat_out(m, T) -> float:
    r = _ModelRef(m)
    return lib().oracle_heat_out(r.ref(), np.ascontiguousarray(T, np.float64).ravel())


def heat_stored(m, T_old, T_new, dt) -> float:
    r = _ModelRef(m)
    return lib().oracle_heat_stored(r.ref(), np.ascontiguousarray(T_old, np.float64).ravel(),
                                    np.ascontiguousarray(T_new, np.float64).ravel(), float(dt))


def apply(m, x, inv_dt=0.0) -> np.ndarray:
    r = _ModelRef(m)
    y = np.empty(r.n)
    lib().oracle_apply(r.ref(), float(inv_dt), np.ascontiguousarray(x, np.float64).ravel(), y)
    return y


@dataclass
class TransientResult:
    steps: np.ndarray  # (nsteps, 6): t, dt, iters, T_max, q_out, q_stored
    T: np.ndarray
    total_iters: int
    converged: bool


def run_transient(m, precond="multigrid", mg_double=True, flexible=False, dt0=1e-5,
                  growth=1.1, dt_max=0.05, t_end=1.0, nsteps=0, tol=1e-9,
                  maxit=50000, max_rec=100000) -> TransientResult:
    """run_transient (src/transient3d.h:48-90); nsteps > 0 runs a fixed number
    of steps instead of up to t_end."""
    r = _ModelRef(m)
    rec = np.zeros((max_rec, 6))
    T = np.empty(r.n)
    tot, allc = C.c_long(0), C.c_int(0)
    k = lib().oracle_run_transient(
        r.ref(), 1 if precond == "multigrid" else 0, int(bool(mg_double)), int(bool(flexible)),
        dt0, growth, dt_max, t_end, int(nsteps), tol, int(maxit), rec.ctypes.data, max_rec, T,
        C.byref(tot), C.byref(allc))
    if k < 0:
        raise ValueError("oracle_run_transient rejected the model")
    return TransientResult(rec[:min(k, max_rec)].copy(), T, tot.value, bool(allc.value))
