"""ctypes bindings to the UNMODIFIED reference solvers (oracle/_ref/).

TEST AND COMPARISON INFRASTRUCTURE ONLY: used to generate tests/golden/
fixtures (tests/golden/make_golden.py), to pin the C oracle against the
reference directly, and as the timed reference arm of bench.py (the
reference CPU solver, and the reference GPU solver on the same inputs).

``oracle/_ref/<machine>/`` is built by ``make -C oracle ref ref-gpu`` from an unmodified
copy of the reference's own sources (src/pcg3d_cpu.cpp, src/pcg3d_gpu.cu and
their headers) that ``make -C oracle stage`` places under baseline/_ref/src
(git-ignored; it travels with the working tree, so machines without a
checkout of the reference can build it too). Nothing on the product path
needs any of it.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref", platform.machine())
REF_SRC = os.environ.get("CT_REFERENCE_SRC", os.path.join(REPO, "baseline", "_ref", "src"))


def stage() -> bool:
    """Copies the reference's solver sources into baseline/_ref/src when a
    checkout of the reference sits beside this repository; True if a staged
    copy is present afterwards."""
    subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF_SRC={REF_SRC}"],
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return available()


def available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "pcg3d_cpu.cpp"))


def build(gpu: bool = False) -> None:
    if not available():
        raise RuntimeError("reference sources not staged (make -C oracle stage)")
    targets = ["ref", "ref-gpu"] if gpu else ["ref"]
    subprocess.run(["make", "-s", "-j8", "-C", HERE, *targets, f"REF_SRC={REF_SRC}"], check=True)


class RefLayer(C.Structure):
    _fields_ = [("thickness", C.c_double), ("k", C.c_double), ("rho_c", C.c_double),
                ("ncells", C.c_int), ("active", C.c_int)]


class RefPower(C.Structure):
    _fields_ = [("kind", C.c_int), ("layer", C.c_int), ("x0", C.c_double), ("y0", C.c_double),
                ("w", C.c_double), ("h", C.c_double), ("watts", C.c_double)]


class RefTsv(C.Structure):
    _fields_ = [("layer", C.c_int), ("x0", C.c_double), ("y0", C.c_double), ("w", C.c_double),
                ("h", C.c_double), ("f", C.c_double)]


_libs = {}


def _bind_model(L) -> None:
    """Argument types of the model, CPU solver and transient entry points
    (ref_harness.cpp), present in every reference library."""
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.ref_model_new.restype = vp
    L.ref_model_new.argtypes = [C.POINTER(RefLayer), C.c_int, C.c_int, C.c_int, C.c_double,
                                C.c_double, C.c_double, C.c_double, C.POINTER(RefPower),
                                C.c_int, C.POINTER(RefTsv), C.c_int]
    L.ref_case_model.restype = vp
    L.ref_case_model.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_char_p, C.c_int]
    L.ref_export_3dice.restype = C.c_int
    L.ref_export_3dice.argtypes = [C.c_char_p, C.c_double, C.c_char_p, C.c_char_p, C.c_int]
    L.ref_example_case_model.restype = vp
    L.ref_example_case_model.argtypes = [C.c_int, C.c_int, C.c_int]
    L.ref_model_free.argtypes = [vp]
    L.ref_model_dims.argtypes = [vp, ip, ip, ip, dp, dp]
    L.ref_model_arrays.argtypes = [vp] + [vp] * 9
    L.ref_total_power.restype = C.c_double
    L.ref_total_power.argtypes = [vp]
    L.ref_analytic_1d.argtypes = [vp, vp]
    L.ref_cpu_pcg.restype = C.c_int
    L.ref_cpu_pcg.argtypes = [vp, C.c_double, C.c_int, C.c_int, vp, ip, dp, dp, dp]
    L.ref_true_relres.restype = C.c_double
    L.ref_true_relres.argtypes = [vp, vp]
    L.ref_heat_out.restype = C.c_double
    L.ref_heat_out.argtypes = [vp, vp]
    L.ref_num_levels.restype = C.c_int
    L.ref_num_levels.argtypes = [vp]
    L.ref_level.argtypes = [vp, C.c_int, ip, ip, vp, vp, vp, vp, vp]
    L.ref_run_transient.restype = C.c_int
    L.ref_run_transient.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_double, C.c_int, vp, C.c_int, vp, C.POINTER(C.c_long), ip]
    L.ref_mg_double.restype = C.c_int
    L.ref_cpu_solver_new.restype = vp
    L.ref_cpu_solver_new.argtypes = [vp, C.c_int]
    L.ref_cpu_solver_free.argtypes = [vp]
    L.ref_cpu_solver_steady.restype = C.c_int
    L.ref_cpu_solver_steady.argtypes = [vp, C.c_double, C.c_int, ip, dp]
    L.ref_cpu_solver_get_x.argtypes = [vp, vp]
    L.ref_default_model_new.restype = vp
    L.ref_default_model_new.argtypes = [C.c_int, C.c_int, C.POINTER(RefPower), C.c_int]


def lib(mg_double: bool):
    key = bool(mg_double)
    if key in _libs:
        return _libs[key]
    path = os.path.join(OUT, "libref_mgd.so" if key else "libref_mgf.so")
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    _bind_model(L)
    _libs[key] = L
    return L


_gpu_libs = {}


def gpu_lib(mg_double: bool):
    """The reference GPU solver (with the same CPU entry points as lib())."""
    key = bool(mg_double)
    if key in _gpu_libs:
        return _gpu_libs[key]
    path = os.path.join(OUT, "libref_gpu_mgd.so" if key else "libref_gpu_mgf.so")
    if not os.path.exists(path):
        build(gpu=True)
    L = C.CDLL(path)
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    _bind_model(L)
    L.refg_mg_double.restype = C.c_int
    L.refg_device_count.restype = C.c_int
    L.refg_use_graphs.argtypes = [C.c_int]
    L.refg_solver_new.restype = vp
    L.refg_solver_new.argtypes = [vp, C.c_int, dp]
    L.refg_solver_free.argtypes = [vp]
    L.refg_solve_steady.restype = C.c_int
    L.refg_solve_steady.argtypes = [vp, C.c_double, C.c_int, ip, dp]
    L.refg_get_x.argtypes = [vp, vp]
    _gpu_libs[key] = L
    return L


@dataclass
class RefModel:
    """A finalized reference Model3D's arrays (natural layout)."""
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    gE: np.ndarray
    gN: np.ndarray
    gU: np.ndarray
    gB: np.ndarray
    cap: np.ndarray
    P: np.ndarray
    dz: np.ndarray
    tsv_frac: np.ndarray
    plane_layer: np.ndarray
    handle: int = 0
    mg_double: bool = True
    owner: object = None  # the library that built it (frees it)

    def __del__(self):
        if self.handle:
            (self.owner or lib(self.mg_double)).ref_model_free(self.handle)
            self.handle = 0


def _wrap(L, h, mg_double) -> RefModel:
    if not h:
        raise RuntimeError("reference model construction failed")
    nx, ny, nz = C.c_int(), C.c_int(), C.c_int()
    dx, dy = C.c_double(), C.c_double()
    L.ref_model_dims(h, C.byref(nx), C.byref(ny), C.byref(nz), C.byref(dx), C.byref(dy))
    n, nxy = nx.value * ny.value * nz.value, nx.value * ny.value
    gE, gN, gU, cap = (np.empty(n, np.float32) for _ in range(4))
    gB = np.empty(nxy, np.float32)
    P, tsv = np.empty(n), np.empty(n)
    dz = np.empty(nz.value)
    pl = np.empty(nz.value, np.int32)
    L.ref_model_arrays(h, *(a.ctypes.data for a in (gE, gN, gU, gB, cap, P, dz, tsv, pl)))
    return RefModel(nx.value, ny.value, nz.value, dx.value, dy.value, gE, gN, gU, gB, cap, P, dz,
                    tsv, pl, h, mg_double, L)


def model(layers, nx, ny, Lx, Ly, h_top, h_bot, power=(), tsvs=(), mg_double=True) -> RefModel:
    """layers: [(thickness, k, rho_c, ncells, active)]; power: [(kind, layer,
    x0, y0, w, h, watts)] with kind "block", "uniform" or "hotspot" (for a
    hotspot x0, y0 are the centre and w the side); tsvs: [(layer, x0, y0, w, h,
    f)]. Applied in order, then finalize()."""
    L = lib(mg_double)
    la = (RefLayer * max(1, len(layers)))(*[RefLayer(*l) for l in layers])
    kinds = {"block": 0, "uniform": 1, "hotspot": 2}
    pw = [RefPower(kinds[p[0]], *p[1:]) for p in power]
    pa = (RefPower * max(1, len(pw)))(*pw)
    tv = [RefTsv(*t) for t in tsvs]
    ta = (RefTsv * max(1, len(tv)))(*tv)
    h = L.ref_model_new(la, len(layers), nx, ny, Lx, Ly, h_top, h_bot, pa, len(pw), ta, len(tv))
    return _wrap(L, h, mg_double)


def default_model(nx, ny, power=(), mg_double=True, gpu=False) -> RefModel:
    """default_model(nx, ny) (src/stack3d.h:165-168) with the power operations
    listed as in model(), then finalize(); gpu: built by the library that also
    holds the reference GPU solver (models are solved by the library that
    built them)."""
    L = gpu_lib(mg_double) if gpu else lib(mg_double)
    kinds = {"block": 0, "uniform": 1, "hotspot": 2}
    pw = [RefPower(kinds[p[0]], *p[1:]) for p in power]
    pa = (RefPower * max(1, len(pw)))(*pw)
    return _wrap(L, L.ref_default_model_new(nx, ny, pa, len(pw)), mg_double)


def case_model(folder, nx, ny, with_tsv=True, mg_double=True) -> RefModel:
    L = lib(mg_double)
    err = C.create_string_buffer(512)
    h = L.ref_case_model(folder.encode(), nx, ny, int(with_tsv), err, 512)
    if not h:
        raise RuntimeError(err.value.decode())
    return _wrap(L, h, mg_double)


def export_3dice(folder, cell_um, outdir):
    """The reference's export_3dice of a case folder into outdir; None on
    success, else its error message."""
    L = lib(False)
    err = C.create_string_buffer(512)
    ok = L.ref_export_3dice(folder.encode(), float(cell_um), outdir.encode(), err, 512)
    return None if ok else err.value.decode()


def example_case_model(nx, ny, with_tsv=True, mg_double=True) -> RefModel:
    L = lib(mg_double)
    return _wrap(L, L.ref_example_case_model(nx, ny, int(with_tsv)), mg_double)


def cpu_pcg(m: RefModel, tol, maxit, precond="multigrid"):
    L = lib(m.mg_double)
    T = np.empty(m.nx * m.ny * m.nz)
    it, rel, sms, vms = C.c_int(), C.c_double(), C.c_double(), C.c_double()
    conv = L.ref_cpu_pcg(m.handle, tol, maxit, 1 if precond == "multigrid" else 0, T.ctypes.data,
                         C.byref(it), C.byref(rel), C.byref(sms), C.byref(vms))
    return dict(T=T, iters=it.value, relres=rel.value, converged=bool(conv),
                setup_ms=sms.value, solve_ms=vms.value)


def true_relres(m: RefModel, T) -> float:
    T = np.ascontiguousarray(T, np.float64)
    return lib(m.mg_double).ref_true_relres(m.handle, T.ctypes.data)


def heat_out(m: RefModel, T) -> float:
    T = np.ascontiguousarray(T, np.float64)
    return lib(m.mg_double).ref_heat_out(m.handle, T.ctypes.data)


def total_power(m: RefModel) -> float:
    return lib(m.mg_double).ref_total_power(m.handle)


def analytic_1d(m: RefModel) -> np.ndarray:
    out = np.empty(m.nz)
    lib(m.mg_double).ref_analytic_1d(m.handle, out.ctypes.data)
    return out


def levels(m: RefModel):
    L = lib(m.mg_double)
    out = []
    for k in range(L.ref_num_levels(m.handle)):
        nx, ny = C.c_int(), C.c_int()
        L.ref_level(m.handle, k, C.byref(nx), C.byref(ny), None, None, None, None, None)
        n, nxy = nx.value * ny.value * m.nz, nx.value * ny.value
        a = [np.empty(n, np.float32) for _ in range(3)] + [np.empty(nxy, np.float32),
                                                           np.empty(n, np.float32)]
        L.ref_level(m.handle, k, C.byref(nx), C.byref(ny), *(x.ctypes.data for x in a))
        out.append(dict(nx=nx.value, ny=ny.value, gE=a[0], gN=a[1], gU=a[2], gB=a[3], cap=a[4]))
    return out


def run_transient(m: RefModel, precond="multigrid", dt0=1e-5, growth=1.1, dt_max=0.05,
                  t_end=1.0, tol=1e-9, maxit=50000, max_rec=100000):
    L = lib(m.mg_double)
    rec = np.zeros((max_rec, 6))
    T = np.empty(m.nx * m.ny * m.nz)
    tot, allc = C.c_long(), C.c_int()
    k = L.ref_run_transient(m.handle, 1 if precond == "multigrid" else 0, dt0, growth, dt_max,
                            t_end, tol, maxit, rec.ctypes.data, max_rec, T.ctypes.data,
                            C.byref(tot), C.byref(allc))
    return dict(steps=rec[:min(k, max_rec)].copy(), T=T, total_iters=tot.value,
                converged=bool(allc.value))
