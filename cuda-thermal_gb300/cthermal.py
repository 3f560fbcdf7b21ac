"""Python mirror of cuda-thermal's solver API over libcthermal's C ABI.

Names follow the reference so that its drivers and checks read the same:
``Layer``, ``Model3D``, ``build_model``, ``finalize``, ``default_stack``,
``default_model``, ``add_power_block``, ``add_uniform_power``, ``add_hotspot``,
``add_tsv_region``, ``total_power``, ``heat_out``, ``heat_stored``,
``analytic_1d`` (src/stack3d.h), ``Precond``, ``PcgStats``, ``GpuPcg``,
``gpu_pcg``, ``true_relres``, ``gpu_use_graphs`` (src/pcg3d.h) and
``TransientOptions``, ``StepRecord``, ``run_transient`` (src/transient3d.h).

Every computation goes through libcthermal.so: the model builder's host code
and the CUDA solver. There is no Python or CPU fallback: without the library,
or without a GPU for the solver, calls raise.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libcthermal.so")
MAXZ = 64

_lib = None


class CtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


STATUS_NAMES = {0: "CT_OK", 1: "CT_NOT_CONVERGED", 2: "CT_BREAKDOWN", 3: "CT_CUDA_ERROR",
                4: "CT_TIMEOUT", 5: "CT_BAD_ARG", 6: "CT_NOT_FINALIZED", 7: "CT_NO_DEVICE",
                8: "CT_OUT_OF_MEMORY", 9: "CT_IO_ERROR"}
CT_OK, CT_NOT_CONVERGED, CT_BREAKDOWN = 0, 1, 2


class CtModel(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("dx", C.c_double),
                ("dy", C.c_double), ("gE", C.c_void_p), ("gN", C.c_void_p), ("gU", C.c_void_p),
                ("gB", C.c_void_p), ("cap", C.c_void_p), ("P", C.c_void_p)]


class CtStats(C.Structure):
    _fields_ = [("iters", C.c_int), ("relres", C.c_double), ("converged", C.c_int),
                ("breakdown", C.c_int)]


class CtSetupTimes(C.Structure):
    _fields_ = [("alloc_ms", C.c_double), ("upload_ms", C.c_double), ("levels_ms", C.c_double),
                ("factor_ms", C.c_double), ("graphs_ms", C.c_double)]


class CtStepRecord(C.Structure):
    _fields_ = [("T_max", C.c_double), ("q_out", C.c_double), ("q_stored", C.c_double)]


class CtKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int), ("total_ms", C.c_double),
                ("bytes", C.c_double)]


class CtLayer(C.Structure):
    _fields_ = [("thickness", C.c_double), ("k", C.c_double), ("rho_c", C.c_double),
                ("ncells", C.c_int), ("active", C.c_int)]


class CtGrid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("Lx", C.c_double),
                ("Ly", C.c_double), ("dx", C.c_double), ("dy", C.c_double)]


# Every symbol the C headers declare, with its signature.
def _signatures():
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    gp, lp = C.POINTER(CtGrid), C.POINTER(CtLayer)
    return {
        "ct_version": (C.c_char_p, []),
        "ct_status_string": (C.c_char_p, [i]),
        "ct_last_error": (C.c_char_p, []),
        "ct_use_graphs": (None, [i]),
        "ct_last_setup": (i, [C.POINTER(CtSetupTimes)]),
        "ct_solver_create": (i, [C.POINTER(CtModel), i, i, C.POINTER(vp)]),
        "ct_solver_destroy": (i, [vp]),
        "ct_solver_create_case": (i, [vp, i, i, i, i, i, C.POINTER(vp)]),
        "ct_set_dt": (i, [vp, d]),
        "ct_set_x_zero": (i, [vp]),
        "ct_set_x": (i, [vp, vp]),
        "ct_set_rhs_steady": (i, [vp]),
        "ct_set_rhs_transient": (i, [vp]),
        "ct_set_power": (i, [vp, vp]),
        "ct_set_power_device": (i, [vp, vp]),
        "ct_solve": (i, [vp, d, i, C.POINTER(CtStats)]),
        "ct_solve_async": (i, [vp, d, i]),
        "ct_solve_wait": (i, [vp, C.POINTER(CtStats)]),
        "ct_get_x": (i, [vp, vp]),
        "ct_set_power_async": (i, [vp, vp]),
        "ct_get_x_async": (i, [vp, vp]),
        "ct_copies_wait": (i, [vp]),
        "ct_device_x": (i, [vp, C.POINTER(vp)]),
        "ct_solver_setup_times": (i, [vp, C.POINTER(CtSetupTimes)]),
        "ct_solver_stream": (i, [vp, C.POINTER(vp)]),
        "ct_true_relres": (i, [vp, dp]),
        "ct_solver_step_record": (i, [vp, d, C.POINTER(CtStepRecord)]),
        "ct_solver_step_record_async": (i, [vp, d, i]),
        "ct_solver_step_records": (i, [vp, i, i, C.POINTER(CtStepRecord), C.POINTER(CtStats)]),
        "ct_num_levels": (i, [vp, ip]),
        "ct_level_dims": (i, [vp, i, ip, ip, ip]),
        "ct_level_operator": (i, [vp, i, vp, vp, vp, vp, vp]),
        "ct_level_factors": (i, [vp, i, vp, vp]),
        "ct_profile_solve": (i, [vp, d, i, C.POINTER(CtStats), C.POINTER(CtKernelTime), i, ip]),
        "ct_true_relres_noalloc": (i, [C.POINTER(CtModel), vp, vp, vp]),
        "ct_batch_create": (i, [i, vp, C.POINTER(vp)]),
        "ct_batch_create_prec": (i, [i, vp, i, C.POINTER(vp)]),
        "ct_batch_destroy": (i, [vp]),
        "ct_batch_size": (i, [vp, ip]),
        "ct_batch_set_dt": (i, [vp, vp]),
        "ct_batch_set_x_zero": (i, [vp]),
        "ct_batch_set_x": (i, [vp, i, vp]),
        "ct_batch_set_rhs_steady": (i, [vp]),
        "ct_batch_set_rhs_transient": (i, [vp]),
        "ct_batch_set_power": (i, [vp, i, vp]),
        "ct_batch_set_power_device": (i, [vp, i, vp]),
        "ct_batch_solve": (i, [vp, d, i, vp]),
        "ct_batch_step_transient": (i, [vp, vp, d, i, vp]),
        "ct_batch_get_x": (i, [vp, i, vp]),
        "ct_batch_true_relres": (i, [vp, i, dp]),
        "ct_batch_step_record": (i, [vp, i, d, C.POINTER(CtStepRecord)]),
        "ct_batch_step_records": (i, [vp, vp, vp]),
        "ct_batch_num_buckets": (i, [vp, ip]),
        "ct_batch_stream": (i, [vp, C.POINTER(vp)]),
        "ct_batch_profile_solve": (i, [vp, d, i, vp, C.POINTER(CtKernelTime), i, ip]),
        "ct_batch_bucket_info": (i, [vp, i, ip, ip, vp, vp, vp]),
        "ct_model_planes": (i, [lp, i, ip, vp, vp]),
        "ct_model_finalize": (i, [gp, lp, vp, vp, d, d, d, d, vp, vp, vp, vp, vp, vp]),
        "ct_model_add_power_block": (i, [gp, lp, vp, i, d, d, d, d, d, vp]),
        "ct_model_add_uniform_power": (i, [gp, lp, vp, i, d, vp]),
        "ct_model_add_hotspot": (i, [gp, vp, i, d, d, d, d, vp]),
        "ct_model_add_tsv_region": (i, [gp, vp, i, d, d, d, d, d, vp]),
        "ct_model_total_power": (d, [gp, vp]),
        "ct_model_heat_out": (d, [gp, vp, vp, vp]),
        "ct_model_heat_stored": (d, [gp, vp, vp, vp, d]),
        "ct_model_analytic_1d": (i, [gp, lp, vp, vp, d, vp, vp]),
        "ct_colorize": (i, [vp, i, i, C.c_float, vp, vp, dp, ip, ip]),
        "ct_block_temps": (i, [vp, i, i, d, d, d, d, dp, dp]),
        "ct_case_load": (i, [C.c_char_p, C.POINTER(vp)]),
        "ct_case_destroy": (i, [vp]),
        "ct_case_new": (i, [C.POINTER(CtLayer), i, d, d, d, d, C.POINTER(vp)]),
        "ct_case_add_block": (i, [vp, i, d, d, d, d, d]),
        "ct_case_add_tsv": (i, [vp, i, d, d, d, d, d]),
        "ct_batch_create_cases": (i, [i, vp, vp, vp, vp, C.POINTER(vp)]),
        "ct_batch_create_cases_prec": (i, [i, vp, vp, vp, vp, i, C.POINTER(vp)]),
        "ct_case_info": (i, [vp, ip, ip, ip, dp, dp, dp, dp, dp]),
        "ct_case_layer": (i, [vp, i, C.POINTER(CtLayer), C.c_char_p, i]),
        "ct_case_block": (i, [vp, i, ip, dp, dp, C.c_char_p, i]),
        "ct_case_tsv": (i, [vp, i, ip, dp, dp]),
        "ct_case_export_3dice": (i, [vp, C.c_double, C.c_char_p]),
        "ct_case_set_name": (i, [vp, i, i, C.c_char_p]),
        "ct_case_set_ambient": (i, [vp, C.c_double]),
        "ct_selftest_bounded_wait": (i, [C.c_uint, ip]),
        "ct_selftest_conversions": (i, [C.c_ulonglong, C.c_ulonglong, C.POINTER(C.c_ulonglong)]),
        "ct_probe_fp64_rate": (i, [C.POINTER(C.c_double)]),
        "ct_probe_sync_costs": (i, [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), ip]),
        "ct_eff_kz": (d, [d, d, d]),
        "ct_eff_kxy": (d, [d, d, d]),
    }


SIGNATURES = _signatures()


def lib():
    """Loads libcthermal.so (built by build.py). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libcthermal.so not built ({LIB_PATH}); run build()")
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def build(force: bool = False) -> str:
    import importlib.util
    spec = importlib.util.spec_from_file_location("ct_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def _check(status: int, allow=(CT_OK,)):
    if status not in allow:
        raise CtError(status, lib().ct_last_error().decode())
    return status


def _ptr(a: np.ndarray):
    return a.ctypes.data


# ---- stack model (src/stack3d.h) ------------------------------------------

@dataclass
class Layer:
    name: str
    thickness: float  # m
    k: float          # W/(m K)
    rho_c: float      # J/(m^3 K)
    ncells: int
    active: bool


@dataclass
class Model3D:
    nx: int = 0
    ny: int = 0
    nz: int = 0
    Lx: float = 0.0
    Ly: float = 0.0
    dx: float = 0.0
    dy: float = 0.0
    h_top: float = 0.0
    h_bot: float = 0.0
    T_amb: float = 25.0
    tsv_k: float = 400.0
    tsv_rho_c: float = 3.45e6
    layers: List[Layer] = field(default_factory=list)
    plane_layer: np.ndarray = None
    dz: np.ndarray = None
    tsv_frac: np.ndarray = None
    P: np.ndarray = None
    gE: np.ndarray = None
    gN: np.ndarray = None
    gU: np.ndarray = None
    gB: np.ndarray = None
    cap: np.ndarray = None
    finalized: bool = False

    def nxy(self) -> int:
        return self.nx * self.ny

    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    def idx(self, i, j, l) -> int:
        return (l * self.ny + j) * self.nx + i

    def layer_index(self, name: str) -> int:
        for k, L in enumerate(self.layers):
            if L.name == name:
                return k
        return -1

    # C views
    def _grid(self) -> CtGrid:
        return CtGrid(self.nx, self.ny, self.nz, self.Lx, self.Ly, self.dx, self.dy)

    def _layers(self):
        arr = (CtLayer * len(self.layers))()
        for k, L in enumerate(self.layers):
            arr[k] = CtLayer(L.thickness, L.k, L.rho_c, L.ncells, 1 if L.active else 0)
        return arr

    def ct_model(self) -> CtModel:
        """The ct_model view of the finalized arrays (kept alive by self)."""
        if not self.finalized:
            raise CtError(6, "Model3D used before finalize()")
        return CtModel(self.nx, self.ny, self.nz, self.dx, self.dy, _ptr(self.gE), _ptr(self.gN),
                       _ptr(self.gU), _ptr(self.gB), _ptr(self.cap), _ptr(self.P))


def build_model(layers, nx, ny, Lx, Ly, h_top, h_bot) -> Model3D:
    """build_model (src/stack3d.h:81-102)."""
    m = Model3D(nx=nx, ny=ny, Lx=Lx, Ly=Ly, dx=Lx / nx, dy=Ly / ny, h_top=h_top, h_bot=h_bot,
                layers=list(layers))
    pl = np.zeros(MAXZ, np.int32)
    dz = np.zeros(MAXZ)
    nz = C.c_int(0)
    _check(lib().ct_model_planes(m._layers(), len(layers), C.byref(nz), _ptr(pl), _ptr(dz)))
    m.nz = nz.value
    m.plane_layer = pl[:m.nz].copy()
    m.dz = dz[:m.nz].copy()
    m.tsv_frac = np.zeros(m.ncells())
    m.P = np.zeros(m.ncells())
    return m


def finalize(m: Model3D) -> None:
    """finalize (src/stack3d.h:110-148)."""
    n, nxy = m.ncells(), m.nxy()
    m.gE, m.gN, m.gU, m.cap = (np.zeros(n, np.float32) for _ in range(4))
    m.gB = np.zeros(nxy, np.float32)
    _check(lib().ct_model_finalize(C.byref(m._grid()), m._layers(), _ptr(m.plane_layer),
                                   _ptr(m.dz), m.h_top, m.h_bot, m.tsv_k, m.tsv_rho_c,
                                   _ptr(m.tsv_frac), _ptr(m.gE), _ptr(m.gN), _ptr(m.gU),
                                   _ptr(m.gB), _ptr(m.cap)))
    m.finalized = True


def default_stack() -> List[Layer]:
    """default_stack (src/stack3d.h:150-162)."""
    return [Layer("Si tier 2 (bottom)", 50e-6, 130.0, 1.66e6, 2, True),
            Layer("bond + BEOL", 10e-6, 2.0, 1.70e6, 1, False),
            Layer("Si tier 1 (top)", 50e-6, 130.0, 1.66e6, 2, True),
            Layer("TIM", 25e-6, 5.0, 2.00e6, 1, False),
            Layer("Cu spreader", 1e-3, 400.0, 3.45e6, 4, False)]


def default_model(nx, ny) -> Model3D:
    """default_model (src/stack3d.h:164-168): 10 x 10 mm, 0.5 K/W sink."""
    return build_model(default_stack(), nx, ny, 10e-3, 10e-3, 2e4, 0.0)


def add_power_block(m: Model3D, layer, x0, y0, w, h, watts) -> None:
    _check(lib().ct_model_add_power_block(C.byref(m._grid()), m._layers(), _ptr(m.plane_layer),
                                          layer, x0, y0, w, h, watts, _ptr(m.P)))


def add_uniform_power(m: Model3D, layer, watts) -> None:
    _check(lib().ct_model_add_uniform_power(C.byref(m._grid()), m._layers(), _ptr(m.plane_layer),
                                            layer, watts, _ptr(m.P)))


def add_hotspot(m: Model3D, layer, xc, yc, size, watts) -> None:
    _check(lib().ct_model_add_hotspot(C.byref(m._grid()), _ptr(m.plane_layer), layer, xc, yc,
                                      size, watts, _ptr(m.P)))


def add_tsv_region(m: Model3D, layer, x0, y0, w, h, f) -> None:
    _check(lib().ct_model_add_tsv_region(C.byref(m._grid()), _ptr(m.plane_layer), layer, x0, y0,
                                         w, h, f, _ptr(m.tsv_frac)))
    m.finalized = False


def total_power(m: Model3D) -> float:
    return lib().ct_model_total_power(C.byref(m._grid()), _ptr(m.P))


def heat_out(m: Model3D, T) -> float:
    T = np.ascontiguousarray(T, np.float64)
    return lib().ct_model_heat_out(C.byref(m._grid()), _ptr(m.gU), _ptr(m.gB), _ptr(T))


def heat_stored(m: Model3D, T_old, T_new, dt) -> float:
    a = np.ascontiguousarray(T_old, np.float64)
    b = np.ascontiguousarray(T_new, np.float64)
    return lib().ct_model_heat_stored(C.byref(m._grid()), _ptr(m.cap), _ptr(a), _ptr(b), dt)


def analytic_1d(m: Model3D) -> np.ndarray:
    T = np.zeros(m.nz)
    _check(lib().ct_model_analytic_1d(C.byref(m._grid()), m._layers(), _ptr(m.plane_layer),
                                      _ptr(m.dz), m.h_top, _ptr(m.P), _ptr(T)))
    return T


def eff_kz(k, kc, f) -> float:
    return lib().ct_eff_kz(k, kc, f)


def eff_kxy(k, kc, f) -> float:
    return lib().ct_eff_kxy(k, kc, f)


def layer_planes(m: Model3D, layer: int):
    """First and last plane of a layer."""
    ls = [l for l in range(m.nz) if m.plane_layer[l] == layer]
    return ls[0], ls[-1]


def write_ppm(path: str, rgba: np.ndarray) -> None:
    """An RGBA die map as a binary PPM image, top row = largest y."""
    ny, nx = rgba.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6 %d %d 255\n" % (nx, ny))
        f.write(np.ascontiguousarray(rgba[::-1, :, :3]).tobytes())


def write_tmap(path: str, m: Model3D, tmap: np.ndarray) -> None:
    """A layer's hottest-plane map as CSV in deg C (row = y from the top,
    column = x, 3 decimals), the tmap_layer*.csv format (src/main3d.cu:303-323)."""
    with open(path, "w") as f:
        for j in range(m.ny - 1, -1, -1):
            f.write(",".join("%.3f" % (float(t) + m.T_amb) for t in tmap[j]) + "\n")


# ---- cases (src/case3d.h) -----------------------------------------------------

@dataclass
class PowerBlock:
    name: str
    layer: int
    x0: float  # m
    y0: float
    w: float
    h: float
    watts: float


@dataclass
class TsvRegion:
    layer: int
    x0: float  # m
    y0: float
    w: float
    h: float
    fraction: float


@dataclass
class CaseSpec:
    layers: List[Layer] = field(default_factory=list)
    Lx: float = 10e-3
    Ly: float = 10e-3
    h_top: float = 2e4
    h_bot: float = 0.0
    T_amb: float = 25.0
    blocks: List[PowerBlock] = field(default_factory=list)
    tsvs: List[TsvRegion] = field(default_factory=list)


def load_case(folder: str) -> CaseSpec:
    """load_case (src/case3d.h:86-156) through the library's CSV reader;
    raises CtError with the reference's message on a bad case."""
    h = C.c_void_p()
    _check(lib().ct_case_load(os.fsencode(folder), C.byref(h)))
    try:
        nl, nb, nt = C.c_int(), C.c_int(), C.c_int()
        Lx, Ly, ht, hb, ta = (C.c_double() for _ in range(5))
        _check(lib().ct_case_info(h, C.byref(nl), C.byref(nb), C.byref(nt), C.byref(Lx), C.byref(Ly),
                                  C.byref(ht), C.byref(hb), C.byref(ta)))
        cs = CaseSpec(Lx=Lx.value, Ly=Ly.value, h_top=ht.value, h_bot=hb.value, T_amb=ta.value)
        name = C.create_string_buffer(256)
        for k in range(nl.value):
            v = CtLayer()
            _check(lib().ct_case_layer(h, k, C.byref(v), name, 256))
            cs.layers.append(Layer(name.value.decode(), v.thickness, v.k, v.rho_c, v.ncells,
                                   bool(v.active)))
        rect = (C.c_double * 4)()
        for k in range(nb.value):
            L, w = C.c_int(), C.c_double()
            _check(lib().ct_case_block(h, k, C.byref(L), rect, C.byref(w), name, 256))
            cs.blocks.append(PowerBlock(name.value.decode(), L.value, rect[0], rect[1], rect[2],
                                        rect[3], w.value))
        for k in range(nt.value):
            L, f = C.c_int(), C.c_double()
            _check(lib().ct_case_tsv(h, k, C.byref(L), rect, C.byref(f)))
            cs.tsvs.append(TsvRegion(L.value, rect[0], rect[1], rect[2], rect[3], f.value))
        return cs
    finally:
        lib().ct_case_destroy(h)


def selftest_bounded_wait(polls: int) -> bool:
    """Runs a device wait that nothing completes, bounded at `polls` polls;
    True when it ran out and its kernel returned (the context stays usable)."""
    t = C.c_int(0)
    _check(lib().ct_selftest_bounded_wait(int(polls), C.byref(t)))
    return bool(t.value)


def selftest_conversions(n: int, seed: int = 1) -> int:
    """The integer float <-> double conversions of the FP64 outer kernels
    against the hardware conversions on n bit patterns: the mismatch count."""
    bad = C.c_ulonglong(0)
    _check(lib().ct_selftest_conversions(int(n), int(seed), C.byref(bad)))
    return int(bad.value)


def probe_fp64_rate() -> float:
    """The device's DFMA rate (instructions per second): the denominator of
    the FP64-pipe roofline."""
    r = C.c_double(0.0)
    _check(lib().ct_probe_fp64_rate(C.byref(r)))
    return float(r.value)


def probe_sync_costs(phases: int = 2000, blocks_per_sm: int = 1) -> dict:
    """Microseconds per dependent phase over SMs x blocks_per_sm blocks: a
    grid-wide barrier inside one persistent cooperative kernel against one
    dependently launched kernel per phase in a CUDA graph."""
    bar, lau, nb = C.c_double(0.0), C.c_double(0.0), C.c_int(0)
    _check(lib().ct_probe_sync_costs(int(phases), int(blocks_per_sm), C.byref(bar), C.byref(lau), C.byref(nb)))
    return {"grid_barrier_us": float(bar.value), "dependent_launch_us": float(lau.value), "blocks": int(nb.value),
            "phases": int(phases)}


def export_3dice(case, cell_um: float, outdir: str) -> None:
    """export_3dice (src/case3d.h:267-383) of a case (a folder of CSV files or
    a CaseSpec) on a grid of cell_um micrometres: case.stk, L<k>.flp and
    LT<k>_<p>.lay in the existing folder outdir (3D-ICE 4.0 input). Raises
    CtError with the reference's message when 3D-ICE cannot express the case."""
    if isinstance(case, CaseSpec):
        h = _CaseHandle(case)
        try:
            _check(lib().ct_case_export_3dice(h.h, float(cell_um), os.fsencode(outdir)))
        finally:
            h.close()
        return
    h = C.c_void_p()
    _check(lib().ct_case_load(os.fsencode(case), C.byref(h)))
    try:
        _check(lib().ct_case_export_3dice(h, float(cell_um), os.fsencode(outdir)))
    finally:
        lib().ct_case_destroy(h)


def read_3dice_tmap(path: str) -> np.ndarray:
    """read_3dice_tmap (src/case3d.h:385-400): a 3D-ICE Tmap text file ('%'
    lines are comments) as a 2-D array, one row per line."""
    rows = []
    with open(path) as f:
        for line in f:
            if not line.strip() or line.startswith("%"):
                continue
            vals = [float(v) for v in line.split()]
            if vals:
                rows.append(vals)
    return np.array(rows)


class _CaseHandle:
    """A C ct_case built from a CaseSpec (ct_case_new + blocks + TSVs)."""

    def __init__(self, cs: CaseSpec):
        arr = (CtLayer * len(cs.layers))()
        for k, L in enumerate(cs.layers):
            arr[k] = CtLayer(L.thickness, L.k, L.rho_c, L.ncells, 1 if L.active else 0)
        h = C.c_void_p()
        _check(lib().ct_case_new(arr, len(cs.layers), cs.Lx, cs.Ly, cs.h_top, cs.h_bot, C.byref(h)))
        self.h = h
        for k, L in enumerate(cs.layers):
            _check(lib().ct_case_set_name(h, 0, k, L.name.encode()))
        for k, b in enumerate(cs.blocks):
            _check(lib().ct_case_add_block(h, b.layer, b.x0, b.y0, b.w, b.h, b.watts))
            _check(lib().ct_case_set_name(h, 1, k, b.name.encode()))
        for t in cs.tsvs:
            _check(lib().ct_case_add_tsv(h, t.layer, t.x0, t.y0, t.w, t.h, t.fraction))
        _check(lib().ct_case_set_ambient(h, cs.T_amb))

    def close(self):
        if self.h:
            lib().ct_case_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def case_geometry(cs: CaseSpec, nx: int, ny: int) -> Model3D:
    """The grid and planes of a case's model, without its arrays."""
    m = Model3D(nx=nx, ny=ny, Lx=cs.Lx, Ly=cs.Ly, dx=cs.Lx / nx, dy=cs.Ly / ny, h_top=cs.h_top,
                h_bot=cs.h_bot, T_amb=cs.T_amb, layers=list(cs.layers))
    arr = (CtLayer * len(cs.layers))()
    for k, L in enumerate(cs.layers):
        arr[k] = CtLayer(L.thickness, L.k, L.rho_c, L.ncells, 1 if L.active else 0)
    pl = np.zeros(MAXZ, np.int32)
    dz = np.zeros(MAXZ)
    nz = C.c_int(0)
    _check(lib().ct_model_planes(arr, len(cs.layers), C.byref(nz), _ptr(pl), _ptr(dz)))
    m.nz = nz.value
    m.plane_layer = pl[:m.nz].copy()
    m.dz = dz[:m.nz].copy()
    return m


def build_case_model(cs: CaseSpec, nx: int, ny: int, with_tsv: bool = True) -> Model3D:
    """build_case_model (src/case3d.h:157-166)."""
    m = build_model(cs.layers, nx, ny, cs.Lx, cs.Ly, cs.h_top, cs.h_bot)
    m.T_amb = cs.T_amb
    for b in cs.blocks:
        add_power_block(m, b.layer, b.x0, b.y0, b.w, b.h, b.watts)
    if with_tsv:
        for t in cs.tsvs:
            add_tsv_region(m, t.layer, t.x0, t.y0, t.w, t.h, t.fraction)
    finalize(m)
    return m


def hotspot_model(n: int) -> Model3D:
    """The reference's benchmark model (src/main3d.cu:59-67): 22 W uniform plus
    a 3 W, 1 mm hotspot at (3, 3) mm in the bottom tier, 25 W in the top tier."""
    m = default_model(n, n)
    add_uniform_power(m, 0, 22.0)
    add_hotspot(m, 0, 3e-3, 3e-3, 1e-3, 3.0)
    add_uniform_power(m, 2, 25.0)
    finalize(m)
    return m


# ---- solver (src/pcg3d.h) --------------------------------------------------

class Precond(enum.IntEnum):
    Jacobi = 0
    Multigrid = 1


class Precision(enum.IntEnum):
    MG_FP64 = 0       # plain FP64 MG-PCG (reference -DMG_DOUBLE)
    MG_FP32 = 1       # float V-cycle, Fletcher-Reeves beta (reference default)
    MG_FP32_FLEX = 2  # float V-cycle inside flexible PCG
    MG_FP32_FLEX_DW = 3  # same, outer iteration in double-word arithmetic on FP32 pipes


@dataclass
class PcgStats:
    iters: int = 0
    relres: float = 0.0
    converged: bool = False
    breakdown: bool = False


def gpu_use_graphs(on: bool) -> None:
    lib().ct_use_graphs(1 if on else 0)


class GpuPcg:
    """GpuPcg (src/pcg3d.h:115-163) on libcthermal."""

    def __init__(self, m: Model3D, pc=Precond.Multigrid, precision=Precision.MG_FP32_FLEX):
        self.m = m
        self._cm = m.ct_model()
        self.n = m.ncells()
        h = C.c_void_p()
        _check(lib().ct_solver_create(C.byref(self._cm), int(pc), int(precision), C.byref(h)))
        self._h = h

    @classmethod
    def from_case(cls, folder: str, nx: int, ny: int, with_tsv: bool = True,
                  pc=Precond.Multigrid, precision=Precision.MG_FP32_FLEX) -> "GpuPcg":
        """A solver for a case folder with the model built on the device
        (ct_solver_create_case): no host arrays, no upload. self.m carries the
        geometry (planes, no arrays)."""
        cs = load_case(folder)
        c = C.c_void_p()
        _check(lib().ct_case_load(os.fsencode(folder), C.byref(c)))
        try:
            h = C.c_void_p()
            _check(lib().ct_solver_create_case(c, int(nx), int(ny), 1 if with_tsv else 0, int(pc),
                                               int(precision), C.byref(h)))
        finally:
            lib().ct_case_destroy(c)
        self = cls.__new__(cls)
        self.m = build_model(cs.layers, nx, ny, cs.Lx, cs.Ly, cs.h_top, cs.h_bot)
        self.m.T_amb = cs.T_amb
        self._cm = None
        self.n = self.m.ncells()
        self._h = h
        return self

    @classmethod
    def from_spec(cls, cs: "CaseSpec", nx: int, ny: int, with_tsv: bool = True,
                  pc=Precond.Multigrid, precision=Precision.MG_FP32_FLEX) -> "GpuPcg":
        """A solver for a CaseSpec with the model built on the device."""
        c = _CaseHandle(cs)
        try:
            h = C.c_void_p()
            _check(lib().ct_solver_create_case(c.h, int(nx), int(ny), 1 if with_tsv else 0, int(pc),
                                               int(precision), C.byref(h)))
        finally:
            c.close()
        self = cls.__new__(cls)
        self.m = case_geometry(cs, nx, ny)
        self._cm = None
        self.n = self.m.ncells()
        self._h = h
        return self

    def close(self):
        if getattr(self, "_h", None):
            lib().ct_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_dt(self, dt):
        _check(lib().ct_set_dt(self._h, float(dt)))

    def set_x_zero(self):
        _check(lib().ct_set_x_zero(self._h))

    def set_x(self, T):
        T = np.ascontiguousarray(T, np.float64)
        assert T.size == self.n
        _check(lib().ct_set_x(self._h, _ptr(T)))

    def set_rhs_steady(self):
        _check(lib().ct_set_rhs_steady(self._h))

    def set_rhs_transient(self):
        _check(lib().ct_set_rhs_transient(self._h))

    def set_power(self, P):
        P = np.ascontiguousarray(P, np.float64)
        assert P.size == self.n
        _check(lib().ct_set_power(self._h, _ptr(P)))

    def set_power_device(self, ptr: int):
        _check(lib().ct_set_power_device(self._h, C.c_void_p(ptr)))

    def solve(self, tol, maxit) -> PcgStats:
        st = CtStats()
        _check(lib().ct_solve(self._h, float(tol), int(maxit), C.byref(st)),
               allow=(CT_OK, CT_NOT_CONVERGED, CT_BREAKDOWN))
        return PcgStats(st.iters, st.relres, bool(st.converged), bool(st.breakdown))

    def solve_async(self, tol, maxit) -> None:
        """Queues a solve on the solver's stream and returns (ct_solve_async);
        solve_wait() returns the last queued solve's statistics."""
        _check(lib().ct_solve_async(self._h, float(tol), int(maxit)))

    def solve_wait(self) -> PcgStats:
        st = CtStats()
        _check(lib().ct_solve_wait(self._h, C.byref(st)), allow=(CT_OK, CT_NOT_CONVERGED, CT_BREAKDOWN))
        return PcgStats(st.iters, st.relres, bool(st.converged), bool(st.breakdown))

    def get_x(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        T = out if out is not None else np.empty(self.n)
        _check(lib().ct_get_x(self._h, _ptr(T)))
        return T

    def set_power_async(self, P: np.ndarray) -> None:
        """Queues the copy of P (float64, contiguous; pinned host memory for
        the copy to overlap the solves) and its conversion
        (ct_set_power_async). P must stay unchanged until copies_wait()."""
        assert P.dtype == np.float64 and P.flags.c_contiguous and P.size == self.n
        self.__dict__.setdefault("_pending", []).append(P)
        _check(lib().ct_set_power_async(self._h, _ptr(P)))

    def get_x_async(self, out: np.ndarray) -> None:
        """Queues x's copy into `out` after the solves queued so far
        (ct_get_x_async); `out` holds it once copies_wait() returns."""
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == self.n
        self.__dict__.setdefault("_pending", []).append(out)
        _check(lib().ct_get_x_async(self._h, _ptr(out)))

    def copies_wait(self) -> None:
        """Blocks until every queued copy and the solver's stream are done."""
        _check(lib().ct_copies_wait(self._h))
        self._pending = []

    def device_x(self) -> int:
        p = C.c_void_p()
        _check(lib().ct_device_x(self._h, C.byref(p)))
        return p.value

    def stream(self) -> int:
        p = C.c_void_p()
        _check(lib().ct_solver_stream(self._h, C.byref(p)))
        return p.value or 0

    def setup_times(self) -> dict:
        t = CtSetupTimes()
        _check(lib().ct_solver_setup_times(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in CtSetupTimes._fields_}

    def true_relres(self) -> float:
        v = C.c_double()
        _check(lib().ct_true_relres(self._h, C.byref(v)))
        return v.value

    def step_record(self, dt) -> CtStepRecord:
        r = CtStepRecord()
        _check(lib().ct_solver_step_record(self._h, float(dt), C.byref(r)))
        return r

    def step_record_async(self, dt, slot: int) -> None:
        """Queues the step record, with the last queued solve's statistics,
        into entry `slot` of the device table (ct_solver_step_record_async)."""
        _check(lib().ct_solver_step_record_async(self._h, float(dt), int(slot)))

    def step_records(self, first: int, count: int):
        """Waits for the solver's stream and returns entries first ..
        first + count - 1 of the table: (records, solve statistics)."""
        recs = (CtStepRecord * max(1, count))()
        sts = (CtStats * max(1, count))()
        _check(lib().ct_solver_step_records(self._h, int(first), int(count), recs, sts))
        return ([recs[k] for k in range(count)],
                [PcgStats(sts[k].iters, sts[k].relres, bool(sts[k].converged), bool(sts[k].breakdown))
                 for k in range(count)])

    def num_levels(self) -> int:
        v = C.c_int()
        _check(lib().ct_num_levels(self._h, C.byref(v)))
        return v.value

    def level_dims(self, k):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _check(lib().ct_level_dims(self._h, k, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def level_operator(self, k) -> dict:
        nx, ny, nz = self.level_dims(k)
        n, nxy = nx * ny * nz, nx * ny
        a = [np.empty(n, np.float32) for _ in range(3)] + [np.empty(nxy, np.float32),
                                                           np.empty(n, np.float32)]
        _check(lib().ct_level_operator(self._h, k, *(_ptr(x) for x in a)))
        return dict(zip(("gE", "gN", "gU", "gB", "cap"), a))

    def level_factors(self, k):
        nx, ny, nz = self.level_dims(k)
        fcp, finv = np.empty(nx * ny * nz), np.empty(nx * ny * nz)
        _check(lib().ct_level_factors(self._h, k, _ptr(fcp), _ptr(finv)))
        return fcp, finv

    def colorize(self, l0, l1, rise_hi):
        """Die map of planes l0..l1 (ct_colorize): (rgba (ny, nx, 4) uint8, the
        per-column maximum (ny, nx) float32, hottest rise, i, j). The device
        buffers are torch CUDA tensors."""
        import torch
        nx, ny = self.m.nx, self.m.ny
        rgba = torch.empty((ny, nx, 4), dtype=torch.uint8, device="cuda")
        mp = torch.empty((ny, nx), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        mx, i, j = C.c_double(), C.c_int(), C.c_int()
        _check(lib().ct_colorize(self._h, int(l0), int(l1), float(rise_hi), C.c_void_p(rgba.data_ptr()),
                                 C.c_void_p(mp.data_ptr()), C.byref(mx), C.byref(i), C.byref(j)))
        return rgba.cpu().numpy(), mp.cpu().numpy(), mx.value, i.value, j.value

    def block_temps(self, l0, l1, x0, y0, w, h):
        tmax, tavg = C.c_double(), C.c_double()
        _check(lib().ct_block_temps(self._h, int(l0), int(l1), float(x0), float(y0), float(w),
                                    float(h), C.byref(tmax), C.byref(tavg)))
        return tmax.value, tavg.value

    def profile_solve(self, tol, maxit):
        st = CtStats()
        out = (CtKernelTime * 256)()
        n = C.c_int()
        _check(lib().ct_profile_solve(self._h, float(tol), int(maxit), C.byref(st), out, 256,
                                      C.byref(n)), allow=(CT_OK, CT_NOT_CONVERGED, CT_BREAKDOWN))
        rows = [dict(name=out[k].name.decode(), launches=out[k].launches,
                     total_ms=out[k].total_ms, bytes=out[k].bytes) for k in range(n.value)]
        return PcgStats(st.iters, st.relres, bool(st.converged), bool(st.breakdown)), rows


class GpuBatch:
    """Many independent stacks solved together (ct_batch_*): one launch per
    stage for all instances, per-instance scalars and convergence, one graph
    per size bucket. Instance i is models[i]. precision: Precision.MG_FP32_FLEX
    (FP64 outer iteration) or MG_FP32_FLEX_DW (double words on the FP32
    pipes, the default)."""

    def __init__(self, models, precision=None):
        self.models = list(models)
        self._cms = [m.ct_model() for m in self.models]
        arr = (C.POINTER(CtModel) * len(self._cms))(*[C.pointer(c) for c in self._cms])
        h = C.c_void_p()
        prec = Precision.MG_FP32_FLEX_DW if precision is None else precision
        _check(lib().ct_batch_create_prec(len(self._cms), C.cast(arr, C.c_void_p), int(prec), C.byref(h)))
        self._h = h

    @classmethod
    def from_specs(cls, specs, nx, ny, with_tsv=True, precision=None) -> "GpuBatch":
        """A batch whose instance i is CaseSpec specs[i] on an nx[i] x ny[i]
        grid, every model built on the device (ct_batch_create_cases)."""
        n = len(specs)
        nxs = np.ascontiguousarray(np.broadcast_to(np.asarray(nx, np.int32), (n,)))
        nys = np.ascontiguousarray(np.broadcast_to(np.asarray(ny, np.int32), (n,)))
        wt = np.ascontiguousarray(np.broadcast_to(np.asarray(with_tsv, np.int32), (n,)))
        handles = [_CaseHandle(cs) for cs in specs]
        try:
            arr = (C.c_void_p * n)(*[hd.h.value for hd in handles])
            h = C.c_void_p()
            prec = Precision.MG_FP32_FLEX_DW if precision is None else precision
            _check(lib().ct_batch_create_cases_prec(n, C.cast(arr, C.c_void_p), _ptr(nxs), _ptr(nys), _ptr(wt),
                                                    int(prec), C.byref(h)))
        finally:
            for hd in handles:
                hd.close()
        self = cls.__new__(cls)
        self.models = [case_geometry(cs, int(nxs[i]), int(nys[i])) for i, cs in enumerate(specs)]
        self._cms = []
        self._h = h
        return self

    def __len__(self):
        return len(self.models)

    def close(self):
        if getattr(self, "_h", None):
            lib().ct_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_dt(self, dt=None):
        if dt is None:
            _check(lib().ct_batch_set_dt(self._h, None))
            return
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float64), (len(self),)))
        _check(lib().ct_batch_set_dt(self._h, _ptr(d)))

    def set_x_zero(self):
        _check(lib().ct_batch_set_x_zero(self._h))

    def set_x(self, i, T):
        T = np.ascontiguousarray(T, np.float64)
        assert T.size == self.models[i].ncells()
        _check(lib().ct_batch_set_x(self._h, int(i), _ptr(T)))

    def set_rhs_steady(self):
        _check(lib().ct_batch_set_rhs_steady(self._h))

    def set_rhs_transient(self):
        _check(lib().ct_batch_set_rhs_transient(self._h))

    def set_power(self, i, P):
        P = np.ascontiguousarray(P, np.float64)
        assert P.size == self.models[i].ncells()
        _check(lib().ct_batch_set_power(self._h, int(i), _ptr(P)))

    def set_power_device(self, i, ptr: int):
        """Instance i's power map from device memory (natural layout, ncells
        doubles), ordered on the batch's stream."""
        _check(lib().ct_batch_set_power_device(self._h, int(i), C.c_void_p(ptr)))

    @staticmethod
    def _stats(arr):
        return [PcgStats(s.iters, s.relres, bool(s.converged), bool(s.breakdown)) for s in arr]

    def solve(self, tol, maxit) -> List[PcgStats]:
        st = (CtStats * len(self))()
        _check(lib().ct_batch_solve(self._h, float(tol), int(maxit), C.cast(st, C.c_void_p)),
               allow=(CT_OK, CT_NOT_CONVERGED, CT_BREAKDOWN))
        return self._stats(st)

    def step_transient(self, dt, tol, maxit) -> List[PcgStats]:
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float64), (len(self),)))
        st = (CtStats * len(self))()
        _check(lib().ct_batch_step_transient(self._h, _ptr(d), float(tol), int(maxit),
                                             C.cast(st, C.c_void_p)),
               allow=(CT_OK, CT_NOT_CONVERGED, CT_BREAKDOWN))
        return self._stats(st)

    def get_x(self, i, out: Optional[np.ndarray] = None) -> np.ndarray:
        T = out if out is not None else np.empty(self.models[i].ncells())
        _check(lib().ct_batch_get_x(self._h, int(i), _ptr(T)))
        return T

    def true_relres(self, i) -> float:
        v = C.c_double()
        _check(lib().ct_batch_true_relres(self._h, int(i), C.byref(v)))
        return v.value

    def step_record(self, i, dt) -> CtStepRecord:
        r = CtStepRecord()
        _check(lib().ct_batch_step_record(self._h, int(i), float(dt), C.byref(r)))
        return r

    def profile_solve(self, tol, maxit):
        st = (CtStats * len(self))()
        out = (CtKernelTime * 256)()
        n = C.c_int()
        _check(lib().ct_batch_profile_solve(self._h, float(tol), int(maxit), C.cast(st, C.c_void_p),
                                            out, 256, C.byref(n)),
               allow=(CT_OK, CT_NOT_CONVERGED, CT_BREAKDOWN))
        rows = [dict(name=out[k].name.decode(), launches=out[k].launches,
                     total_ms=out[k].total_ms, bytes=out[k].bytes) for k in range(n.value)]
        return self._stats(st), rows

    def stream(self) -> int:
        p = C.c_void_p()
        _check(lib().ct_batch_stream(self._h, C.byref(p)))
        return p.value or 0

    def step_records(self, dt) -> np.ndarray:
        """(n, 3) array: T_max, q_out, q_stored of every instance's last step."""
        d = np.ascontiguousarray(np.broadcast_to(np.asarray(dt, np.float64), (len(self),)))
        out = (CtStepRecord * len(self))()
        _check(lib().ct_batch_step_records(self._h, _ptr(d), C.cast(out, C.c_void_p)))
        return np.array([(r.T_max, r.q_out, r.q_stored) for r in out])

    def buckets(self) -> List[dict]:
        nb = C.c_int()
        _check(lib().ct_batch_num_buckets(self._h, C.byref(nb)))
        out = []
        for k in range(nb.value):
            n, dep = C.c_int(), C.c_int()
            _check(lib().ct_batch_bucket_info(self._h, k, C.byref(n), C.byref(dep), None, None,
                                              None))
            sw = (C.c_uint * max(1, dep.value))()
            rs = (C.c_uint * max(1, dep.value))()
            sg = (C.c_int * max(1, dep.value))()
            _check(lib().ct_batch_bucket_info(self._h, k, None, None, sw, rs, sg))
            out.append(dict(instances=n.value, depth=dep.value,
                            sweep_tiles=list(sw)[:dep.value], restrict_tiles=list(rs)[:dep.value],
                            staged=[bool(v) for v in list(sg)[:dep.value]]))
        return out


@dataclass
class SolveResult:
    T: np.ndarray
    iters: int = 0
    relres: float = 0.0
    ms: float = 0.0
    setup_ms: float = 0.0
    solve_ms: float = 0.0
    converged: bool = False


def gpu_pcg(m: Model3D, tol, maxit, pc=Precond.Multigrid,
            precision=Precision.MG_FP32_FLEX) -> SolveResult:
    """gpu_pcg (src/pcg3d_gpu.cu:684-719): steady solve from T = 0."""
    t0 = time.perf_counter()
    s = GpuPcg(m, pc, precision)
    s.set_x_zero()
    s.set_rhs_steady()
    t1 = time.perf_counter()
    st = s.solve(tol, maxit)
    t2 = time.perf_counter()
    T = s.get_x()
    s.close()
    t3 = time.perf_counter()
    return SolveResult(T, st.iters, st.relres, (t3 - t0) * 1e3, (t1 - t0) * 1e3, (t2 - t1) * 1e3,
                       st.converged)


def true_relres(m: Model3D, T) -> float:
    """||P - A T|| / ||P|| in double (src/pcg3d_cpu.cpp:207-220), on the GPU."""
    s = GpuPcg(m, Precond.Jacobi)
    s.set_x(T)
    v = s.true_relres()
    s.close()
    return v


# ---- transient (src/transient3d.h) -----------------------------------------

@dataclass
class TransientOptions:
    dt0: float = 1e-5
    growth: float = 1.1
    dt_max: float = 0.05
    t_end: float = 1.0
    tol: float = 1e-9
    maxit: int = 50000
    precond: Precond = Precond.Multigrid
    precision: Precision = Precision.MG_FP32_FLEX
    nsteps: int = 0  # > 0: run this many steps instead of up to t_end


@dataclass
class StepRecord:
    t: float
    dt: float
    iters: int
    T_max: float
    q_out: float
    q_stored: float


@dataclass
class TransientResult:
    steps: List[StepRecord] = field(default_factory=list)
    T: np.ndarray = None
    total_iters: int = 0
    ms: float = 0.0
    solve_ms: float = 0.0
    converged: bool = True


def write_transient_csv(path: str, steps: List["StepRecord"], T_amb: float) -> None:
    """The transient log of the reference driver (src/main3d.cu:549-557): one
    row per step, t and dt in s, PCG iterations, hottest cell in C, heat out
    and heat stored in W."""
    with open(path, "w") as f:
        f.write("t_s,dt_s,pcg_iters,T_max_C,heat_out_W,heat_stored_W\n")
        for r in steps:
            f.write("%.6e,%.6e,%d,%.6f,%.6f,%.6f\n" % (r.t, r.dt, r.iters, r.T_max + T_amb, r.q_out,
                                                      r.q_stored))


def run_transient(m: Model3D, o: TransientOptions = TransientOptions(),
                  device_records: bool = True) -> TransientResult:
    """run_transient (src/transient3d.h:48-90): backward Euler from T = 0 with
    geometric dt growth. With device_records the per-step T_max, heat out and
    heat stored are reduced on the GPU and every step is queued on the
    solver's stream (ct_solve_async, ct_solver_step_record_async) with one
    wait at the end, the field staying on the device; otherwise T is copied
    to the host every step, as the reference does."""
    t0 = time.perf_counter()
    res = TransientResult()
    s = GpuPcg(m, o.precond, o.precision)
    s.set_x_zero()
    T_old = np.zeros(m.ncells())
    t, dt, last_dt = 0.0, o.dt0, -1.0
    k = 0
    if device_records:
        steps = []
        while (k < o.nsteps) if o.nsteps > 0 else (t < o.t_end * (1 - 1e-12)):
            if o.nsteps <= 0:
                dt = min(dt, o.t_end - t)
            if dt != last_dt:
                s.set_dt(dt)
                last_dt = dt
            s.set_rhs_transient()
            s.solve_async(o.tol, o.maxit)
            s.step_record_async(dt, k)
            t += dt
            steps.append((t, dt))
            dt = min(dt * o.growth, o.dt_max)
            k += 1
        recs, sts = s.step_records(0, k)
        for (tk, dtk), r, st in zip(steps, recs, sts):
            res.steps.append(StepRecord(tk, dtk, st.iters, r.T_max, r.q_out, r.q_stored))
            res.total_iters += st.iters
            res.converged = res.converged and st.converged
        res.solve_ms = (time.perf_counter() - t0) * 1e3
        res.T = s.get_x()
        s.close()
        res.ms = (time.perf_counter() - t0) * 1e3
        return res
    while (k < o.nsteps) if o.nsteps > 0 else (t < o.t_end * (1 - 1e-12)):
        if o.nsteps <= 0:
            dt = min(dt, o.t_end - t)
        ts = time.perf_counter()
        if dt != last_dt:
            s.set_dt(dt)
            last_dt = dt
        s.set_rhs_transient()
        st = s.solve(o.tol, o.maxit)
        res.solve_ms += (time.perf_counter() - ts) * 1e3
        t += dt
        T_new = s.get_x()
        rec = StepRecord(t, dt, st.iters, float(T_new.max()), heat_out(m, T_new),
                         heat_stored(m, T_old, T_new, dt))
        T_old = T_new
        res.steps.append(rec)
        res.total_iters += st.iters
        res.converged = res.converged and st.converged
        dt = min(dt * o.growth, o.dt_max)
        k += 1
    res.T = s.get_x()
    s.close()
    res.ms = (time.perf_counter() - t0) * 1e3
    return res
