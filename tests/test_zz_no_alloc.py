"""ct_true_relres_noalloc: the allocation-free residual check, for callers
that must not allocate device memory (a frame loop that may not stall the
GPU, a host framework that owns the device memory pool). It works on the
caller's device arrays with a fixed scratch array inside the library.

Checked through the C ABI against the existing entry point (ct_true_relres on
a solver holding the same temperatures), on two calls in a row, with a call on
a different model in between (the calls share one scratch array), on a
stream other than the current one, on a model of exactly the largest size
the scratch allows, and for the size limit. This file is named to be
collected last.
Tolerance: relative 1e-12 (both compute the same per-cell residuals in FP64;
only the grouping of the two sums differs).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def device_model(ct, torch, m):
    """Copies a model's arrays to device tensors; returns (ct_model, keepalive)."""
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(m, k))).cuda()
         for k in ("gE", "gN", "gU", "gB", "cap", "P")}
    cm = ct.CtModel(m.nx, m.ny, m.nz, m.dx, m.dy, t["gE"].data_ptr(), t["gN"].data_ptr(),
                    t["gU"].data_ptr(), t["gB"].data_ptr(), t["cap"].data_ptr(),
                    t["P"].data_ptr())
    return cm, t


def noalloc_relres(ct, torch, cm, T_dev, stream=None):
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    s = stream if stream is not None else torch.cuda.current_stream()
    if stream is not None:
        s.wait_stream(torch.cuda.current_stream())  # inputs were written on the current stream
    st = ct.lib().ct_true_relres_noalloc(C.byref(cm), C.c_void_p(T_dev.data_ptr()),
                                         C.c_void_p(out.data_ptr()), C.c_void_p(s.cuda_stream))
    assert st == 0, ct.lib().ct_last_error().decode()
    torch.cuda.synchronize()
    return float(out.item())


def solved_field(ct, m, tol):
    with ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        s.solve(tol, 200)
        return s.get_x(), s.true_relres()


def test_noalloc_matches_existing_entry_point(ct):
    torch = pytest.importorskip("torch")
    import workloads

    mA = workloads.steady_hotspot(96, seed=11)
    mB = workloads.four_tier(40, seed=5)
    TA, refA = solved_field(ct, mA, 1e-6)   # a loose solve: a residual well above rounding
    TB, refB = solved_field(ct, mB, 1e-4)
    cmA, keepA = device_model(ct, torch, mA)
    cmB, keepB = device_model(ct, torch, mB)
    TA_dev = torch.from_numpy(TA).cuda()
    TB_dev = torch.from_numpy(TB).cuda()

    a1 = noalloc_relres(ct, torch, cmA, TA_dev)
    a2 = noalloc_relres(ct, torch, cmA, TA_dev)   # second call in a row
    b1 = noalloc_relres(ct, torch, cmB, TB_dev)   # another model through the same scratch
    a3 = noalloc_relres(ct, torch, cmA, TA_dev)
    assert abs(a1 - refA) <= REL_TOL * refA
    assert a2 == a1 and a3 == a1
    assert abs(b1 - refB) <= REL_TOL * refB
    # the same on a stream of its own
    side = torch.cuda.Stream()
    a4 = noalloc_relres(ct, torch, cmA, TA_dev, stream=side)
    assert a4 == a1


def test_noalloc_at_its_column_limit(ct):
    """A model of exactly CT_NOALLOC_MAX_COLUMNS columns (1536 x 1365, two
    planes): every scratch slot is used, and the result matches the solver's."""
    torch = pytest.importorskip("torch")
    nx, ny = 1536, 1365
    assert nx * ny == 2096640  # CT_NOALLOC_MAX_COLUMNS
    layers = [ct.Layer("Si", 50e-6, 130.0, 1.66e6, 1, True), ct.Layer("Cu", 1e-3, 400.0, 3.45e6, 1, False)]
    m = ct.build_model(layers, nx, ny, 10e-3, 10e-3, 2e4, 0.0)
    ct.add_uniform_power(m, 0, 10.0)
    ct.add_hotspot(m, 0, 4e-3, 6e-3, 1e-3, 2.0)
    ct.finalize(m)
    T, ref = solved_field(ct, m, 1e-4)
    cm, keep = device_model(ct, torch, m)
    T_dev = torch.from_numpy(T).cuda()
    r1 = noalloc_relres(ct, torch, cm, T_dev)
    r2 = noalloc_relres(ct, torch, cm, T_dev)
    assert abs(r1 - ref) <= REL_TOL * ref
    assert r2 == r1


def test_noalloc_rejects_models_beyond_its_scratch(ct):
    lib = ct.lib()
    ncol_max = 2096640  # CT_NOALLOC_MAX_COLUMNS
    nx = 2048
    ny = ncol_max // nx + 1
    dummy = C.c_void_p(256)  # never dereferenced: the size check comes first
    cm = ct.CtModel(nx, ny, 10, 1e-5, 1e-5, dummy, dummy, dummy, dummy, dummy, dummy)
    st = lib.ct_true_relres_noalloc(C.byref(cm), dummy, dummy, None)
    assert st == 5  # CT_BAD_ARG
    assert b"exceed the limit" in lib.ct_last_error()
