"""ct_true_relres_noalloc: the allocation-free residual check, for callers
that must not allocate device memory (a frame loop that may not stall the
GPU, a host framework that owns the device memory pool). It works on the
caller's device arrays with a fixed scratch array inside the library.

Checked through the C ABI against the existing entry point (ct_true_relres on
a solver holding the same temperatures), on two calls in a row, with a call on
a different model in between (the calls share one scratch array), and for the
size limit. This file is named to be collected last.
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


def noalloc_relres(ct, torch, cm, T_dev):
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = ct.lib().ct_true_relres_noalloc(C.byref(cm), C.c_void_p(T_dev.data_ptr()),
                                         C.c_void_p(out.data_ptr()), C.c_void_p(stream))
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
