"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; the Python mirror binds each of them."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(INCLUDE, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(ct_[a-z0-9_]+)\s*\(",
                             src, flags=re.M):
            names.add(m.group(1))
    return names


def test_headers_declare_functions():
    names = declared_functions()
    assert "ct_solver_create" in names and "ct_solve" in names and "ct_model_finalize" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(ctlib, ct):
    out = subprocess.run(["nm", "-D", "--defined-only", ct.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = declared_functions() - exported
    assert not missing, missing


def test_python_mirror_binds_every_symbol(ctlib, ct):
    assert declared_functions() <= set(ct.SIGNATURES)
    for name in declared_functions():
        assert getattr(ctlib, name) is not None


def test_status_strings_and_errors_without_gpu(ctlib, ct):
    assert ctlib.ct_status_string(0) == b"ok"
    assert ctlib.ct_status_string(2) == b"breakdown"
    assert b"sm_103a" in ctlib.ct_version()
    # argument checks run before any device call
    import ctypes as C
    h = C.c_void_p()
    assert ctlib.ct_solver_create(None, 1, 2, C.byref(h)) == 5
    assert b"null model" in ctlib.ct_last_error()
    assert ctlib.ct_solve(None, 1e-6, 10, None) == 5


def test_queued_calls_refuse_a_null_solver_without_gpu(ctlib, ct):
    """The queued copies and queued step records check their solver before
    any device call."""
    import ctypes as C
    buf = (C.c_double * 4)()
    assert ctlib.ct_set_power_async(None, buf) == 5
    assert ctlib.ct_get_x_async(None, buf) == 5
    assert ctlib.ct_copies_wait(None) == 5
    assert ctlib.ct_solver_step_record_async(None, 1e-3, 0) == 5
    assert ctlib.ct_solver_step_records(None, 0, 1, None, None) == 5
    assert ctlib.ct_solve_async(None, 1e-6, 10) == 5
    assert ctlib.ct_solve_wait(None, None) == 5


def test_unfinalized_model_rejected(ctlib, ct):
    m = ct.default_model(8, 8)
    with pytest.raises(ct.CtError) as e:
        ct.GpuPcg(m)
    assert e.value.status == 6


def test_noalloc_argument_checks_without_gpu(ctlib, ct):
    """ct_true_relres_noalloc rejects bad arguments before any device call:
    too many planes, a null model array, a null output."""
    import ctypes as C
    dummy = C.c_void_p(256)  # never dereferenced
    deep = ct.CtModel(8, 8, 65, 1e-5, 1e-5, dummy, dummy, dummy, dummy, dummy, dummy)
    assert ctlib.ct_true_relres_noalloc(C.byref(deep), dummy, dummy, None) == 5
    assert b"bad size" in ctlib.ct_last_error()
    no_gb = ct.CtModel(8, 8, 10, 1e-5, 1e-5, dummy, dummy, dummy, None, dummy, dummy)
    assert ctlib.ct_true_relres_noalloc(C.byref(no_gb), dummy, dummy, None) == 5
    assert b"null model array" in ctlib.ct_last_error()
    ok = ct.CtModel(8, 8, 10, 1e-5, 1e-5, dummy, dummy, dummy, dummy, dummy, dummy)
    assert ctlib.ct_true_relres_noalloc(C.byref(ok), dummy, None, None) == 5
    assert b"null argument" in ctlib.ct_last_error()
