"""The C oracle is pinned to the reference CPU solver's own outputs: for every
golden case it must reproduce the reference's temperatures bit for bit (same
SHA-256 of the T bytes), iteration counts and residuals, in both V-cycle
precisions, with Jacobi, through transients, and its multigrid hierarchy must
equal mg_build_levels (src/mg3d.h:147-183) bit for bit."""
import hashlib

import numpy as np
import pytest

from conftest import build_spec_model


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


CASES = ["hotspot64", "uniform64", "blocks_tsv_17x13", "blocks_tsv_40x24", "tiny3x5",
         "column1x1", "row1x9", "tsv_layer64", "base3dice_50"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_steady_bitwise(orc, ct, golden, name):
    rec = golden["cases"][name]
    m = build_spec_model(ct, rec["spec"])
    for key, kw, tol in (("mg_f64", dict(precond="multigrid", mg_double=True), 1e-10),
                         ("mg_f32", dict(precond="multigrid", mg_double=False), 1e-10),
                         ("jacobi", dict(precond="jacobi", mg_double=True), 1e-6)):
        r = orc.solve_steady(m, tol, 50000, **kw)
        g = rec[key]
        assert r.iters == g["iters"], key
        assert r.converged == g["converged"], key
        assert r.relres == g["relres"], key
        assert sha(r.T) == g["T_sha"], key
        assert orc.true_relres(m, r.T) == g["true_relres"], key
        assert orc.heat_out(m, r.T) == g["heat_out"], key


@pytest.mark.parametrize("name", ["tiny3x5", "column1x1", "row1x9", "blocks_tsv_17x13"])
def test_oracle_small_arrays(orc, ct, golden, name):
    arr = golden["arrays"]
    m = build_spec_model(ct, golden["cases"][name]["spec"])
    r = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
    np.testing.assert_array_equal(r.T, arr[f"{name}.T_mg_f64"])


@pytest.mark.parametrize("name", ["hotspot64", "blocks_tsv_17x13", "tiny3x5", "row1x9"])
def test_oracle_levels_bitwise(orc, ct, golden, name):
    rec = golden["cases"][name]
    m = build_spec_model(ct, rec["spec"])
    s = orc.Solver(m, "multigrid", mg_double=True)
    assert s.num_levels() == len(rec["levels"])
    for k, L in enumerate(rec["levels"]):
        nx, ny, nz = s.level_dims(k)
        assert (nx, ny) == (L["nx"], L["ny"])
        op = s.level_operator(k)
        for a in ("gE", "gN", "gU", "gB", "cap"):
            assert sha(op[a]) == L["sha"][a], (k, a)


@pytest.mark.parametrize("key", ["hotspot32_multigrid_f32", "hotspot32_multigrid_f64",
                                 "hotspot32_jacobi_f64"])
def test_oracle_transient_bitwise(orc, ct, golden, key):
    g = golden["transients"][key]
    spec = dict(golden["cases"]["hotspot64"]["spec"])
    spec["nx"] = spec["ny"] = 32
    m = build_spec_model(ct, spec)
    pc = "jacobi" if "jacobi" in key else "multigrid"
    tr = orc.run_transient(m, pc, mg_double=key.endswith("f64"), dt0=1e-5, growth=1.2,
                           dt_max=0.05, t_end=0.02, tol=1e-9)
    np.testing.assert_array_equal(tr.steps, np.array(g["steps"]))
    assert sha(tr.T) == g["T_sha"]
    assert tr.total_iters == g["total_iters"]


def test_oracle_energy_and_1d(orc, ct, golden):
    """Checks the oracle the reference's way (src/main3d.cu:97-125): uniform
    power vs the exact 1D chain, energy balance, true residual."""
    rec = golden["cases"]["uniform64"]
    m = build_spec_model(ct, rec["spec"])
    r = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
    Tz = np.array(rec["analytic_1d"])
    err = np.abs(r.T.reshape(m.nz, -1) - Tz[:, None]).max()
    assert err / Tz.max() < 1e-4
    P = ct.total_power(m)
    assert abs(orc.heat_out(m, r.T) - P) / P < 1e-8
    assert orc.true_relres(m, r.T) < 1e-9
