"""GPU solver parity against the C oracle (itself pinned bit-for-bit to the
reference CPU solver), through the C ABI.

Tolerances (written here, used below):
  * plain FP64 MG-PCG and the reference-default FP32 V-cycle vs the oracle of
    the same arithmetic: max|dT| <= 1e-7 * Tmax; iteration counts within 1.
  * FP32 V-cycle inside flexible PCG vs the FP64 oracle: max|dT| <= 5e-4 K
    (the stated bound) and, in practice, <= 1e-7 * Tmax.
  * Jacobi (tol 1e-6) vs the oracle's Jacobi: max|dT| / Tmax <= 1e-6, the
    reference's own GPU-vs-CPU bound (src/main3d.cu:41).
  * true residual ||P - A T|| / ||P|| (FP64, recomputed by the oracle) <= 1e-9
    for solves to 1e-10.
Setup is checked bit for bit: level sizes, every coarse operator array and
every column factor.
"""
import hashlib

import numpy as np
import pytest

from conftest import build_spec_model

pytestmark = pytest.mark.gpu

DT_BOUND_K = 5e-4
CASES = ["hotspot64", "blocks_tsv_17x13", "blocks_tsv_40x24", "tiny3x5", "column1x1", "row1x9",
         "tsv_layer64", "base3dice_50"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def deep_stack(ct, nx, cu_planes, ny=None):
    """The default stack with a copper spreader of cu_planes planes (6 +
    cu_planes planes in all), 10 x 9 mm, 35 W with a hotspot."""
    layers = [ct.Layer("Si tier 2 (bottom)", 50e-6, 130.0, 1.66e6, 2, True),
              ct.Layer("bond + BEOL", 10e-6, 2.0, 1.70e6, 1, False),
              ct.Layer("Si tier 1 (top)", 50e-6, 130.0, 1.66e6, 2, True),
              ct.Layer("TIM", 25e-6, 5.0, 2.00e6, 1, False),
              ct.Layer("Cu spreader", 1e-3, 400.0, 3.45e6, cu_planes, False)]
    m = ct.build_model(layers, nx, ny or nx, 10e-3, 9e-3, 2e4, 0.0)
    ct.add_uniform_power(m, 0, 20.0)
    ct.add_hotspot(m, 0, 3e-3, 4e-3, 1e-3, 3.0)
    ct.add_uniform_power(m, 2, 15.0)
    ct.finalize(m)
    return m


class env_vars:
    """Sets environment variables (None: unset) while a solver is created
    (the solver reads its switches then), and restores them after."""

    def __init__(self, **kw):
        self.kw = kw
        self.old = {}

    def __enter__(self):
        import os
        for k, v in self.kw.items():
            self.old[k] = os.environ.get(k)
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        return self

    def __exit__(self, *a):
        import os
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def steady_then_steps(ct, m, prec):
    """A steady solve, then two backward-Euler steps: iteration counts and
    fields, in order."""
    with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        res = [s.solve(1e-10, 1000).iters, s.get_x()]
        s.set_dt(1e-3)
        for _ in range(2):
            s.set_rhs_transient()
            res += [s.solve(1e-9, 1000).iters, s.get_x()]
        return res


def assert_same_results(a, b):
    for x, y in zip(a, b):
        if isinstance(x, np.ndarray):
            assert np.array_equal(x, y)
        else:
            assert x == y


def gpu_solve(ct, m, tol, pc, prec):
    with ct.GpuPcg(m, pc, prec) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        st = s.solve(tol, 50000)
        return st, s.get_x()


@pytest.mark.parametrize("name", CASES)
def test_fp64_mg_matches_oracle(ct, orc, golden, name):
    m = build_spec_model(ct, golden["cases"][name]["spec"])
    ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
    st, T = gpu_solve(ct, m, 1e-10, ct.Precond.Multigrid, ct.Precision.MG_FP64)
    assert st.converged and not st.breakdown
    assert abs(st.iters - ref.iters) <= 1
    tmax = np.abs(ref.T).max()
    assert np.abs(T - ref.T).max() <= 1e-7 * tmax
    assert orc.true_relres(m, T) <= 1e-9


@pytest.mark.parametrize("name", CASES)
def test_fp32_mg_matches_oracle(ct, orc, golden, name):
    m = build_spec_model(ct, golden["cases"][name]["spec"])
    ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=False)
    st, T = gpu_solve(ct, m, 1e-10, ct.Precond.Multigrid, ct.Precision.MG_FP32)
    assert st.converged
    assert abs(st.iters - ref.iters) <= 1
    assert np.abs(T - ref.T).max() <= 1e-7 * np.abs(ref.T).max()


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW"])
@pytest.mark.parametrize("name", CASES)
def test_fp32_flexible_within_bound_of_fp64(ct, orc, golden, name, prec):
    m = build_spec_model(ct, golden["cases"][name]["spec"])
    ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
    st, T = gpu_solve(ct, m, 1e-10, ct.Precond.Multigrid, getattr(ct.Precision, prec))
    assert st.converged
    dT = np.abs(T - ref.T).max()
    assert dT <= DT_BOUND_K
    assert dT <= 1e-7 * np.abs(ref.T).max()
    assert orc.true_relres(m, T) <= 1e-9
    # same iterates as the oracle's flexible variant
    refx = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=False, flexible=True)
    assert abs(st.iters - refx.iters) <= 1


@pytest.mark.parametrize("name", ["hotspot64", "blocks_tsv_17x13", "tiny3x5", "row1x9"])
def test_jacobi_matches_oracle(ct, orc, golden, name):
    m = build_spec_model(ct, golden["cases"][name]["spec"])
    ref = orc.solve_steady(m, 1e-6, 50000, "jacobi", mg_double=True)
    st, T = gpu_solve(ct, m, 1e-6, ct.Precond.Jacobi, ct.Precision.MG_FP64)
    assert st.converged
    assert abs(st.iters - ref.iters) <= 2
    assert np.abs(T - ref.T).max() / np.abs(ref.T).max() <= 1e-6


@pytest.mark.parametrize("name", ["hotspot64", "blocks_tsv_17x13", "blocks_tsv_40x24", "tiny3x5",
                                  "row1x9", "column1x1"])
def test_levels_and_factors_bitwise(ct, orc, golden, name):
    rec = golden["cases"][name]
    m = build_spec_model(ct, rec["spec"])
    for prec, mgd in ((ct.Precision.MG_FP64, True), (ct.Precision.MG_FP32, False)):
        o = orc.Solver(m, "multigrid", mg_double=mgd)
        with ct.GpuPcg(m, ct.Precond.Multigrid, prec) as s:
            assert s.num_levels() == len(rec["levels"])
            for dt in (0.0, 1e-4):
                s.set_dt(dt)
                o.set_dt(dt)
                for k, L in enumerate(rec["levels"]):
                    nx, ny, nz = s.level_dims(k)
                    assert (nx, ny, nz) == (L["nx"], L["ny"], m.nz)
                    op = s.level_operator(k)
                    for a in ("gE", "gN", "gU", "gB", "cap"):
                        assert sha(op[a]) == L["sha"][a], (k, a)
                    fcp, finv = s.level_factors(k)
                    ofcp, ofinv = o.level_factors(k)
                    np.testing.assert_array_equal(fcp, ofcp)
                    np.testing.assert_array_equal(finv, ofinv)


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
def test_graphs_match_direct_launches_bitwise(ct, golden, prec):
    """verify 4 (src/main3d.cu:212-222), tightened: graph replay and direct
    launches give the same bits through a transient where 1/dt changes."""
    m = build_spec_model(ct, golden["cases"]["blocks_tsv_40x24"]["spec"])
    o = ct.TransientOptions(t_end=0.02, growth=1.2, precision=getattr(ct.Precision, prec))
    a = ct.run_transient(m, o)
    ct.gpu_use_graphs(False)
    try:
        b = ct.run_transient(m, o)
    finally:
        ct.gpu_use_graphs(True)
    assert a.total_iters == b.total_iters
    np.testing.assert_array_equal(a.T, b.T)


@pytest.mark.parametrize("prec,mgd", [("MG_FP64", True), ("MG_FP32", False)])
def test_transient_matches_oracle(ct, orc, golden, prec, mgd):
    spec = dict(golden["cases"]["hotspot64"]["spec"])
    spec["nx"] = spec["ny"] = 32
    m = build_spec_model(ct, spec)
    o = ct.TransientOptions(dt0=1e-5, growth=1.2, dt_max=0.05, t_end=0.02, tol=1e-9,
                            precision=getattr(ct.Precision, prec))
    g = ct.run_transient(m, o)
    r = orc.run_transient(m, "multigrid", mg_double=mgd, dt0=1e-5, growth=1.2, dt_max=0.05,
                          t_end=0.02, tol=1e-9)
    assert len(g.steps) == len(r.steps)
    P = ct.total_power(m)
    for k, s in enumerate(g.steps):
        t, dt, it, tmax, qo, qs = r.steps[k]
        assert s.t == t and s.dt == dt
        assert abs(s.iters - it) <= 1
        assert abs(s.T_max - tmax) <= 1e-7 * tmax
        assert abs(s.q_out + s.q_stored - P) / P < 1e-6  # energy balance per step
    assert np.abs(g.T - r.T).max() <= 1e-7 * np.abs(r.T).max()


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW"])
def test_device_records_match_host_records(ct, golden, prec):
    spec = dict(golden["cases"]["hotspot64"]["spec"])
    spec["nx"] = spec["ny"] = 24
    m = build_spec_model(ct, spec)
    o = ct.TransientOptions(t_end=0.005, growth=1.3, precision=getattr(ct.Precision, prec))
    a = ct.run_transient(m, o, device_records=True)
    b = ct.run_transient(m, o, device_records=False)
    for x, y in zip(a.steps, b.steps):
        assert x.iters == y.iters
        assert x.T_max == y.T_max
        assert abs(x.q_out - y.q_out) <= 1e-12 * abs(y.q_out)
        assert abs(x.q_stored - y.q_stored) <= 1e-9 * max(1.0, abs(y.q_stored))


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW"])
def test_true_relres_on_device(ct, orc, golden, prec):
    m = build_spec_model(ct, golden["cases"]["blocks_tsv_40x24"]["spec"])
    with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        s.solve(1e-6, 100)
        T = s.get_x()
        dev = s.true_relres()
    host = orc.true_relres(m, T)
    assert abs(dev - host) <= 1e-6 * host


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW"])
def test_zero_power_gives_zero(ct, prec):
    m = ct.default_model(16, 16)
    ct.finalize(m)
    with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
        s.set_x(np.ones(m.ncells()))
        s.set_rhs_steady()
        st = s.solve(1e-10, 100)
        assert st.converged and st.iters == 0
        assert np.all(s.get_x() == 0)


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW"])
def test_power_roundtrip_and_warm_start(ct, orc, prec):
    import workloads
    m = workloads.steady_hotspot(48, seed=7)
    ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
    with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        s.solve(1e-10, 100)
        # a second solve from the converged state takes no iteration
        s.set_rhs_steady()
        st = s.solve(1e-10, 100)
        assert st.iters == 0 and st.converged
        # new power map: twice the power -> twice the temperature rise
        s.set_power(2 * m.P)
        s.set_rhs_steady()
        st = s.solve(1e-10, 100)
        assert st.converged
        T2 = s.get_x()
    assert np.abs(T2 - 2 * ref.T).max() <= 1e-7 * np.abs(ref.T).max()


def test_singular_stack_reports_status_not_hang(ct):
    """No heat sink and an adiabatic bottom: A is singular and P is not in its
    range. The solve must end with a status (not converged or breakdown)."""
    m = ct.build_model(ct.default_stack(), 12, 12, 10e-3, 10e-3, 0.0, 0.0)
    ct.add_uniform_power(m, 0, 1.0)
    ct.finalize(m)
    with ct.GpuPcg(m) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        st = s.solve(1e-12, 200)
        assert not st.converged
        assert st.iters <= 200


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
def test_nan_power_is_breakdown(ct, prec):
    m = ct.default_model(8, 8)
    ct.add_uniform_power(m, 0, 1.0)
    ct.finalize(m)
    m.P[5] = np.nan
    with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        st = s.solve(1e-10, 50)
        assert st.breakdown and not st.converged


def test_dw_true_residual_meets_tol_on_larger_grid(ct, orc):
    """The double-word mode's FP64 residual replacement: the FP64 true residual
    of a 256 x 256 solve meets tol, as the plain FP64 solve's does."""
    import workloads
    m = workloads.steady_hotspot(256, seed=3)
    for prec in (ct.Precision.MG_FP32_FLEX_DW, ct.Precision.MG_FP32_FLEX):
        st, T = gpu_solve(ct, m, 1e-10, ct.Precond.Multigrid, prec)
        assert st.converged
        assert orc.true_relres(m, T) <= 1.5e-10


@pytest.mark.parametrize("prec", ["MG_FP32", "MG_FP32_FLEX", "MG_FP32_FLEX_DW"])
def test_staged_sweeps_bitwise(ct, prec):
    """Sweeps staged in shared memory by bulk tensor copies give the grid
    sweeps' results bit for bit (odd sizes: partial tiles, padded half-rows),
    with the x = 0 sweeps of the staged levels on the grid kernel (the
    default) or staged too. CT_SWEEP_TMA_COLS=1 stages every level with a
    full tile row (by default only levels of more than 256 x 256 columns)."""
    import workloads
    m = workloads.steady_hotspot(203, seed=7)
    out = []
    for flags in ({"CT_SWEEP_TMA": "0"},
                  {"CT_SWEEP_TMA": "1", "CT_SWEEP_TMA_COLS": "1"},
                  {"CT_SWEEP_TMA": "1", "CT_SWEEP_TMA_COLS": "1", "CT_SWEEP0_GRID": "0"}):
        with env_vars(**flags):
            out.append(gpu_solve(ct, m, 1e-10, ct.Precond.Multigrid, getattr(ct.Precision, prec)))
    for o in out[1:]:
        assert o[0].iters == out[0][0].iters
        assert np.array_equal(o[1], out[0][1])


@pytest.mark.parametrize("n,prec", [(203, "MG_FP32_FLEX_DW"), (130, "MG_FP32_FLEX"), (203, "MG_FP32")])
def test_staged_sweeps_bitwise_single_and_batch(ct, n, prec, tmp_path):
    """The staged sweeps (producer warp, per-stage release barriers) give the
    grid sweeps' results bit for bit, single solver and batch (the form is
    read when a solver or batch is created: one child process each)."""
    import os
    import subprocess
    import sys
    code = ("import sys, numpy as np; sys.path[:0]=['.', 'cuda-thermal_gb300']; import cthermal as ct, "
            "workloads; m=workloads.steady_hotspot(%d, seed=3); s=ct.GpuPcg(m, ct.Precond.Multigrid, "
            "ct.Precision.%s); s.set_x_zero(); s.set_rhs_steady(); st=s.solve(1e-10, 1000); "
            "ms=[workloads.steady_hotspot(k, seed=k) for k in (96, 160, 203)]; "
            "b=ct.GpuBatch(ms); b.set_x_zero(); b.set_rhs_steady(); bs=b.solve(1e-10, 300); "
            "np.save(sys.argv[1], np.concatenate([[st.iters], s.get_x()] + "
            "[[r.iters for r in bs]] + [b.get_x(i) for i in range(len(ms))]))" % (n, prec))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = []
    for flag in ("0", "1"):
        f = str(tmp_path / f"staged_{flag}.npy")
        env = dict(os.environ, CT_SWEEP_TMA=flag, CT_SWEEP_TMA_COLS="1")
        subprocess.run([sys.executable, "-c", code, f], check=True, cwd=root, env=env, timeout=300)
        out.append(np.load(f))
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
def test_queued_transient_steps_match_blocking(ct, prec, graphs):
    """Backward-Euler steps queued on the solver's stream (ct_solve_async and
    ct_solver_step_record_async into the device table, 70 steps so the table
    grows past its first 64 entries) give the blocking steps' records,
    iteration counts and field bit for bit."""
    import workloads
    m = workloads.steady_hotspot(48, seed=11)
    ct.gpu_use_graphs(graphs)
    try:
        out = []
        for queued in (False, True):
            with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
                s.set_x_zero()
                dt, recs, sts = 1e-5, [], []
                for k in range(70):
                    s.set_dt(dt)
                    s.set_rhs_transient()
                    if queued:
                        s.solve_async(1e-9, 200)
                        s.step_record_async(dt, k)
                    else:
                        sts.append(s.solve(1e-9, 200))
                        recs.append(s.step_record(dt))
                    dt = min(dt * 1.1, 0.05)
                if queued:
                    recs, sts = s.step_records(0, 70)
                out.append(([(r.T_max, r.q_out, r.q_stored) for r in recs],
                            [(st.iters, st.converged, st.relres) for st in sts], s.get_x()))
    finally:
        ct.gpu_use_graphs(True)
    assert out[0][0] == out[1][0]
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
def test_queued_copies_match_blocking_calls(ct, prec, pinned):
    """A power-map sweep with queued copies (ct_set_power_async,
    ct_solve_async, ct_get_x_async; two staging buffers each way, so five
    steps reuse both) gives each step's field exactly as the blocking calls
    do, in pinned or pageable host memory."""
    import torch
    import workloads
    m = workloads.steady_hotspot(96, seed=5)
    n = m.ncells()

    def host(a=None):
        if pinned:
            t = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
        else:
            t = np.empty(n)
        if a is not None:
            t[:] = a
        return t

    powers = [host(m.P * f) for f in (1.0, 0.5, 2.0, 0.25, 3.0)]
    with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
        ref = []
        for P in powers:
            s.set_power(P)
            s.set_x_zero()
            s.set_rhs_steady()
            s.solve(1e-10, 200)
            ref.append(s.get_x())
        outs = [host() for _ in powers]
        for P, o in zip(powers, outs):
            s.set_power_async(P)
            s.set_x_zero()
            s.set_rhs_steady()
            s.solve_async(1e-10, 200)
            s.get_x_async(o)
        s.copies_wait()
        assert s.solve_wait().converged
        for a, b in zip(ref, outs):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", ["graph", "parts", "direct"])
@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32", "MG_FP64", "MG_FP32_FLEX_DW"])
@pytest.mark.parametrize("n,lag", [(130, "0"), (130, "1"), (130, "99"), (37, "1"), (9, "1")])
def test_lagged_x_update_bitwise(ct, prec, n, lag, mode):
    """x += alpha p run beside the next V-cycle (forked after the restriction
    out of level `lag`, the last restricted level for 99, or at the start of
    the iteration when the whole V-cycle is the shared-memory bottom, n = 9)
    and once after the loop gives the fused update's fields and iteration
    counts bit for bit: steady solve, two backward-Euler steps, and a solve
    stopped by maxit (its last update still pending when the loop ends); one
    conditional graph, part graphs polled by the host, or direct launches."""
    import workloads
    m = workloads.steady_hotspot(n, seed=23)
    ct.gpu_use_graphs(mode != "direct")
    try:
        out = []
        for flag in ("-1", lag):
            with env_vars(CT_XLAG=flag, CT_COND_GRAPHS="0" if mode == "parts" else None):
                res = steady_then_steps(ct, m, prec)
                with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
                    s.set_x_zero()
                    s.set_rhs_steady()
                    st = s.solve(1e-10, 3)
                    res += [(st.iters, st.converged), s.get_x()]
                out.append(res)
    finally:
        ct.gpu_use_graphs(True)
    assert_same_results(out[0], out[1])


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX_DW", "MG_FP32", "MG_FP64"])
@pytest.mark.parametrize("n", [203, 130, 37])
def test_fused_first_sweep_bitwise(ct, n, prec):
    """Each level's first (x = 0) sweep run inside the restriction into that
    level (the default) gives the separate launches' results bit for bit:
    steady solve, then two backward-Euler steps."""
    import workloads
    m = workloads.steady_hotspot(n, seed=13)
    out = []
    for flag in ("0", "1"):
        with env_vars(CT_FUSE_SWEEP0=flag):
            out.append(steady_then_steps(ct, m, prec))
    assert_same_results(out[0], out[1])


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
@pytest.mark.parametrize("n", [203, 130, 37])
def test_small_level_split_sweeps_bitwise(ct, n, prec):
    """Sweeps of the small grid levels with one thread per column and plane
    (the default) give the one-thread-per-column sweeps' results
    (CT_SWEEP_SPLIT=0) bit for bit: steady solve, then two backward-Euler
    steps."""
    import workloads
    m = workloads.steady_hotspot(n, seed=19)
    out = []
    for flag in ("0", None):
        with env_vars(CT_SWEEP_SPLIT=flag):
            out.append(steady_then_steps(ct, m, prec))
    assert_same_results(out[0], out[1])


@pytest.mark.parametrize("graphs", [True, False])
@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
def test_queued_solves_match_blocking_solve(ct, prec, graphs):
    """Solves queued with solve_async (x = 0 and b = P set before each) and
    one solve_wait give the blocking solve's field and statistics bit for
    bit; a queued solve with no heat in leaves x = 0; a wait with nothing
    queued is refused."""
    import workloads
    m = workloads.steady_hotspot(96, seed=31)
    pr = getattr(ct.Precision, prec)
    ct.gpu_use_graphs(graphs)
    try:
        with ct.GpuPcg(m, ct.Precond.Multigrid, pr) as s:
            s.set_x_zero()
            s.set_rhs_steady()
            ref = s.solve(1e-10, 200)
            Tref = s.get_x()
            for _ in range(3):
                s.set_x_zero()
                s.set_rhs_steady()
                s.solve_async(1e-10, 200)
            st = s.solve_wait()
            assert (st.iters, st.converged, st.relres) == (ref.iters, ref.converged, ref.relres)
            assert np.array_equal(s.get_x(), Tref)
            with pytest.raises(ct.CtError):
                s.solve_wait()
            s.set_power(np.zeros(m.ncells()))
            s.set_rhs_steady()
            s.solve_async(1e-10, 200)
            st = s.solve_wait()
            assert st.converged and not np.any(s.get_x())
    finally:
        ct.gpu_use_graphs(True)


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP32", "MG_FP64"])
@pytest.mark.parametrize("n", [203, 37])
def test_factor_levels_one_launch_bitwise(ct, n, prec):
    """set_dt with every level's factors and the FP64 diagonal in one launch
    (the default) gives the per-level launches' results (CT_FACTOR_LEVELS=0)
    bit for bit: steady solve, then two backward-Euler steps."""
    import workloads
    m = workloads.steady_hotspot(n, seed=29)
    out = []
    for flag in ("0", None):
        with env_vars(CT_FACTOR_LEVELS=flag):
            out.append(steady_then_steps(ct, m, prec))
    assert_same_results(out[0], out[1])


@pytest.mark.parametrize("cu_planes", [2, 16])
def test_small_level_split_sweeps_bitwise_deep(ct, cu_planes):
    """The same on 8- and 22-plane stacks (the 8- and 32-plane forms)."""
    m = deep_stack(ct, 90, cu_planes, ny=70)
    out = []
    for flag in ("0", None):
        with env_vars(CT_SWEEP_SPLIT=flag):
            out.append(steady_then_steps(ct, m, "MG_FP32_FLEX"))
    assert_same_results(out[0], out[1])


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX_DW", "MG_FP32", "MG_FP64"])
@pytest.mark.parametrize("n", [203, 64, 9])
def test_shared_memory_bottom_bitwise(ct, n, prec):
    """The bottom levels run by one block out of shared memory give the
    grid-wide launches' results (CT_SMALL_BYTES=0: no shared-memory bottom)
    bit for bit, with its FP32 sweeps one thread per column (the default) or
    gathering every plane's right-hand side with one task per column and
    plane before the recurrences (CT_SMALL_COL_SWEEPS=0, the FP64 form):
    steady solve, then two backward-Euler steps."""
    import workloads
    m = workloads.steady_hotspot(n, seed=17)
    out = []
    for flags in ({"CT_SMALL_BYTES": "0"}, {}, {"CT_SMALL_COL_SWEEPS": "0"}):
        with env_vars(**flags):
            out.append(steady_then_steps(ct, m, prec))
    assert_same_results(out[0], out[1])
    assert_same_results(out[0], out[2])


def test_bounded_wait_runs_out_and_context_survives(ct):
    """Failure detection without a fault: a device wait that nothing
    completes runs out after its poll limit, its kernel returns and reports
    it, and the context goes on to solve normally."""
    import workloads
    assert ct.selftest_bounded_wait(20000) is True
    m = workloads.steady_hotspot(64, seed=1)
    st, T = gpu_solve(ct, m, 1e-10, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX_DW)
    assert st.converged and np.isfinite(T).all()


@pytest.mark.parametrize("cu_planes,prec", [(16, "MG_FP32_FLEX_DW"), (16, "MG_FP32"), (34, "MG_FP32_FLEX_DW"),
                                            (34, "MG_FP64")])
def test_deep_stacks_match_oracle(ct, orc, cu_planes, prec):
    """Stacks deeper than the common ones: 22 planes (the 32-plane register
    forms of the staged sweeps, the fused restrictions and the shared-memory
    bottom) and 40 planes (past 32: the general column path, no staging),
    on a 160 x 144 grid so level 0 is staged where it can be. Against the
    FP64 oracle within 5e-4 K and 1e-7 of Tmax, FP64 true residual <= 1e-9."""
    m = deep_stack(ct, 160, cu_planes, 144)
    assert m.nz == 6 + cu_planes
    ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
    st, T = gpu_solve(ct, m, 1e-10, ct.Precond.Multigrid, getattr(ct.Precision, prec))
    assert st.converged and not st.breakdown
    tmax = np.abs(ref.T).max()
    assert np.abs(T - ref.T).max() <= min(5e-4, 1e-7 * tmax)
    assert orc.true_relres(m, T) <= 1e-9


def test_integer_conversions_equal_hardware(ct):
    """The FP64 outer kernels widen floats and narrow doubles with integer
    operations (the hardware conversions issue at the FP64 rate); on 2^24 bit
    patterns, every float exponent and doubles around the float range with
    mantissas at and beside the rounding tie included, they give the
    hardware's results bit for bit."""
    assert ct.selftest_conversions(1 << 24, seed=7) == 0


@pytest.mark.parametrize("blocks_per_sm", [1, 8])
def test_sync_cost_probe(ct, blocks_per_sm):
    """The stage-separation probe runs to completion on a full grid: both
    costs are positive and below a millisecond per phase."""
    r = ct.probe_sync_costs(500, blocks_per_sm)
    assert r["blocks"] >= 1
    assert 0 < r["grid_barrier_us"] < 1e3 and 0 < r["dependent_launch_us"] < 1e3


def test_fp64_rate_probe(ct):
    """The FP64-pipe roofline's denominator: a DFMA rate between 0.1e12 and
    1e14 per second (GB300: about 0.53e12)."""
    r = ct.probe_fp64_rate()
    assert 1e11 < r < 1e14
