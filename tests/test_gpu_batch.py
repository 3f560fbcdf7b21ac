"""Batched solver (ct_batch_*) against the oracle and the single solver,
through the C ABI.

Tolerances (written here, used below):
  * every instance of a steady batch vs the FP64 oracle: max|dT| <= 1e-7 * Tmax
    (far inside the stated 5e-4 K bound, also asserted) and FP64 true residual
    <= 1.5e-10 for solves to 1e-10;
  * vs the single solver in the same precision (CT_MG_FP32_FLEX_DW): iteration
    counts within 1 (the per-instance reductions add the same values in a
    different grouping);
  * a batch run through graphs and the same batch run through direct launches
    (fixed tiles): bit-identical;
  * batched backward-Euler steps vs the single solver's steps: max|dT| <=
    1e-7 * Tmax, the same step records within 1e-7, energy balance per step
    within 1e-5 of the power (the step just after a power switch, solved to
    1e-9 of ||P + C/dt T||, balances to about 1e-6).
"""
import os

import numpy as np
import pytest

from conftest import build_spec_model

pytestmark = pytest.mark.gpu

DT_BOUND_K = 5e-4


def mixed_models(ct, golden):
    """Uneven stacks: random floorplan stacks of the batched workload's kind,
    plus golden cases of odd shapes (a single column, a single row, a tiny
    grid)."""
    import workloads
    rng = np.random.default_rng(11)
    ms = []
    for _ in range(5):
        m = workloads.batch_instance(rng)
        ms.append(m)
    for name in ("hotspot64", "blocks_tsv_17x13", "column1x1", "row1x9", "tiny3x5"):
        ms.append(build_spec_model(ct, golden["cases"][name]["spec"]))
    return ms


def single_solve(ct, m, tol):
    with ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX_DW) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        st = s.solve(tol, 50000)
        return st, s.get_x()


@pytest.fixture(scope="module")
def mixed(ct, golden):
    return mixed_models(ct, golden)


def test_batch_steady_matches_oracle_and_single(ct, orc, mixed):
    with ct.GpuBatch(mixed) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        stats = b.solve(1e-10, 50000)
        for i, m in enumerate(mixed):
            st = stats[i]
            assert st.converged and not st.breakdown, (i, st)
            T = b.get_x(i)
            ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
            tmax = np.abs(ref.T).max()
            dT = np.abs(T - ref.T).max()
            assert dT <= DT_BOUND_K
            assert dT <= 1e-7 * tmax, (i, dT, tmax)
            assert orc.true_relres(m, T) <= 1.5e-10
            s1, T1 = single_solve(ct, m, 1e-10)
            assert abs(st.iters - s1.iters) <= 1, (i, st.iters, s1.iters)
            assert np.abs(T - T1).max() <= 1e-7 * tmax


def test_batch_buckets_cover_instances(ct, mixed):
    """Buckets cover every instance once; the tiles are candidates of the
    tuner. Where the staged form is not forced, the tuner keeps it only where
    it timed faster than the grid sweep; with a fixed number of tiles per
    block (CT_BATCH_TMA_TILES) every level that holds a full tile row is
    staged."""
    for forced in (None, "2"):
        old = _env(CT_BATCH_TMA_TILES=forced) if forced else {}
        try:
            with ct.GpuBatch(mixed) as b:
                info = b.buckets()
                assert sum(k["instances"] for k in info) == len(mixed)
                for k in info:
                    assert len(k["sweep_tiles"]) == k["depth"] == len(k["staged"])
                    for t, staged in zip(k["sweep_tiles"], k["staged"]):
                        assert t in ((1, 2, 4, 8) if staged else (256, 512, 1024, 2048))
                    assert all(t in (256, 512, 1024, 2048, 4096) for t in k["restrict_tiles"])
                if forced:
                    # the large levels of the workload's stacks are staged
                    assert any(any(k["staged"]) for k in info)
                    assert all(t == 2 for k in info for t, st in zip(k["sweep_tiles"], k["staged"]) if st)
        finally:
            _restore(old)


def test_batch_resolve_and_power_change(ct, orc, mixed):
    """Two solves in a row with a power map changed in between: the second
    solve sees the new map, the other instances are unchanged."""
    with ct.GpuBatch(mixed) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        b.solve(1e-10, 50000)
        first = [b.get_x(i) for i in range(len(mixed))]
        m0 = mixed[0]
        P2 = m0.P * 2.0
        b.set_power(0, P2)
        b.set_x_zero()
        b.set_rhs_steady()
        stats = b.solve(1e-10, 50000)
        assert all(s.converged for s in stats)
        T0 = b.get_x(0)
        # linear in P with T measured above ambient 0
        assert np.abs(T0 - 2.0 * first[0]).max() <= 1e-7 * np.abs(T0).max()
        for i in range(1, len(mixed)):
            assert np.abs(b.get_x(i) - first[i]).max() <= 1e-9 * np.abs(first[i]).max()
        b.set_power(0, m0.P)


def test_batch_zero_power_instance(ct, golden):
    """An instance with no heat converges at once with T = 0 (the reference's
    bb = 0 exit, src/pcg3d_cpu.cpp:146) and leaves the others alone."""
    m = build_spec_model(ct, golden["cases"]["hotspot64"]["spec"])
    z = build_spec_model(ct, golden["cases"]["hotspot64"]["spec"])
    z.P[:] = 0.0
    with ct.GpuBatch([m, z, m]) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        stats = b.solve(1e-10, 50000)
        assert stats[1].converged and stats[1].iters == 0
        assert not b.get_x(1).any()
        assert stats[0].iters == stats[2].iters > 0
        assert np.array_equal(b.get_x(0), b.get_x(2))


def test_batch_not_converged_reports(ct, mixed):
    with ct.GpuBatch(mixed[:3]) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        stats = b.solve(1e-14, 2)
        assert all(s.iters <= 2 for s in stats)
        assert not all(s.converged for s in stats)


def test_batch_graph_and_direct_bitwise(ct, mixed):
    old = {k: os.environ.get(k) for k in ("CT_BATCH_TILE", "CT_COND_GRAPHS")}
    try:
        os.environ["CT_BATCH_TILE"] = "512"
        out = []
        for cond in ("1", "0"):
            os.environ["CT_COND_GRAPHS"] = cond
            with ct.GpuBatch(mixed) as b:
                b.set_x_zero()
                b.set_rhs_steady()
                st = b.solve(1e-10, 50000)
                out.append(([s.iters for s in st], [b.get_x(i) for i in range(len(mixed))]))
        assert out[0][0] == out[1][0]
        for a, c in zip(out[0][1], out[1][1]):
            assert np.array_equal(a, c)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def test_batch_transient_matches_single(ct, golden):
    """Backward-Euler steps with a different dt per instance, warm-started
    from the steady field: the batch's steps equal the single solver's."""
    import workloads
    rng = np.random.default_rng(5)
    ms = [workloads.batch_instance(rng) for _ in range(3)]
    ms.append(build_spec_model(ct, golden["cases"]["blocks_tsv_17x13"]["spec"]))
    n = len(ms)
    dts = np.array([1e-5, 3e-5, 2e-4, 1e-3][:n])
    singles = []
    for m in ms:
        s = ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX_DW)
        s.set_x_zero()
        s.set_rhs_steady()
        s.solve(1e-10, 50000)
        singles.append(s)
    powers = [ct.total_power(m) for m in ms]
    with ct.GpuBatch(ms) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        st0 = b.solve(1e-10, 50000)
        for i in range(n):
            assert st0[i].converged
            assert b.true_relres(i) <= 1.5e-10, (i, st0[i], b.true_relres(i))
        for step in range(4):
            # change the power halfway (a switching schedule's event)
            if step == 2:
                for i, m in enumerate(ms):
                    P = m.P * (0.5 + 0.25 * i)
                    b.set_power(i, P)
                    singles[i].set_power(P)
                    powers[i] = float(np.sum(P))
            dt = dts * (1.1 ** step)
            stats = b.step_transient(dt, 1e-9, 50000)
            all_rec = b.step_records(dt)  # one launch for every instance
            for i, m in enumerate(ms):
                s = singles[i]
                s.set_dt(dt[i])
                s.set_rhs_transient()
                st1 = s.solve(1e-9, 50000)
                assert stats[i].converged
                T, T1 = b.get_x(i), s.get_x()
                assert abs(stats[i].iters - st1.iters) <= 1, (step, i, stats[i], st1, b.true_relres(i))
                assert np.abs(T - T1).max() <= 1e-7 * np.abs(T1).max()
                r, r1 = b.step_record(i, dt[i]), s.step_record(dt[i])
                # same sums, grouped per block differently: equal to ~1e-12
                assert all_rec[i][0] == r.T_max
                assert abs(all_rec[i][1] - r.q_out) <= 1e-12 * abs(r.q_out)
                assert abs(all_rec[i][2] - r.q_stored) <= 1e-12 * max(abs(r.q_stored), powers[i])
                assert abs(r.q_out - r1.q_out) <= 1e-7 * abs(r1.q_out)
                assert abs(r.q_stored - r1.q_stored) <= 1e-7 * max(abs(r1.q_stored), powers[i])
                # energy balance: tol 1e-9 is relative to ||P + C/dt T||, so the
                # balance holds to about 1e-6 of the power right after a switch
                assert abs(r.q_out + r.q_stored - powers[i]) / powers[i] < 1e-5
    for s in singles:
        s.close()


def _env(**kv):
    old = {k: os.environ.get(k) for k in kv}
    for k, v in kv.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v
    return old


def _restore(old):
    for k, v in old.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v


def test_batch_staged_sweeps_bitwise(ct, mixed):
    """The sweeps staged by bulk tensor copies (forced on every level that
    holds a full tile row; mixed depths run the rest on the grid kernel)
    compute exactly what the grid sweeps compute: same iterations, same
    bits; and so do the x = 0 sweeps on the grid kernel beside staged
    others (CT_SWEEP0_GRID=1)."""
    out = []
    for flag, grid0 in (("0", None), ("1", None), ("1", "1")):
        old = _env(CT_SWEEP_TMA=flag, CT_BATCH_TMA_TILES="1", CT_SWEEP0_GRID=grid0)
        try:
            with ct.GpuBatch(mixed) as b:
                b.set_x_zero()
                b.set_rhs_steady()
                st = b.solve(1e-10, 50000)
                out.append(([s.iters for s in st], [b.get_x(i) for i in range(len(mixed))]))
        finally:
            _restore(old)
    for o in out[1:]:
        assert o[0] == out[0][0]
        for a, c in zip(out[0][1], o[1]):
            assert np.array_equal(a, c)


def test_batch_from_device_built_specs_bitwise(ct):
    """A batch whose models are built on the device from case descriptions
    (ct_batch_create_cases) solves exactly as the batch of host-built models."""
    import workloads
    specs = workloads.batch_instance_specs(6, seed=21)
    models = [ct.build_case_model(cs, nx, ny, False) for cs, nx, ny in specs]
    out = []
    for make in (lambda: ct.GpuBatch(models),
                 lambda: ct.GpuBatch.from_specs([s[0] for s in specs], [s[1] for s in specs],
                                                [s[2] for s in specs], False)):
        with make() as b:
            b.set_x_zero()
            b.set_rhs_steady()
            st = b.solve(1e-10, 1000)
            out.append(([s.iters for s in st], [b.get_x(i) for i in range(len(specs))]))
    assert out[0][0] == out[1][0]
    for a, c in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, c)


def test_batch_deep_stacks_match_oracle(ct, orc):
    """A batch mixing deep stacks (22 and 40 planes) with a common one:
    every instance within 1e-7 * Tmax of the FP64 oracle, staged sweeps
    forced where a level holds a full tile row."""
    def stack(cu_planes, nx, ny):
        layers = [ct.Layer("Si tier 2 (bottom)", 50e-6, 130.0, 1.66e6, 2, True),
                  ct.Layer("bond + BEOL", 10e-6, 2.0, 1.70e6, 1, False),
                  ct.Layer("Si tier 1 (top)", 50e-6, 130.0, 1.66e6, 2, True),
                  ct.Layer("TIM", 25e-6, 5.0, 2.00e6, 1, False),
                  ct.Layer("Cu spreader", 1e-3, 400.0, 3.45e6, cu_planes, False)]
        m = ct.build_model(layers, nx, ny, 10e-3, 8e-3, 2e4, 0.0)
        ct.add_uniform_power(m, 0, 20.0)
        ct.add_hotspot(m, 0, 3e-3, 4e-3, 1e-3, 3.0)
        ct.add_uniform_power(m, 2, 15.0)
        ct.finalize(m)
        return m
    ms = [stack(16, 128, 96), stack(34, 96, 80), stack(4, 160, 128)]
    old = _env(CT_BATCH_TMA_TILES="1")
    try:
        with ct.GpuBatch(ms) as b:
            b.set_x_zero()
            b.set_rhs_steady()
            st = b.solve(1e-10, 50000)
            for i, m in enumerate(ms):
                assert st[i].converged and not st[i].breakdown, (i, st[i])
                ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
                T = b.get_x(i)
                tmax = np.abs(ref.T).max()
                assert np.abs(T - ref.T).max() <= min(DT_BOUND_K, 1e-7 * tmax), i
                assert b.true_relres(i) <= 1.5e-10, i
    finally:
        _restore(old)


def test_batch_power_from_device_memory(ct, mixed):
    """ct_batch_set_power_device: power maps handed over in device memory
    give the host-array path's results bit for bit."""
    import torch
    out = []
    for dev in (False, True):
        with ct.GpuBatch(mixed) as b:
            keep = []
            for i, m in enumerate(mixed):
                P = np.asarray(m.P, np.float64) * 1.25
                if dev:
                    t = torch.from_numpy(P).cuda()
                    keep.append(t)
                    torch.cuda.synchronize()
                    b.set_power_device(i, t.data_ptr())
                else:
                    b.set_power(i, P)
            b.set_x_zero()
            b.set_rhs_steady()
            st = b.solve(1e-10, 50000)
            out.append(([s.iters for s in st], [b.get_x(i) for i in range(len(mixed))]))
    assert out[0][0] == out[1][0]
    for a, c in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, c)
