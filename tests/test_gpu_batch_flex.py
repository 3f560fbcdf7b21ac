"""The batched solver with its outer iteration in FP64 (ct_batch_create_prec
with CT_MG_FP32_FLEX), against the oracle and the single solver in the same
precision, through the C ABI.

Tolerances (written here, used below):
  * every instance of a steady batch vs the FP64 oracle: max|dT| <= 5e-4 K and
    <= 1e-7 * Tmax, FP64 true residual <= 1e-9 for solves to 1e-10;
  * vs the single CT_MG_FP32_FLEX solver: iteration counts within 1 (the
    per-instance reductions group the same FP64 products differently),
    max|dT| <= 1e-7 * Tmax;
  * the batch through its graphs and through direct launches: bit-identical;
  * backward-Euler steps with per-instance dt and a power change: the single
    solver's iteration counts within 1 and fields within 1e-7 * Tmax;
  * a zero-power instance solves to T = 0 beside the others.
"""
import numpy as np
import pytest

from conftest import build_spec_model

pytestmark = pytest.mark.gpu


def mixed_models(ct, golden):
    import workloads
    rng = np.random.default_rng(23)
    ms = [workloads.batch_instance(rng) for _ in range(4)]
    for name in ("hotspot64", "blocks_tsv_17x13", "column1x1", "row1x9", "tiny3x5"):
        ms.append(build_spec_model(ct, golden["cases"][name]["spec"]))
    return ms


@pytest.fixture(scope="module")
def mixed(ct, golden):
    return mixed_models(ct, golden)


def single(ct, m):
    s = ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX)
    s.set_x_zero()
    s.set_rhs_steady()
    st = s.solve(1e-10, 50000)
    return s, st


def test_flex_batch_steady_matches_oracle_and_single(ct, orc, mixed):
    with ct.GpuBatch(mixed, precision=ct.Precision.MG_FP32_FLEX) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        stats = b.solve(1e-10, 50000)
        for i, m in enumerate(mixed):
            st = stats[i]
            assert st.converged and not st.breakdown, (i, st)
            T = b.get_x(i)
            ref = orc.solve_steady(m, 1e-10, 50000, "multigrid", mg_double=True)
            tmax = np.abs(ref.T).max()
            dT = float(np.abs(T - ref.T).max())
            assert dT <= 5e-4 and dT <= 1e-7 * tmax, (i, dT, tmax)
            assert orc.true_relres(m, T) <= 1e-9
            s, s1 = single(ct, m)
            T1 = s.get_x()
            s.close()
            assert abs(st.iters - s1.iters) <= 1, (i, st.iters, s1.iters)
            assert np.abs(T - T1).max() <= 1e-7 * tmax


def test_flex_batch_graph_and_direct_bitwise(ct, mixed):
    import os
    out = []
    for flag in (None, "0"):
        old = os.environ.get("CT_COND_GRAPHS")
        if flag is None:
            os.environ.pop("CT_COND_GRAPHS", None)
        else:
            os.environ["CT_COND_GRAPHS"] = flag
        try:
            with ct.GpuBatch(mixed, precision=ct.Precision.MG_FP32_FLEX) as b:
                b.set_x_zero()
                b.set_rhs_steady()
                st = b.solve(1e-10, 50000)
                out.append(([s.iters for s in st], [b.get_x(i) for i in range(len(mixed))]))
        finally:
            if old is None:
                os.environ.pop("CT_COND_GRAPHS", None)
            else:
                os.environ["CT_COND_GRAPHS"] = old
    assert out[0][0] == out[1][0]
    for a, c in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, c)


def test_flex_batch_transient_matches_single(ct, golden):
    import workloads
    rng = np.random.default_rng(29)
    ms = [workloads.batch_instance(rng) for _ in range(2)]
    ms.append(build_spec_model(ct, golden["cases"]["blocks_tsv_17x13"]["spec"]))
    n = len(ms)
    dts = np.array([2e-5, 1e-4, 1e-3][:n])
    singles = [single(ct, m)[0] for m in ms]
    with ct.GpuBatch(ms, precision=ct.Precision.MG_FP32_FLEX) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        assert all(s.converged for s in b.solve(1e-10, 50000))
        for step in range(4):
            if step == 2:
                for i, m in enumerate(ms):
                    P = m.P * (0.5 + 0.25 * i)
                    b.set_power(i, P)
                    singles[i].set_power(P)
            dt = dts * (1.1 ** step)
            stats = b.step_transient(dt, 1e-9, 50000)
            for i in range(n):
                s = singles[i]
                s.set_dt(dt[i])
                s.set_rhs_transient()
                st1 = s.solve(1e-9, 50000)
                assert stats[i].converged
                assert abs(stats[i].iters - st1.iters) <= 1, (step, i, stats[i], st1)
                T, T1 = b.get_x(i), s.get_x()
                assert np.abs(T - T1).max() <= 1e-7 * np.abs(T1).max()
    for s in singles:
        s.close()


def test_flex_batch_zero_power_instance(ct, golden):
    m = build_spec_model(ct, golden["cases"]["hotspot64"]["spec"])
    z = build_spec_model(ct, golden["cases"]["hotspot64"]["spec"])
    z.P[:] = 0.0
    with ct.GpuBatch([m, z], precision=ct.Precision.MG_FP32_FLEX) as b:
        b.set_x_zero()
        b.set_rhs_steady()
        st = b.solve(1e-10, 50000)
        assert st[0].converged and st[1].converged
        assert not np.any(b.get_x(1))
        assert np.abs(b.get_x(0)).max() > 1.0


def test_batch_rejects_other_precisions(ct, mixed):
    with pytest.raises(ct.CtError) as e:
        ct.GpuBatch(mixed[:2], precision=ct.Precision.MG_FP64)
    assert e.value.status == 5
