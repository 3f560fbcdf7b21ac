"""The four-tier 1024 x 1024 x 16 stack (Si/bond tiers with 2 % copper TSV
blocks, 12 log-normal floorplan blocks per tier): the FP32 V-cycle forms
against the plain FP64 MG-PCG on the same GPU, and size-independent
properties of the steady answer.

Tolerances: max|dT| <= 5e-4 K (the stated bound) and <= 1e-7 * Tmax; FP64
true residual ||P - A T|| / ||P|| <= 1e-9 at tol 1e-10; steady energy
balance |heat out - power| / power <= 1e-8 (heat out = the sink and bottom
faces' flux, src/stack3d.h:252-262).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def four(ct):
    import workloads
    return workloads.four_tier(1024, seed=3)


def solve(ct, m, prec):
    with ct.GpuPcg(m, ct.Precond.Multigrid, prec) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        st = s.solve(1e-10, 50000)
        return st, s.get_x(), s.true_relres()


def test_four_tier_fp32_forms_match_fp64(ct, four):
    st64, T64, rel64 = solve(ct, four, ct.Precision.MG_FP64)
    assert st64.converged and rel64 <= 1e-9
    tmax = T64.max()
    for prec in (ct.Precision.MG_FP32_FLEX, ct.Precision.MG_FP32_FLEX_DW):
        st, T, rel = solve(ct, four, prec)
        assert st.converged, prec
        assert abs(st.iters - st64.iters) <= 2
        dT = np.abs(T - T64).max()
        assert dT <= 5e-4 and dT <= 1e-7 * tmax, (prec, dT, tmax)
        assert rel <= 1e-9, (prec, rel)
        # steady state: all the power leaves through the sink and bottom faces
        P = ct.total_power(four)
        assert abs(ct.heat_out(four, T) - P) / P <= 1e-8
