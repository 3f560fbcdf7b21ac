"""GPU parity against the oracle at the benchmark's own sizes, and the
reference's published and exact answers, through the C ABI.

* 800 x 800 x 10 (the steady benchmark: default stack, 25 W per Si tier + a
  seeded 3 W, 1 mm hotspot) and 1024 x 1024 x 16 (four Si/bond tiers with 2 %
  copper TSV blocks, log-normal floorplans): every precision mode against the
  oracle's plain FP64 MG-PCG (the reference CPU solver's -DMG_DOUBLE
  arithmetic, itself pinned bit for bit to the compiled reference).
  Tolerances: max|dT| <= 5e-4 K (the stated bound) and <= 1e-7 * Tmax;
  iteration counts within 1 of the oracle's; the FP64 true residual
  ||P - A T|| / ||P||, recomputed by the oracle, <= 1e-9 at tol 1e-10.
* The reference's grid-convergence answer (README "Grid convergence"):
  hotspot_model (src/main3d.cu:60-67) has a bottom-tier peak that prints as
  79.80 / 79.81 / 79.82 C at 200 / 400 / 800 cells (%.2f, as print_layers,
  src/main3d.cu:77-92, prints it): the peak must lie in [v - 0.005, v + 0.005).
* Uniform power (25 W per Si tier, no TSVs, adiabatic bottom): every column
  is the 1D resistor chain of analytic_1d (src/stack3d.h:279-297), computed in
  FP64 from the layer data, independently of the float operator. Bound:
  max|T - T_1d| <= 1e-6 * max T_1d (the reference's own check is 1e-4,
  src/main3d.cu:97-125; the float operator's rounding is ~1e-7 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRECISIONS = ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64", "MG_FP32"]


def solve(ct, m, prec, tol=1e-10):
    with ct.GpuPcg(m, ct.Precond.Multigrid, getattr(ct.Precision, prec)) as s:
        s.set_x_zero()
        s.set_rhs_steady()
        st = s.solve(tol, 1000)
        return st, s.get_x()


def check_against_oracle(orc, m, ref, st, T, prec):
    assert st.converged and not st.breakdown, prec
    assert abs(st.iters - ref.iters) <= 1, (prec, st.iters, ref.iters)
    tmax = np.abs(ref.T).max()
    dT = float(np.abs(T - ref.T).max())
    assert dT <= 5e-4 and dT <= 1e-7 * tmax, (prec, dT, tmax)
    rel = orc.true_relres(m, T)
    assert rel <= 1e-9, (prec, rel)


@pytest.fixture(scope="module")
def c800(ct, orc):
    import workloads
    m = workloads.steady_hotspot(800, seed=2)
    ref = orc.solve_steady(m, 1e-10, 1000, "multigrid", mg_double=True)
    assert ref.converged
    return m, ref


@pytest.mark.parametrize("prec", PRECISIONS)
def test_800x800x10_matches_oracle(ct, orc, c800, prec):
    m, ref = c800
    st, T = solve(ct, m, prec)
    check_against_oracle(orc, m, ref, st, T, prec)


@pytest.fixture(scope="module")
def c1024(ct, orc):
    import workloads
    m = workloads.four_tier(1024, seed=3)
    ref = orc.solve_steady(m, 1e-10, 1000, "multigrid", mg_double=True)
    assert ref.converged
    return m, ref


@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
def test_1024x1024x16_four_tier_matches_oracle(ct, orc, c1024, prec):
    m, ref = c1024
    st, T = solve(ct, m, prec)
    check_against_oracle(orc, m, ref, st, T, prec)


def hotspot_model(ct, n):
    """hotspot_model (src/main3d.cu:60-67)."""
    m = ct.default_model(n, n)
    ct.add_uniform_power(m, 0, 22.0)
    ct.add_hotspot(m, 0, 3e-3, 3e-3, 1e-3, 3.0)
    ct.add_uniform_power(m, 2, 25.0)
    ct.finalize(m)
    return m


@pytest.mark.parametrize("n,printed", [(200, 79.80), (400, 79.81), (800, 79.82)])
@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP64"])
def test_published_bottom_tier_peak(ct, n, printed, prec):
    m = hotspot_model(ct, n)
    st, T = solve(ct, m, prec)
    assert st.converged
    planes = np.asarray(m.plane_layer) == 0  # the bottom Si tier's planes
    peak = float(T.reshape(m.nz, -1)[planes].max()) + 25.0  # T_amb = 25 C
    assert printed - 0.005 <= peak < printed + 0.005, (n, prec, peak)


@pytest.mark.parametrize("n", [64, 256])
@pytest.mark.parametrize("prec", ["MG_FP32_FLEX", "MG_FP32_FLEX_DW", "MG_FP64"])
def test_uniform_power_equals_1d_chain(ct, n, prec):
    import workloads
    m = workloads.uniform_power(n)
    st, T = solve(ct, m, prec)
    assert st.converged
    Tz = ct.analytic_1d(m)
    err = float(np.abs(T.reshape(m.nz, -1) - Tz[:, None]).max())
    assert err <= 1e-6 * Tz.max(), (n, prec, err, Tz.max())
