"""The per-step energy balance |heat out + heat stored - P| / P of a
backward-Euler run after a power switch, and why it can exceed the
reference's 1e-6 (src/main3d.cu:172) at tol 1e-9.

The solve stops at ||r|| / ||b|| < tol with b = P + C/dt T_old
(src/transient3d.h:58-66). Right after a switch, with dt reset to 10 us, the
C/dt T_old term outweighs the power by three to four orders of magnitude
(||b|| / ||P|| ~ 6e3 here), so a residual within tol of ||b|| is up to
~tol * 6e3 of P, and the balance error follows it. It is a property of the
stopping rule, not of the arithmetic: the reference's own FP64 MG-PCG
arithmetic (the oracle) shows it, it shrinks in proportion to tol, and the
1e-6 bound holds once tol is tightened by that ratio.

CPU tests run the oracle; the GPU test runs the batched solver (FP32
V-cycle, flexible PCG) through the C ABI on the same schedule.
"""
import numpy as np
import pytest


def switching_case(ct, n=32):
    m = ct.default_model(n, n)
    ct.finalize(m)
    m.P[:] = 0.0
    ct.add_power_block(m, 0, 2e-3, 2e-3, 3e-3, 3e-3, 4.0)
    P1 = np.array(m.P)
    m.P[:] = 0.0
    ct.add_power_block(m, 2, 5e-3, 5e-3, 2e-3, 2e-3, 3.0)
    P2 = np.array(m.P)
    return m, P1, P2


def oracle_run(orc, m, P1, P2, tol, steps=40):
    """Steady with both blocks on, then block 1 off and 40 steps from dt =
    10 us growing 10 %: (worst balance, worst ||b|| / ||P||)."""
    s = orc.Solver(m, "multigrid", mg_double=True)
    s.set_power(P1 + P2)
    s.set_x_zero()
    s.set_rhs_steady()
    s.solve(1e-12, 1000)
    T = s.get_x()
    s.set_power(P2)
    ptot, dt = P2.sum(), 1e-5
    cap = np.asarray(m.cap, dtype=np.float64)
    ebs, ratio = [], 0.0
    for _ in range(steps):
        s.set_dt(dt)
        s.set_rhs_transient()
        s.solve(tol, 1000)
        Tn = s.get_x()
        ebs.append(abs(orc.heat_out(m, Tn) + orc.heat_stored(m, T, Tn, dt) - ptot) / ptot)
        ratio = max(ratio, np.linalg.norm(P2 + cap / dt * T) / np.linalg.norm(P2))
        T = Tn
        dt = min(dt * 1.1, 0.05)
    return max(ebs), ratio


def test_balance_after_a_switch_follows_the_tolerance(ct, orc):
    m, P1, P2 = switching_case(ct)
    eb9, ratio = oracle_run(orc, m, P1, P2, 1e-9)
    eb11, _ = oracle_run(orc, m, P1, P2, 1e-11)
    eb13, _ = oracle_run(orc, m, P1, P2, 1e-13)
    assert ratio > 1e3                       # C/dt T_old dominates b after the switch
    assert eb9 <= 1e-9 * ratio * 10          # within a small factor of tol * ||b|| / ||P||
    assert eb11 <= eb9 / 20 and eb13 <= eb11 / 20   # shrinks with tol
    assert eb13 < 1e-6                       # the reference's bound, with tol tightened


@pytest.mark.gpu
def test_batched_balance_after_a_switch(ct, orc):
    """The batched solver on the same schedule (one switching instance, one
    steady companion): its worst balance is within a small factor of the
    oracle's at tol 1e-9, and meets 1e-6 at tol 1e-12."""
    m, P1, P2 = switching_case(ct)
    ptot = P2.sum()
    for tol, bound in ((1e-9, None), (1e-12, 1e-6)):
        with ct.GpuBatch([m, m]) as b:
            b.set_power(0, P1 + P2)
            b.set_power(1, P1 + P2)
            b.set_x_zero()
            b.set_rhs_steady()
            b.solve(1e-12, 1000)
            b.set_power(0, P2)
            dt, worst = 1e-5, 0.0
            for _ in range(40):
                b.step_transient(np.array([dt, dt]), tol, 1000)
                rec = b.step_records(np.array([dt, dt]))
                worst = max(worst, abs(rec[0, 1] + rec[0, 2] - ptot) / ptot)
                dt = min(dt * 1.1, 0.05)
        if bound is None:
            ref, _ = oracle_run(orc, m, P1, P2, tol)
            assert worst <= 10 * ref + 1e-9, (worst, ref)
        else:
            assert worst < bound, worst
