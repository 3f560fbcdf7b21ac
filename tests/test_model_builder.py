"""The library's model builder (stack3d.h restated in model.cpp, called through
the C ABI) reproduces the reference's Model3D arrays bit for bit, and keeps
its invariants: power conserved for blocks off the cell edges, TSV fractions
capped at 1, adiabatic sides, the 1D chain."""
import hashlib

import numpy as np
import pytest

from conftest import build_spec_model


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["hotspot64", "uniform64", "blocks_tsv_17x13", "blocks_tsv_40x24",
                                  "tiny3x5", "column1x1", "row1x9", "tsv_layer64",
                                  "base3dice_50"])
def test_model_arrays_bitwise(ct, golden, name):
    rec = golden["cases"][name]
    m = build_spec_model(ct, rec["spec"])
    assert m.nz == rec["nz"]
    assert m.dx == rec["dx"] and m.dy == rec["dy"]
    for k, h in rec["model_sha"].items():
        assert sha(getattr(m, k)) == h, k
    assert ct.total_power(m) == rec["total_power"]
    np.testing.assert_array_equal(ct.analytic_1d(m), np.array(rec["analytic_1d"]))


def test_power_block_conservation(ct):
    """verify 5 (src/main3d.cu:232-241): blocks moved off the cell edges keep
    their exact total."""
    m = ct.default_model(64, 64)
    want = 0.0
    for (layer, x0, y0, w, h, watts) in [(0, 0.5e-3, 0.5e-3, 2e-3, 2e-3, 6.0),
                                         (0, 5.5e-3, 0.5e-3, 4e-3, 4.5e-3, 3.0),
                                         (2, 0.0, 0.0, 10e-3, 10e-3, 12.0),
                                         (2, 4e-3, 4e-3, 2e-3, 2e-3, 3.0)]:
        sx = 0.037e-3 if x0 + w + 0.037e-3 <= m.Lx else 0.0
        sy = 0.011e-3 if y0 + h + 0.011e-3 <= m.Ly else 0.0
        ct.add_power_block(m, layer, x0 + sx, y0 + sy, w, h, watts)
        want += watts
    assert abs(ct.total_power(m) - want) / want < 1e-12


def test_tsv_fraction_capped(ct):
    m = ct.default_model(8, 8)
    ct.add_tsv_region(m, 1, 0, 0, 10e-3, 10e-3, 0.7)
    ct.add_tsv_region(m, 1, 0, 0, 10e-3, 10e-3, 0.7)
    assert m.tsv_frac.max() == 1.0
    assert not m.finalized
    ct.finalize(m)
    assert m.finalized


def test_boundary_faces(ct):
    m = ct.default_model(5, 4)
    ct.finalize(m)
    gE = m.gE.reshape(m.nz, m.ny, m.nx)
    gN = m.gN.reshape(m.nz, m.ny, m.nx)
    assert np.all(gE[:, :, -1] == 0) and np.all(gE[:, :, :-1] > 0)
    assert np.all(gN[:, -1, :] == 0) and np.all(gN[:, :-1, :] > 0)
    assert np.all(m.gB == 0)  # adiabatic bottom (h_bot = 0)


def test_errors_are_status_codes(ct):
    too_deep = [ct.Layer("x", 1e-3, 1.0, 1.0, 40, False), ct.Layer("y", 1e-3, 1.0, 1.0, 40, False)]
    with pytest.raises(ct.CtError) as e:
        ct.build_model(too_deep, 4, 4, 1e-3, 1e-3, 1e4, 0)
    assert e.value.status == 5
    m = ct.default_model(4, 4)
    with pytest.raises(ct.CtError):
        ct.add_hotspot(m, 0, 50e-3, 50e-3, 1e-6, 1.0)  # covers no cell
