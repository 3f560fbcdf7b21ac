"""Field products on the device (ct_colorize, ct_block_temps) against numpy
restatements of the reference's k_colorize (src/viewer.cu:52-87),
block_temps (src/main3d.cu:286-300) and for_each_overlap
(src/stack3d.h:175-191), on a solved example case.

Tolerances: the per-column maximum map and the hottest cell exactly; RGBA
within one unit per channel (the colour scale's last rounding); block
maximum exactly, area-weighted mean to 1e-12 relative (summation order)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR

pytestmark = pytest.mark.gpu

STOPS = np.array([[0, 0, 4], [87, 16, 110], [188, 55, 84], [249, 142, 9], [252, 255, 164]], np.float64)


def colour_ref(v, rise_hi):
    s = np.clip((v / np.float32(rise_hi)).astype(np.float32), 0, 1)
    f = (s * np.float32(4)).astype(np.float32)
    k = np.minimum(f.astype(np.int32), 3)
    f = (f - k).astype(np.float32)
    out = np.empty(v.shape + (4,), np.int64)
    for ch in range(3):
        a, b = STOPS[k, ch], STOPS[k + 1, ch]
        out[..., ch] = np.floor((a + f.astype(np.float64) * (b - a)).astype(np.float32))
    out[..., 3] = 255
    return out


def overlap(a0, a1, b0, b1):
    return max(0.0, min(a1, b1) - max(a0, b0))


def block_ref(m, T, l0, l1, x0, y0, w, h):
    import math
    i0, i1 = max(0, math.floor(x0 / m.dx)), min(m.nx - 1, math.ceil((x0 + w) / m.dx))
    j0, j1 = max(0, math.floor(y0 / m.dy)), min(m.ny - 1, math.ceil((y0 + h) / m.dy))
    tmax, s, ws = -1e30, 0.0, 0.0
    for l in range(l0, l1 + 1):
        for j in range(j0, j1 + 1):
            for i in range(i0, i1 + 1):
                a = overlap(i * m.dx, (i + 1) * m.dx, x0, x0 + w) * overlap(j * m.dy, (j + 1) * m.dy, y0, y0 + h)
                if a > 1e-9 * m.dx * m.dy:
                    t = T[m.idx(i, j, l)]
                    tmax = max(tmax, t)
                    s += a / (m.dx * m.dy) * t
                    ws += a / (m.dx * m.dy)
    return tmax, s / ws


@pytest.fixture(scope="module")
def solved(ct):
    cs = ct.load_case(os.path.join(GOLDEN_DIR, "cases", "example"))
    m = ct.build_case_model(cs, 48, 40, True)
    s = ct.GpuPcg(m, ct.Precond.Multigrid, ct.Precision.MG_FP32_FLEX_DW)
    s.set_x_zero()
    s.set_rhs_steady()
    assert s.solve(1e-10, 1000).converged
    yield cs, m, s, s.get_x()
    s.close()


def test_colorize_matches_reference(ct, solved, tmp_path):
    cs, m, s, T = solved
    for layer in range(len(m.layers)):
        l0, l1 = ct.layer_planes(m, layer)
        rise_hi = float(T.max()) * 1.1
        rgba, mp, mx, i, j = s.colorize(l0, l1, rise_hi)
        T3 = T.reshape(m.nz, m.ny, m.nx)
        ref = np.maximum(0.0, T3[l0:l1 + 1].astype(np.float32).max(axis=0))
        assert np.array_equal(mp, ref)
        assert np.abs(rgba.astype(np.int64) - colour_ref(ref, rise_hi)).max() <= 1
        key = (ref.view(np.uint32).astype(np.uint64) << np.uint64(32)) | np.arange(m.nx * m.ny, dtype=np.uint64).reshape(m.ny, m.nx)
        q = int(key.max() & np.uint64(0xffffffff))
        assert (i, j) == (q % m.nx, q // m.nx) and mx == float(ref.max())
    ct.write_ppm(str(tmp_path / "die.ppm"), rgba)
    ct.write_tmap(str(tmp_path / "tmap.csv"), m, mp)
    header = b"P6 %d %d 255\n" % (m.nx, m.ny)
    assert (tmp_path / "die.ppm").stat().st_size == len(header) + 3 * m.nx * m.ny
    rows = (tmp_path / "tmap.csv").read_text().splitlines()
    assert len(rows) == m.ny and len(rows[0].split(",")) == m.nx


def test_block_temps_match_reference(ct, solved):
    cs, m, s, T = solved
    for b in cs.blocks:
        l0, l1 = ct.layer_planes(m, b.layer)
        tmax, tavg = s.block_temps(l0, l1, b.x0, b.y0, b.w, b.h)
        rmax, ravg = block_ref(m, T, l0, l1, b.x0, b.y0, b.w, b.h)
        assert tmax == rmax
        assert abs(tavg - ravg) <= 1e-12 * abs(ravg)
