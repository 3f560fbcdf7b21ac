"""Case loader (load_case / build_case_model, src/case3d.h:84-166) against
the reference's own loader: the four example cases (tests/golden/cases, the
reference's CSV inputs) built on a 40 x 40 grid with and without TSVs give
the same model arrays bit for bit (SHA-256 from the reference, golden.json)
and the same total power; malformed cases fail with the reference's checks.
The GPU test solves each case and matches the reference's FP64 result."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR

CASES = ["example", "tsv_under_core0", "validate_3dice", "validate_tsv"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def case_dir(name):
    return os.path.join(GOLDEN_DIR, "cases", name)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("with_tsv", [True, False])
def test_case_model_matches_reference(ct, golden, name, with_tsv):
    ref = golden["case_files"][f"{name}_{int(with_tsv)}"]
    cs = ct.load_case(case_dir(name))
    m = ct.build_case_model(cs, 40, 40, with_tsv)
    assert m.nz == ref["nz"]
    for k, h in ref["model_sha"].items():
        assert sha(getattr(m, k)) == h, k
    assert ct.total_power(m) == ref["total_power"]


def test_case_settings_and_names(ct):
    cs = ct.load_case(case_dir("example"))
    assert cs.Lx == pytest.approx(10e-3) and cs.Ly == pytest.approx(10e-3)
    assert cs.h_top == 2e4 and cs.h_bot == 0.0 and cs.T_amb == 25.0
    assert [L.name for L in cs.layers][0] == "Si tier 2 (bottom)"
    assert all(cs.layers[b.layer].active for b in cs.blocks)
    assert len(cs.tsvs) > 0


def write_case(tmp_path, stack, floorplan, tsv=None):
    d = tmp_path / "case"
    d.mkdir(exist_ok=True)
    (d / "stack.csv").write_text(stack)
    (d / "floorplan.csv").write_text(floorplan)
    if tsv is not None:
        (d / "tsv.csv").write_text(tsv)
    return str(d)


STACK = ("# die_mm, 5, 4\n# h_top, 1e4\nname, t, k, rc, planes, active\n"
         "Si, 50, 130, 1.66e6, 2, 1\nCu, 1000, 400, 3.45e6, 2, 0\n")


def test_case_errors(ct, tmp_path):
    ok = write_case(tmp_path, STACK, "h\ncore, Si, 0.5, 0.5, 1, 1, 2\n")
    cs = ct.load_case(ok)
    assert cs.Lx == pytest.approx(5e-3) and cs.Ly == pytest.approx(4e-3) and cs.h_top == 1e4
    assert len(cs.blocks) == 1 and cs.blocks[0].watts == 2.0 and cs.tsvs == []
    bad = [
        (STACK, "h\ncore, Cu, 0.5, 0.5, 1, 1, 2\n", None, "not active"),
        (STACK, "h\ncore, Xx, 0.5, 0.5, 1, 1, 2\n", None, "unknown layer"),
        (STACK, "h\ncore, Si, 4.5, 0.5, 1, 1, 2\n", None, "outside the die"),
        (STACK, "h\ncore, Si, 0.5, 0.5, 1\n", None, "expected 7 columns"),
        (STACK, "h\ncore, Si, 0.5, 0.5, one, 1, 2\n", None, "could not parse a number"),
        (STACK, "h\ncore, Si, 0.5, 0.5, 1, 1, 2\n", "h\nSi, 0, 0, 1, 1, 1.5\n", "between 0 and 1"),
        ("name, t, k, rc, planes, active\n", "h\n", None, "no layers"),
    ]
    for stack, fp, tsv, msg in bad:
        d = write_case(tmp_path, stack, fp, tsv)
        with pytest.raises(ct.CtError) as e:
            ct.load_case(d)
        assert msg in str(e.value), (msg, str(e.value))
    with pytest.raises(ct.CtError) as e:
        ct.load_case(str(tmp_path / "missing"))
    assert e.value.status == 9  # CT_IO_ERROR


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_case_solve_matches_reference(ct, golden, name):
    ref = golden["case_files"][f"{name}_1"]["mg_f64"]
    m = ct.build_case_model(ct.load_case(case_dir(name)), 40, 40, True)
    r = ct.gpu_pcg(m, 1e-10, 50000, ct.Precond.Multigrid, ct.Precision.MG_FP64)
    assert r.converged and abs(r.iters - ref["iters"]) <= 1
    assert abs(r.T.max() - ref["T_max"]) <= 1e-7 * ref["T_max"]
    assert abs(r.T.min() - ref["T_min"]) <= 1e-7 * ref["T_max"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("nx,ny", [(40, 40), (203, 157)])
def test_device_built_model_matches_host_build(ct, name, nx, ny):
    """ct_solver_create_case builds the model on the device: every fine-level
    operator array equals the host build's bit for bit, and the two solvers
    give the same temperatures bit for bit (so the power maps agree too)."""
    folder = case_dir(name)
    for with_tsv in (True, False):
        m = ct.build_case_model(ct.load_case(folder), nx, ny, with_tsv)
        prec = ct.Precision.MG_FP32_FLEX_DW
        with ct.GpuPcg(m, ct.Precond.Multigrid, prec) as a, \
                ct.GpuPcg.from_case(folder, nx, ny, with_tsv, ct.Precond.Multigrid, prec) as b:
            oa, ob = a.level_operator(0), b.level_operator(0)
            for k in oa:
                assert np.array_equal(oa[k], ob[k]), (name, with_tsv, k)
            for s in (a, b):
                s.set_x_zero()
                s.set_rhs_steady()
                assert s.solve(1e-10, 1000).converged
            assert np.array_equal(a.get_x(), b.get_x())


def _export_index():
    import json
    with open(os.path.join(GOLDEN_DIR, "export3dice", "index.json")) as f:
        return json.load(f)


def _content_lines(path):
    """A 3D-ICE file's lines with the // comments and trailing blanks removed
    (the comments are free text; everything else is what 3D-ICE reads)."""
    out = []
    with open(path) as f:
        for line in f:
            k = line.find("//")
            if k >= 0:
                line = line[:k]
            out.append(line.rstrip())
    return out


@pytest.mark.parametrize("key", sorted(_export_index()))
def test_export_3dice_matches_reference(ct, key, tmp_path):
    """export_3dice (src/case3d.h:267-383) against the reference's own export
    of the same case folder and cell size: the same files with the same
    contents line for line (comments aside), or the same refusal message."""
    rec = _export_index()[key]
    folder = os.path.join(GOLDEN_DIR, rec["folder"])
    if "error" in rec:
        with pytest.raises(ct.CtError) as e:
            ct.export_3dice(folder, rec["cell_um"], str(tmp_path))
        assert e.value.status == 5  # CT_BAD_ARG
        assert str(e.value).endswith(rec["error"])
        return
    ct.export_3dice(folder, rec["cell_um"], str(tmp_path))
    assert sorted(os.listdir(tmp_path)) == rec["files"]
    for name in rec["files"]:
        want = _content_lines(os.path.join(GOLDEN_DIR, "export3dice", key, name))
        got = _content_lines(os.path.join(str(tmp_path), name))
        assert got == want, name


def test_export_3dice_io_error(ct, tmp_path):
    with pytest.raises(ct.CtError) as e:
        ct.export_3dice(case_dir("validate_3dice"), 100.0, str(tmp_path / "missing"))
    assert e.value.status == 9  # CT_IO_ERROR


def test_read_3dice_tmap_and_transient_csv(ct, tmp_path):
    p = tmp_path / "tmap.txt"
    p.write_text("% 3D-ICE Tmap\n% rows\n300.5 301.25\n\n302 303.5\n")
    T = ct.read_3dice_tmap(str(p))
    assert T.shape == (2, 2) and T[1, 1] == 303.5
    steps = [ct.StepRecord(1e-5, 1e-5, 7, 1.25, 10.0, 40.0), ct.StepRecord(2.1e-5, 1.1e-5, 6, 2.5, 11.0, 39.0)]
    f = tmp_path / "transient.csv"
    ct.write_transient_csv(str(f), steps, 25.0)
    lines = f.read_text().splitlines()
    assert lines[0] == "t_s,dt_s,pcg_iters,T_max_C,heat_out_W,heat_stored_W"
    assert lines[1] == "1.000000e-05,1.000000e-05,7,26.250000,10.000000,40.000000"
    assert lines[2] == "2.100000e-05,1.100000e-05,6,27.500000,11.000000,39.000000"


def test_export_3dice_from_case_spec(ct, tmp_path):
    """A CaseSpec (here the one loaded from the folder) exports the same files
    as the folder itself: names and ambient travel with it."""
    folder = case_dir("validate_tsv")
    a, b = tmp_path / "a", tmp_path / "b"
    a.mkdir()
    b.mkdir()
    ct.export_3dice(folder, 100.0, str(a))
    ct.export_3dice(ct.load_case(folder), 100.0, str(b))
    assert sorted(os.listdir(a)) == sorted(os.listdir(b))
    for name in os.listdir(a):
        assert (a / name).read_text() == (b / name).read_text(), name
