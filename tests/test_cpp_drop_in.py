"""A C++ caller written against the reference's solver names
(tests/cpp/drop_in.cpp) builds against include/cthermal.hpp, links
libcthermal.so and runs: without a GPU it reports the missing device through
the adapter's exception; on a GPU its steady result matches the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(ctlib, tmp_path):
    import cthermal
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "drop_in")
    libdir = os.path.dirname(cthermal.LIB_PATH)
    cmd = [gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "drop_in.cpp"), "-L", libdir, "-lcthermal",
           f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def model(ct):
    m = ct.default_model(64, 64)
    ct.add_uniform_power(m, 0, 25.0)
    ct.add_hotspot(m, 0, 3e-3, 4e-3, 1e-3, 3.0)
    ct.add_uniform_power(m, 2, 25.0)
    ct.finalize(m)
    return m


def parse(out):
    d = {}
    for line in out.splitlines():
        k, *rest = line.split()
        d[k] = rest
    return d


def test_cpp_adapter_builds_and_runs(ctlib, ct, tmp_path):
    exe = build_driver(ctlib, tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    d = parse(r.stdout)
    assert float(d["total_power"][0]) == ct.total_power(model(ct))
    if r.returncode == 3:  # no GPU here: the adapter throws, the caller reports it
        assert "no CUDA device" in r.stdout
    else:
        assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_adapter_matches_oracle(ctlib, ct, orc, tmp_path):
    exe = build_driver(ctlib, tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    d = parse(r.stdout)
    st = d["steady"]
    assert st[st.index("converged") + 1] == "1"
    tmax = float(st[st.index("tmax") + 1])
    ref = orc.solve_steady(model(ct), 1e-10, 50000, "multigrid", mg_double=True)
    assert abs(tmax - ref.T.max()) <= 1e-7 * ref.T.max()
    assert float(st[st.index("true_relres") + 1]) <= 1e-9
    assert int(d["transient"][1]) > 0


@pytest.mark.parametrize("case", ["example", "tsv_under_core0", "validate_3dice", "validate_tsv"])
def test_cpp_case_adapter(ctlib, ct, tmp_path, case):
    """load_case / build_case_model / export_3dice through the C++ adapter:
    the same model as the Python path, and the reference's 3D-ICE export (or
    its refusal message) for the case on 100 um cells."""
    import json
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    import cthermal
    libdir = os.path.dirname(cthermal.LIB_PATH)
    exe = str(tmp_path / "case_drop_in")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "case_drop_in.cpp"), "-L", libdir, "-lcthermal",
                        f"-Wl,-rpath,{libdir}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    golden = os.path.join(ROOT, "tests", "golden")
    folder = os.path.join(golden, "cases", case)
    out = tmp_path / "ice"
    out.mkdir()
    r = subprocess.run([exe, folder, str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    d = {}
    for line in r.stdout.splitlines():
        k, _, rest = line.partition(" ")
        d[k] = rest
    cs = ct.load_case(folder)
    m = ct.build_case_model(cs, 40, 40, True)
    assert int(d["nz"]) == m.nz
    assert float(d["total_power"]) == ct.total_power(m)
    assert d["counts"].split() == [str(len(cs.layers)), str(len(cs.blocks)), str(len(cs.tsvs))]
    with open(os.path.join(golden, "export3dice", "index.json")) as f:
        ref = json.load(f)[f"{case}_100"]
    if "error" in ref:
        assert d["export_error"] == ref["error"]
        return
    assert "export_ok" in d
    assert sorted(os.listdir(out)) == ref["files"]

    def content(path):
        lines = []
        with open(path) as f:
            for line in f:
                k = line.find("//")
                lines.append((line[:k] if k >= 0 else line).rstrip())
        return lines
    for name in ref["files"]:
        assert content(os.path.join(out, name)) == content(os.path.join(golden, "export3dice", f"{case}_100", name))
