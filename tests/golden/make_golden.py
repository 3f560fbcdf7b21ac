"""Generates tests/golden/golden.json (+ golden_arrays.npz) from the UNMODIFIED
reference CPU solver (oracle/_ref, compiled from the reference sources by
`make -C oracle ref`).

Run where the reference sources are present:
    python tests/golden/make_golden.py          (everything)
    python tests/golden/make_golden.py export   (the 3D-ICE export fixtures only)
The fixtures pin both the C oracle (bit-for-bit: the same T bytes, iteration
counts and residuals) and the library's model builder (bit-for-bit arrays).
Large arrays are stored as SHA-256 digests of their little-endian bytes;
arrays of the small cases are stored whole.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402

DEFAULT = [(50e-6, 130.0, 1.66e6, 2, 1), (10e-6, 2.0, 1.70e6, 1, 0), (50e-6, 130.0, 1.66e6, 2, 1),
           (25e-6, 5.0, 2.00e6, 1, 0), (1e-3, 400.0, 3.45e6, 4, 0)]
BASE3DICE = [(1e-6, 130.0, 1.66e6, 1, 0), (50e-6, 130.0, 1.66e6, 1, 1), (10e-6, 2.0, 1.70e6, 1, 0),
             (50e-6, 130.0, 1.66e6, 1, 1), (25e-6, 5.0, 2.00e6, 1, 0), (1e-3, 400.0, 3.45e6, 4, 0)]
HOT = [("uniform", 0, 0, 0, 0, 0, 22.0), ("hotspot", 0, 3e-3, 3e-3, 1e-3, 0, 3.0),
       ("uniform", 2, 0, 0, 0, 0, 25.0)]
UNI = [("uniform", 0, 0, 0, 0, 0, 25.0), ("uniform", 2, 0, 0, 0, 0, 25.0)]
MM = 1e-3
# example_case() power blocks (src/case3d.h:170-190), moved off the cell edges
BLOCKS = [("block", 0, 0.537 * MM, 0.511 * MM, 2.0 * MM, 2.0 * MM, 6.0),
          ("block", 0, 3.037 * MM, 0.511 * MM, 2.0 * MM, 2.0 * MM, 6.0),
          ("block", 0, 5.537 * MM, 0.511 * MM, 4.0 * MM, 4.5 * MM, 3.0),
          ("block", 2, 0.0, 0.0, 10.0 * MM, 10.0 * MM, 12.0),
          ("block", 2, 4.037 * MM, 4.011 * MM, 2.0 * MM, 2.0 * MM, 3.0)]
TSVS = [(1, 2.55 * MM, 0.5 * MM, 0.40 * MM, 4.5 * MM, 0.15),
        (1, 0.5 * MM, 2.55 * MM, 4.5 * MM, 0.40 * MM, 0.15),
        (2, 2.55 * MM, 0.5 * MM, 0.40 * MM, 4.5 * MM, 0.15)]

# name: (layers, nx, ny, Lx, Ly, h_top, h_bot, power, tsvs)
CASES = {
    "hotspot64": (DEFAULT, 64, 64, 10e-3, 10e-3, 2e4, 0.0, HOT, []),
    "uniform64": (DEFAULT, 64, 64, 10e-3, 10e-3, 2e4, 0.0, UNI, []),
    "blocks_tsv_17x13": (DEFAULT, 17, 13, 10e-3, 10e-3, 2e4, 0.0, BLOCKS, TSVS),
    "blocks_tsv_40x24": (DEFAULT, 40, 24, 10e-3, 6e-3, 2e4, 1e3, BLOCKS, TSVS),
    "tiny3x5": (DEFAULT, 3, 5, 10e-3, 10e-3, 2e4, 0.0, UNI + [("block", 0, 0, 0, 4e-3, 3e-3, 2.0)], []),
    "column1x1": (DEFAULT, 1, 1, 10e-3, 10e-3, 2e4, 0.0, UNI, []),
    "row1x9": (DEFAULT, 1, 9, 10e-3, 10e-3, 2e4, 0.0, UNI + [("block", 2, 0, 0, 10e-3, 2e-3, 1.0)], []),
    "tsv_layer64": (DEFAULT, 64, 64, 10e-3, 10e-3, 2e4, 0.0, UNI, [(1, 0.0, 0.0, 10e-3, 10e-3, 0.2)]),
    "base3dice_50": (BASE3DICE, 50, 50, 10e-3, 10e-3, 2e4, 0.0,
                     [("block", 1, 0.5 * MM, 0.5 * MM, 2 * MM, 2 * MM, 6.0),
                      ("block", 3, 0, 0, 10 * MM, 4 * MM, 4.8)], []),
}
FULL_ARRAYS_BELOW = 2500  # cells


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def solve_record(m, tol, precond):
    r = ref.cpu_pcg(m, tol, 50000, precond)
    T = r["T"]
    return dict(iters=r["iters"], relres=r["relres"], converged=r["converged"], T_sha=sha(T),
                T_max=float(T.max()), T_min=float(T.min()), true_relres=ref.true_relres(m, T),
                heat_out=ref.heat_out(m, T)), T


CASES = ("example", "tsv_under_core0", "validate_3dice", "validate_tsv")


def copy_cases():
    """The reference's four example case folders (its CSV inputs, a few KB),
    as fixtures for the case-loader tests: tests/golden/cases/<case>/*.csv."""
    import shutil
    src_root = os.path.join(ref.REF_SRC, "cases")
    for case in CASES:
        dst = os.path.join(HERE, "cases", case)
        os.makedirs(dst, exist_ok=True)
        for f in sorted(os.listdir(os.path.join(src_root, case))):
            if f.endswith(".csv"):
                shutil.copyfile(os.path.join(src_root, case, f), os.path.join(dst, f))


EXPORT_CELLS = (100.0, 250.0, 333.0)  # um; 333 does not divide the 10 mm die


def export_variants():
    """Case folders the 3D-ICE export must refuse, each made from
    validate_3dice by one edit: tests/golden/cases_export/<variant>/."""
    src = os.path.join(HERE, "cases", "validate_3dice")
    stack = open(os.path.join(src, "stack.csv")).read()
    plan = open(os.path.join(src, "floorplan.csv")).read()
    variants = {
        "bottom_sink": (stack.replace("# h_bottom, 0", "# h_bottom, 500"), plan),
        "two_plane_die": (stack.replace("Si tier 1 (top), 50, 130, 1.66e6, 1, 1",
                                        "Si tier 1 (top), 50, 130, 1.66e6, 2, 1"), plan),
        "overlapping_blocks": (stack, plan + "hot_overlap, Si tier 2 (bottom), 1.5, 1.5, 1.0, 1.0, 1\n"),
        "empty_die": (stack, "\n".join(l for l in plan.splitlines() if "Si tier 1" not in l) + "\n"),
    }
    names = []
    for name, (st, fp) in variants.items():
        assert st != stack or fp != plan, name
        d = os.path.join(HERE, "cases_export", name)
        os.makedirs(d, exist_ok=True)
        with open(os.path.join(d, "stack.csv"), "w") as f:
            f.write(st)
        with open(os.path.join(d, "floorplan.csv"), "w") as f:
            f.write(fp)
        names.append(name)
    return names


def export_golden():
    """The reference's 3D-ICE export of every case folder (and of the
    variants above) at a few cell sizes: tests/golden/export3dice/<case>_<cell>/
    holds the files it wrote, and index.json lists them (or the error message
    when it refused)."""
    import shutil
    root = os.path.join(HERE, "export3dice")
    index = {}
    folders = [(c, os.path.join("cases", c)) for c in CASES]
    folders += [(v, os.path.join("cases_export", v)) for v in export_variants()]
    for case, rel in folders:
        for cell in EXPORT_CELLS:
            key = f"{case}_{int(cell)}"
            d = os.path.join(root, key)
            shutil.rmtree(d, ignore_errors=True)
            os.makedirs(d)
            err = ref.export_3dice(os.path.join(HERE, rel), cell, d)
            if err is not None:
                shutil.rmtree(d)
                index[key] = dict(folder=rel, cell_um=cell, error=err)
            else:
                index[key] = dict(folder=rel, cell_um=cell, files=sorted(os.listdir(d)))
            print("export", key, index[key].get("error", index[key].get("files")))
    with open(os.path.join(root, "index.json"), "w") as f:
        json.dump(index, f, indent=1)


def main():
    if sys.argv[1:] == ["export"]:
        ref.lib(False)
        export_golden()
        return
    for mgd in (False, True):
        ref.lib(mgd)
    out = {"generator": "tests/golden/make_golden.py", "reference": "cuda-thermal src/pcg3d_cpu.cpp",
           "cases": {}}
    arrays = {}
    for name, (layers, nx, ny, Lx, Ly, ht, hb, power, tsvs) in CASES.items():
        md = ref.model(layers, nx, ny, Lx, Ly, ht, hb, power, tsvs, mg_double=True)
        mf = ref.model(layers, nx, ny, Lx, Ly, ht, hb, power, tsvs, mg_double=False)
        spec = dict(layers=layers, nx=nx, ny=ny, Lx=Lx, Ly=Ly, h_top=ht, h_bot=hb,
                    power=power, tsvs=tsvs)
        rec = dict(spec=spec, nz=md.nz, dx=md.dx, dy=md.dy, total_power=ref.total_power(md))
        rec["model_sha"] = {k: sha(getattr(md, k)) for k in
                            ("gE", "gN", "gU", "gB", "cap", "P", "dz", "tsv_frac")}
        rec["analytic_1d"] = ref.analytic_1d(md).tolist()
        lv = ref.levels(md)
        rec["levels"] = [dict(nx=L["nx"], ny=L["ny"],
                              sha={k: sha(L[k]) for k in ("gE", "gN", "gU", "gB", "cap")})
                         for L in lv]
        rec["mg_f64"], Td = solve_record(md, 1e-10, "multigrid")
        rec["mg_f32"], Tf = solve_record(mf, 1e-10, "multigrid")
        rec["jacobi"], Tj = solve_record(md, 1e-6, "jacobi")
        if nx * ny * md.nz < FULL_ARRAYS_BELOW:
            for k in ("gE", "gN", "gU", "gB", "cap", "P"):
                arrays[f"{name}.{k}"] = getattr(md, k)
            arrays[f"{name}.T_mg_f64"] = Td
            arrays[f"{name}.T_mg_f32"] = Tf
            arrays[f"{name}.T_jacobi"] = Tj
        out["cases"][name] = rec
        print(name, rec["mg_f64"]["iters"], rec["mg_f32"]["iters"], rec["jacobi"]["iters"])

    # Transients: the verify-3/4 settings (src/main3d.cu:146-176) on a 32 x 32 grid.
    out["transients"] = {}
    for mgd in (False, True):
        m = ref.model(DEFAULT, 32, 32, 10e-3, 10e-3, 2e4, 0.0, HOT, [], mg_double=mgd)
        for pc in ("multigrid", "jacobi"):
            if pc == "jacobi" and not mgd:
                continue
            tr = ref.run_transient(m, pc, dt0=1e-5, growth=1.2, dt_max=0.05, t_end=0.02, tol=1e-9)
            key = f"hotspot32_{pc}_{'f64' if mgd else 'f32'}"
            out["transients"][key] = dict(steps=tr["steps"].tolist(), T_sha=sha(tr["T"]),
                                          total_iters=tr["total_iters"],
                                          converged=tr["converged"], T_max=float(tr["T"].max()))
            print(key, len(tr["steps"]), tr["total_iters"])

    # The example case from its CSV files (load_case + build_case_model).
    out["case_files"] = {}
    case_root = os.path.join(ref.REF_SRC, "cases")
    copy_cases()
    for case in CASES:
        for with_tsv in (True, False):
            m = ref.case_model(os.path.join(case_root, case), 40, 40, with_tsv, mg_double=True)
            r, _ = solve_record(m, 1e-10, "multigrid")
            out["case_files"][f"{case}_{int(with_tsv)}"] = dict(
                nz=m.nz, total_power=ref.total_power(m),
                model_sha={k: sha(getattr(m, k)) for k in ("gE", "gN", "gU", "gB", "cap", "P")},
                mg_f64=r)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "golden_arrays.npz"), **arrays)
    export_golden()


if __name__ == "__main__":
    main()
