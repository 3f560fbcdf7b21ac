"""Generates tests/golden/golden.json (+ golden_arrays.npz) from the UNMODIFIED
reference CPU solver (oracle/_ref, compiled from the reference sources by
`make -C oracle ref`).

Run where the reference sources are present:
    python tests/golden/make_golden.py
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


def main():
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


if __name__ == "__main__":
    main()
