"""Test configuration: the `gpu` marker, import paths and one-time builds.

Tests marked `gpu` need a CUDA device and call the CUDA library through its
C ABI. Everything else runs on the CPU: the oracle against the golden
fixtures, the model builder, the host logic, and the library's symbol table.
"""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "cuda-thermal_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def ctlib():
    """The built CUDA library (built here if missing)."""
    import cthermal
    if not os.path.exists(cthermal.LIB_PATH):
        cthermal.build()
    return cthermal.lib()


@pytest.fixture(scope="session")
def ct(ctlib):
    import cthermal
    return cthermal


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
        g = json.load(f)
    g["arrays"] = dict(np.load(os.path.join(GOLDEN_DIR, "golden_arrays.npz")))
    return g


def build_spec_model(ct, spec):
    """Builds a golden case's model with the library's model builder, applying
    the power and TSV operations in the generator's order."""
    layers = [ct.Layer(f"layer{k}", *l[:4], bool(l[4])) for k, l in enumerate(spec["layers"])]
    m = ct.build_model(layers, spec["nx"], spec["ny"], spec["Lx"], spec["Ly"], spec["h_top"],
                       spec["h_bot"])
    for kind, layer, x0, y0, w, h, watts in spec["power"]:
        if kind == "block":
            ct.add_power_block(m, layer, x0, y0, w, h, watts)
        elif kind == "uniform":
            ct.add_uniform_power(m, layer, watts)
        else:
            ct.add_hotspot(m, layer, x0, y0, w, watts)
    for layer, x0, y0, w, h, f in spec["tsvs"]:
        ct.add_tsv_region(m, layer, x0, y0, w, h, f)
    ct.finalize(m)
    return m
