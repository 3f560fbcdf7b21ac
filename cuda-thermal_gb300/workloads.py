"""Seeded synthetic stacks for the benchmark and parity workloads.

Each generator builds a finalized model through the library's model builder
(the reference's stack3d.h functions). Sizes, layers and power statistics are
those of the workloads the solver is measured on:

  steady_hotspot   two-tier default stack (Si 50 um / bond 10 um / Si 50 um /
                   TIM 25 um / Cu 1 mm, 10 cell layers), 10 x 10 mm, 25 W
                   uniform in each Si tier plus a 3 W, 1 x 1 mm hotspot at a
                   seeded position in the bottom tier; 64 x 64 and 800 x 800.
  four_tier        1024 x 1024 x 16: Si/bond tiers four times (no bond above
                   the top tier), TIM, Cu; 8 x 8-cell copper TSV blocks on 2 %
                   of every bond layer; 12 log-normal floorplan blocks per Si
                   tier (median 30 W/cm^2, sigma 0.6), 20 W per tier.
  batch_instances  stacks of uneven size for batched solves: nx, ny in
                   {64, 96, ..., 512}, 6-16 cell layers from a layer table.
  switching_instances  the default 256 x 256 x 10 stack, each instance with 9
                   blocks on the Si tiers switched on and off at Poisson
                   times (mean 5 ms between toggles of a block), for batched
                   backward-Euler runs with per-instance dt.
"""
from __future__ import annotations

import numpy as np

import cthermal as ct

SI = ("Si", 50e-6, 130.0, 1.66e6)
BOND = ("bond", 10e-6, 2.0, 1.70e6)
TIM = ("TIM", 25e-6, 5.0, 2.00e6)
CU = ("Cu", 1e-3, 400.0, 3.45e6)


def _layer(spec, ncells, active):
    name, t, k, rc = spec
    return ct.Layer(name, t, k, rc, ncells, active)


def steady_hotspot(n: int, seed: int = 1, hotspot: bool = True) -> ct.Model3D:
    """Default stack, 25 W per Si tier plus a seeded 3 W, 1 mm hotspot."""
    rng = np.random.default_rng(seed)
    m = ct.default_model(n, n)
    ct.add_uniform_power(m, 0, 25.0)
    if hotspot:
        xc, yc = rng.uniform(0.5e-3, 9.5e-3, size=2)
        ct.add_hotspot(m, 0, float(xc), float(yc), 1e-3, 3.0)
    ct.add_uniform_power(m, 2, 25.0)
    ct.finalize(m)
    return m


def uniform_power(n: int) -> ct.Model3D:
    """25 W uniform in each Si tier: the exact answer is the 1D chain."""
    m = ct.default_model(n, n)
    ct.add_uniform_power(m, 0, 25.0)
    ct.add_uniform_power(m, 2, 25.0)
    ct.finalize(m)
    return m


def _floorplan_blocks(Lx, Ly, rng, layer: int, nblocks: int, watts: float):
    """nblocks rectangles, log-normal density (median 30 W/cm^2, sigma 0.6),
    scaled so the tier dissipates `watts`."""
    w = rng.uniform(0.05, 0.3, size=nblocks) * Lx
    h = rng.uniform(0.05, 0.3, size=nblocks) * Ly
    x0 = rng.uniform(0, 1, size=nblocks) * (Lx - w)
    y0 = rng.uniform(0, 1, size=nblocks) * (Ly - h)
    dens = 30e4 * np.exp(0.6 * rng.standard_normal(nblocks))  # W/m^2
    pw = dens * w * h
    pw *= watts / pw.sum()
    return [ct.PowerBlock(f"b{k}", layer, float(x0[k]), float(y0[k]), float(w[k]), float(h[k]),
                          float(pw[k])) for k in range(nblocks)]


def _floorplan(m: ct.Model3D, rng, layer: int, nblocks: int, watts: float) -> None:
    for b in _floorplan_blocks(m.Lx, m.Ly, rng, layer, nblocks, watts):
        ct.add_power_block(m, b.layer, b.x0, b.y0, b.w, b.h, b.watts)


def _tsv_blocks(m: ct.Model3D, rng, layer: int, coverage: float, block: int = 8) -> None:
    """Copper (f = 1) TSV clusters of block x block cells on a seeded set of
    distinct block-aligned tiles covering `coverage` of the layer."""
    tx, ty = m.nx // block, m.ny // block
    ntiles = max(1, int(round(coverage * m.nx * m.ny / (block * block))))
    tiles = rng.choice(tx * ty, size=min(ntiles, tx * ty), replace=False)
    for t in tiles:
        i0, j0 = (t % tx) * block, (t // tx) * block
        ct.add_tsv_region(m, layer, i0 * m.dx, j0 * m.dy, block * m.dx, block * m.dy, 1.0)


def four_tier(n: int = 1024, seed: int = 3) -> ct.Model3D:
    rng = np.random.default_rng(seed)
    layers = []
    for tier in range(4):
        layers.append(_layer(SI, 2, True))
        if tier < 3:
            layers.append(_layer(BOND, 1, False))
    layers += [_layer(TIM, 1, False), _layer(CU, 4, False)]
    m = ct.build_model(layers, n, n, 10e-3, 10e-3, 2e4, 0.0)
    for L, lay in enumerate(layers):
        if lay.name == "Si":
            _floorplan(m, rng, L, 12, 20.0)
    for L, lay in enumerate(layers):
        if lay.name == "bond":
            _tsv_blocks(m, rng, L, 0.02)
    ct.finalize(m)
    return m


def batch_instance_spec(rng):
    """One stack of the batched workload as a case description and its grid
    (the same draws as batch_instance): (CaseSpec, nx, ny)."""
    sizes = np.arange(64, 513, 32)
    nx, ny = int(rng.choice(sizes)), int(rng.choice(sizes))
    target = int(rng.integers(6, 17))
    layers = [_layer(TIM, 1, False), _layer(CU, 1, False)]
    cells = 2
    tiers = 0
    while True:
        si_cells = int(rng.integers(1, 3))
        need = si_cells + (1 if tiers > 0 else 0)
        if cells + need > target:
            break
        new = [_layer(SI, si_cells, True)]
        if tiers > 0:
            new.append(_layer(BOND, 1, False))
        layers = new + layers
        cells += need
        tiers += 1
    if tiers == 0:
        layers = [_layer(SI, 1, True)] + layers
        cells += 1
    cu = layers[-1]
    layers[-1] = ct.Layer(cu.name, cu.thickness, cu.k, cu.rho_c, cu.ncells + (target - cells), False)
    Lx, Ly = 10e-3 * nx / 256, 10e-3 * ny / 256
    cs = ct.CaseSpec(layers=layers, Lx=Lx, Ly=Ly, h_top=2e4, h_bot=0.0)
    for L, lay in enumerate(layers):
        if lay.active:
            cs.blocks += _floorplan_blocks(Lx, Ly, rng, L, 12, 20.0 * (nx * ny) / 256**2)
    return cs, nx, ny


def batch_instance_specs(count: int = 256, seed: int = 4):
    rng = np.random.default_rng(seed)
    return [batch_instance_spec(rng) for _ in range(count)]


def batch_instance(rng) -> ct.Model3D:
    """One stack of the batched workload: nx, ny in {64, 96, ..., 512}, 6-16
    cell layers (Si/bond tiers, then TIM and Cu), random floorplans."""
    sizes = np.arange(64, 513, 32)
    nx, ny = int(rng.choice(sizes)), int(rng.choice(sizes))
    target = int(rng.integers(6, 17))
    layers = [_layer(TIM, 1, False), _layer(CU, 1, False)]
    cells = 2
    tiers = 0
    # add Si (+ bond) tiers below TIM/Cu until the layer budget is used
    while True:
        si_cells = int(rng.integers(1, 3))
        need = si_cells + (1 if tiers > 0 else 0)
        if cells + need > target:
            break
        new = [_layer(SI, si_cells, True)]
        if tiers > 0:
            new.append(_layer(BOND, 1, False))
        layers = new + layers
        cells += need
        tiers += 1
    if tiers == 0:
        layers = [_layer(SI, 1, True)] + layers
        cells += 1
    # spread the remaining budget over the copper spreader
    cu = layers[-1]
    layers[-1] = ct.Layer(cu.name, cu.thickness, cu.k, cu.rho_c, cu.ncells + (target - cells), False)
    m = ct.build_model(layers, nx, ny, 10e-3 * nx / 256, 10e-3 * ny / 256, 2e4, 0.0)
    for L, lay in enumerate(layers):
        if lay.active:
            _floorplan(m, rng, L, 12, 20.0 * (nx * ny) / 256**2)
    ct.finalize(m)
    return m


def batch_instances(count: int = 256, seed: int = 4):
    rng = np.random.default_rng(seed)
    return [batch_instance(rng) for _ in range(count)]


class Switching:
    """One instance of the batched transient: its model (power all off), the
    power map of each block, each block's toggle times and initial state."""

    def __init__(self, model, maps, toggles, on):
        self.model = model
        self.maps = maps          # list of (ncells,) power maps, one per block
        self.toggles = toggles    # list of sorted toggle times (s), one per block
        self.on = list(on)        # block states at t = 0
        self._next = [0] * len(maps)
        # each block's nonzero cells: summing only those, block by block in
        # the same order, gives the dense sum's bits (adding 0.0 changes nothing)
        self._sparse = [(np.flatnonzero(m), m[np.flatnonzero(m)]) for m in maps]

    def power(self) -> np.ndarray:
        P = np.zeros(self.model.ncells())
        for b, (idx, vals) in enumerate(self._sparse):
            if self.on[b]:
                P[idx] += vals
        return P

    def advance(self, t: float) -> bool:
        """Applies every toggle at or before t; True if any block switched."""
        changed = False
        for b, times in enumerate(self.toggles):
            while self._next[b] < len(times) and times[self._next[b]] <= t:
                self.on[b] = not self.on[b]
                self._next[b] += 1
                changed = True
        return changed


def switching_instances(count: int = 64, n: int = 256, seed: int = 5, blocks: int = 9,
                        mean_s: float = 5e-3, horizon_s: float = 1.0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m = ct.default_model(n, n)
        ct.finalize(m)
        maps = []
        for b in range(blocks):
            layer = 0 if b % 2 == 0 else 2
            w, h = rng.uniform(0.1, 0.3, size=2) * m.Lx
            x0, y0 = rng.uniform(0, 1, size=2) * (m.Lx - w)
            watts = float(rng.uniform(2.0, 6.0))
            m.P[:] = 0.0
            ct.add_power_block(m, layer, float(x0), float(y0), float(w), float(h), watts)
            maps.append(np.array(m.P, dtype=np.float64))
        toggles = []
        for b in range(blocks):
            ts, t = [], 0.0
            while True:
                t += float(rng.exponential(mean_s))
                if t > horizon_s:
                    break
                ts.append(t)
            toggles.append(ts)
        on = rng.integers(0, 2, size=blocks).astype(bool)
        m.P[:] = 0.0
        out.append(Switching(m, maps, toggles, on))
    return out
