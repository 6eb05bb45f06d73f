"""Tile-shape autotuner for the batched ensemble.

The tile side sets how finely a simulation's active region follows the flow (smaller
tiles waste fewer dry cells and leave more interior tiles on small grids) against the
per-tile overheads (ghost tiles, edge bookkeeping, the 2-cell halos of the 16 x 16 blocks
at tile seams).  For each grid-size class the tuner runs one representative member through
the batched engine with every admissible tile side and keeps the one with the shortest
wall time per simulated second; other sides map to the nearest class.
"""
from __future__ import annotations

import json
import math
import os
import time

from . import workloads
from .batch import Batch

CANDIDATES = (16, 32, 64)
CLASSES = (128, 256, 512, 1024, 2048)


def candidates(side: int):
    """Tile sides that divide the grid and leave at least 4 x 4 tiles (an interior)."""
    return [t for t in CANDIDATES if side % t == 0 and side // t >= 4]


def trial(side: int, tile: int, t_sim: float = 30.0, seed: int = 4242, max_wall: float = 1.5) -> float:
    """Wall seconds per simulated second of one representative member (a cap of 1e5 m^3,
    Voellmy drag, no erosion), integrated towards t_sim for at most max_wall seconds."""
    p, b0, _ = workloads.ensemble_member(seed, side=side, tend=t_sim, tile=tile, volume=1e5, drag="Voellmy",
                                         morpho=False, kind="cap")
    b = Batch(1)
    try:
        b.add(p, b0)
        b.step()  # first step: tile activation and caches
        t0 = time.perf_counter()
        sim = b.member(0)
        t_start = sim.time[0]
        while b.step() > 0 and time.perf_counter() - t0 < max_wall:
            pass
        dt_sim = max(sim.time[0] - t_start, 1e-9)
        return (time.perf_counter() - t0) / dt_sim
    finally:
        b.close()


def tune(classes=CLASSES, t_sim: float = 30.0, cache: str | None = None, log=None) -> dict:
    """{class side: best tile side}; read from / written to `cache` (JSON) when given."""
    if cache and os.path.exists(cache):
        with open(cache) as f:
            return {int(k): int(v) for k, v in json.load(f).items()}
    best = {}
    for side in classes:
        cands = candidates(side)
        if not cands:
            continue
        # two interleaved trials per candidate, the faster kept, so that one noisy trial
        # does not decide
        timing = {t: trial(side, t, t_sim) for t in cands}
        for t in cands:
            timing[t] = min(timing[t], trial(side, t, t_sim))
        best[side] = choose(timing)
        if log:
            log(f"autotune side {side}: " + ", ".join(f"{t}: {v:.3g} s/s" for t, v in timing.items()) + f" -> {best[side]}")
    if cache:
        with open(cache, "w") as f:
            json.dump(best, f)
    return best


def choose(timing: dict, margin: float = 0.05) -> int:
    """The tile side with the least wall time per simulated second; a smaller side must
    beat the largest one within `margin` of the best by more than that margin (fewer, larger
    tiles carry less per-tile bookkeeping), so candidates within the timing noise of each
    other always resolve to the same choice."""
    fastest = min(timing.values())
    near = [t for t, v in timing.items() if v <= fastest * (1.0 + margin)]
    return max(near)


def tile_for(side: int, tuned: dict) -> int:
    """The tuned tile of the class nearest to `side` (in log size), reduced to a
    candidate that fits this side."""
    if not tuned:
        cands = candidates(side)
        return max(cands) if cands else CANDIDATES[0]
    cls = min(tuned, key=lambda c: abs(math.log(c) - math.log(side)))
    ok = candidates(side) or [CANDIDATES[0]]
    fit = [t for t in ok if t <= tuned[cls]]
    return max(fit) if fit else min(ok)
