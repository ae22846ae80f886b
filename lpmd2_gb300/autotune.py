"""Measured choice of the batched step's tuning parameters.

The Verlet skin trades list length (work per force evaluation) against rebuild frequency;
the cell edge of the list build ((cutoff + skin) or half of it, with a 27- or 125-cell
stencil) trades candidates per atom against lanes per cell; lanes per atom in the force pass
(1, 2, 4, 8, 16 or 32, i.e. 32 to 1 atoms per warp) trade per-lane work against parallelism for
batches too small to fill the GPU.  None of the optima can be read off the workload, so each
choice is timed on a sample of the ensemble and the fastest wins: the skin x cell grid at one
lane per atom, then the lane counts at the best grid point (the lane count does not change
which pairs are listed, so the two searches are nearly independent).
"""
from __future__ import annotations

from typing import Callable

SKINS_SIGMA = (0.2, 0.3, 0.4)
CELL_SCALES = (1, 2)
LANES_PER_ATOM = (1, 2, 4, 8, 16, 32)


def tune_batch(make: Callable[[dict], object], ms_per_step: Callable[[object], float],
               skins=SKINS_SIGMA, cell_scales=CELL_SCALES, lanes=LANES_PER_ATOM) -> tuple[dict, list[dict]]:
    """make(params) builds a batch (params: skin_sigma, cell_scale, lanes_per_atom);
    ms_per_step(batch) times it.  Returns the fastest params and every trial."""
    trials = []

    def trial(p: dict) -> float:
        b = make(p)
        try:
            ms = float(ms_per_step(b))
        finally:
            b.close()
        trials.append(dict(p, ms_per_step=ms))
        return ms

    for skin in skins:
        for cs in cell_scales:
            trial({"skin_sigma": float(skin), "cell_scale": int(cs), "lanes_per_atom": 1})
    best = min(trials, key=lambda t: t["ms_per_step"])
    for ln in lanes:
        if ln != 1:
            trial({"skin_sigma": best["skin_sigma"], "cell_scale": best["cell_scale"], "lanes_per_atom": int(ln)})
    best = min(trials, key=lambda t: t["ms_per_step"])
    return {k: best[k] for k in ("skin_sigma", "cell_scale", "lanes_per_atom")}, trials


# Verlet skins (A) tried for a single system whose cell manager leaves the skin to the device
# (linkedcell: the reference has no skin; the device's list adds one).  For Sutton-Chen copper
# at 300 K (495,000 atoms, cutoff 7.22 A) the GB300 times per step, rebuilds included, were
# 0.532 / 0.509 / 0.509 / 0.533 / 0.538 / 0.571 ms at 0.2 / 0.3 / 0.4 / 0.5 / 0.722 / 1.0 A.
SKINS_A = (0.3, 0.4, 0.5, 0.722)


def tune_skin(make: Callable[[float], object], ms_per_step: Callable[[object], float],
              skins=SKINS_A) -> tuple[float, list[dict]]:
    """make(skin) builds a simulation with that Verlet skin; ms_per_step(sim) times it (rebuilds
    included, so over enough steps to see several).  Returns the fastest skin and every trial."""
    trials = []
    for skin in skins:
        sim = make(float(skin))
        try:
            trials.append({"skin": float(skin), "ms_per_step": float(ms_per_step(sim))})
        finally:
            sim.close()
    return min(trials, key=lambda t: t["ms_per_step"])["skin"], trials

