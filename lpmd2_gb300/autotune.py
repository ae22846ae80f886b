"""Measured choice of the batched step's tuning parameters.

The Verlet skin trades list length (work per force evaluation) against rebuild frequency;
the cell edge of the list build ((cutoff + skin) or half of it, with a 27- or 125-cell
stencil) trades candidates per atom against lanes per cell.  Neither optimum can be read off
the workload, so each combination is timed on a sample of the ensemble and the fastest wins.
"""
from __future__ import annotations

from typing import Callable

SKINS_SIGMA = (0.2, 0.3, 0.4)
CELL_SCALES = (1, 2)


def tune_batch(make: Callable[[dict], object], ms_per_step: Callable[[object], float],
               skins=SKINS_SIGMA, cell_scales=CELL_SCALES) -> tuple[dict, list[dict]]:
    """make(params) builds a batch (params: skin_sigma, cell_scale); ms_per_step(batch) times
    it.  Returns the fastest params and every trial."""
    trials = []
    for skin in skins:
        for cs in cell_scales:
            p = {"skin_sigma": float(skin), "cell_scale": int(cs)}
            b = make(p)
            try:
                ms = float(ms_per_step(b))
            finally:
                b.close()
            trials.append(dict(p, ms_per_step=ms))
    best = min(trials, key=lambda t: t["ms_per_step"])
    return {"skin_sigma": best["skin_sigma"], "cell_scale": best["cell_scale"]}, trials
