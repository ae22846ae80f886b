"""Generates the golden fixtures in this folder by running the reference LPMD plugins.

The reference sources are compiled by ``make -C oracle ref`` into oracle/_ref/ (only possible
where the reference checkout is present) and driven through oracle/ref_driver.cpp.  Each
fixture stores the exact inputs (so the GPU machine, which has no reference, replays identical
inputs) and the reference's outputs:

  acc0, thermo0          after the initial CombinedPotential::UpdateForces
  neigh_*                BuildNeighborList(i, full, rcut) for every atom after that call
                         (full index lists for small cases, counts + multiset hashes always)
  thermo                 one record per DoStep (see oracle.THERMO_FIELDS; stress at 13..21)
  pos, vel, acc          the final state

The EAM driver leaves its stress accumulator uninitialised (liblpmd/simulation/metalpotential.cc:68),
so the stress entries of EAM fixtures are stored as NaN ("not pinned").

Usage:  python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle  # noqa: E402
from helpers import GOLDEN, GOLDEN_CASES, INTEG_CASES, neighbor_hashes, workload  # noqa: E402


def make(name: str) -> None:
    w = workload(name)
    out = oracle.run_reference(w["pos"], w["L"], w["symbol"], w["vel"], w["cm"], w["cm_args"],
                               w["pots"], w["dt"], w["nsteps"], neigh=w["neigh"], integrator=w.get("integ"))
    n = len(w["pos"])
    rec = dict(
        pos_in=w["pos"], vel_in=w["vel"], L=w["L"], Z=np.full(n, w["Z"], dtype=np.int32),
        mass=out["mass"], dt=np.float64(w["dt"]), nsteps=np.int64(w["nsteps"]),
        acc0=out["acc0"], thermo0=out["thermo0"], thermo=out["thermo"],
        pos=out["pos"], vel=out["vel"], acc=out["acc"],
        neigh_full=np.int64(w["neigh"][0]), neigh_rcut=np.float64(w["neigh"][1]),
        neigh_counts=out["neigh_counts"].astype(np.int32),
        neigh_hash=neighbor_hashes(out["neigh_counts"], out["neigh_idx"]),
    )
    if n <= 1000:
        rec["neigh_idx"] = out["neigh_idx"].astype(np.int32)
    if any(p[0] != "lennardjones" for p in w["pots"]):
        rec["thermo0"][13:22] = np.nan
        rec["thermo"][:, 13:22] = np.nan
    # plugin description, as text arrays
    rec["cm"] = np.array(w["cm"])
    rec["cm_args"] = np.array(w["cm_args"])
    rec["pot_names"] = np.array([p[0] for p in w["pots"]])
    rec["pot_args"] = np.array([p[1] for p in w["pots"]])
    rec["pot_species"] = np.array([[p[2], p[3]] for p in w["pots"]], dtype=np.int32)
    integ = w.get("integ", ("velocityverlet", ""))
    rec["integ_name"] = np.array(integ[0])
    rec["integ_args"] = np.array(integ[1])
    np.savez_compressed(GOLDEN / f"{name}.npz", **rec)
    print(f"{name}: N={n} E0={out['thermo0'][1]:.10f} steps={w['nsteps']}")


if __name__ == "__main__":
    if not oracle.reference_available():
        oracle.build()
    for case in sys.argv[1:] or GOLDEN_CASES + INTEG_CASES:
        make(case)
