"""Small boxes of the batched ensemble against the oracle's minimum-image restatement.

The ensemble's densest small systems (FCC 4^3 and 5^3 at rho* 0.90-0.95) have box edges below
three list radii, 3 (rc + skin) = 28.6 A for argon with rc = 2.5 sigma and skin 0.3 sigma.  Their
Verlet-list grid is then one or two cells wide, a neighbour cell is reached through several
periodic shifts, and the list build keeps one image per pair (the de-duplicated path).  The
reference's cell manager for such boxes is MinimumImageCellManager (plugins/minimumimage.cc:
68-100: all pairs, one wrap per component), restated in the oracle.  Checked, for each system
alone and inside a batch with a larger system, at the initial state and after 25 steps (list
rebuilds and a captured graph block in between):

  neighbour multisets      exact, both precisions (FP32 decision plus the exact guard band)
  FP64 path                forces <= 1e-12 relative norm, energy and virial <= 1e-12
  mixed path               force RMS <= 1e-5, energy <= 1e-6, virial <= 1e-5 relative
"""
import numpy as np
import pytest

import oracle
from helpers import neighbor_hashes, rel_norm_err
from lpmd2_gb300 import inputs as I

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")

SIGMA, EPS = I.LJ_AR["sigma"], I.LJ_AR["epsilon"]
RC = 2.5 * SIGMA
SKIN = 0.3 * SIGMA
LJ = f"sigma {SIGMA} epsilon {EPS} cutoff {RC!r}"
TOL = {"fp64": (1e-12, 1e-12, 1e-12), "mixed": (1e-5, 1e-6, 1e-5)}


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists() or not oracle.PORT_LIB.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def small_systems():
    out = [I.lj_system(4, 0.95, 1.8, seed=61), I.lj_system(4, 0.90, 1.2, seed=62),
           I.lj_system(5, 0.93, 0.9, seed=63), I.lj_system(5, 0.95, 2.0, seed=64)]
    for s in out:
        L = float(s["L"][0])
        # below three list radii (the de-duplicated path), above two (a Verlet list at all)
        assert 2 * (RC + SKIN) < L < 3 * (RC + SKIN)
    return out


def setup(obj, precision):
    obj.set_cell_manager(gbmd.Plugin("verletlist", f"cutoff {RC!r} skin {SKIN!r} maxneighbors 256"))
    obj.add_potential(gbmd.Plugin("lennardjones", LJ))
    obj.set_integrator(gbmd.Plugin("velocityverlet", "dt 10.0"))
    obj.set_precision(precision)
    obj.set_option("graph_block", 10)


def oracle_at(s, pos):
    n = s["natoms"]
    sim = oracle.PortSim(pos, s["L"], np.full(n, s["Z"]), s["mass"])
    sim.set_cell_manager("minimumimage", f"cutoff {RC!r}")
    sim.add_potential("lennardjones", LJ)
    sim.update_forces()
    _, _, acc = sim.atoms()
    counts, idx = sim.neighbors(True, RC)
    return dict(acc=acc, energy=sim.energy(), virial=sim.virial(), counts=counts, hash=neighbor_hashes(counts, idx))


def check(s, atoms, thermo, neigh, precision):
    pos, _, acc = atoms
    ref = oracle_at(s, pos)
    tf, te, tw = TOL[precision]
    assert rel_norm_err(acc, ref["acc"]) <= tf
    assert abs(thermo["potential_energy"] - ref["energy"]) <= te * abs(ref["energy"])
    assert abs(thermo["virial"] - ref["virial"]) <= tw * abs(ref["virial"])
    counts, idx = neigh
    np.testing.assert_array_equal(counts, ref["counts"])
    np.testing.assert_array_equal(neighbor_hashes(counts, idx), ref["hash"])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_small_boxes_alone_match_minimum_image_oracle(precision):
    for s in small_systems():
        sim = gbmd.Simulation(s["natoms"], s["L"])
        sim.set_atoms(s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
        setup(sim, precision)
        sim.update_forces()
        assert sim.stats()["neighbor_mode"] == "verlet"
        check(s, sim.atoms(), sim.thermo(), sim.neighbors(True, RC), precision)
        sim.do_steps(25)
        # forces of the state the run reached, re-evaluated at those positions
        sim.update_forces()
        check(s, sim.atoms(), sim.thermo(), sim.neighbors(True, RC), precision)
        sim.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_small_boxes_in_a_batch_match_minimum_image_oracle(precision):
    systems = small_systems() + [I.lj_system(8, 0.85, 1.4, seed=65)]
    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
    for k, s in enumerate(systems):
        b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    setup(b, precision)
    b.update_forces()
    for k, s in enumerate(systems):
        check(s, b.atoms(k), b.thermo(k), b.neighbors(k, True, RC), precision)
    b.do_steps(25)
    b.update_forces()
    for k, s in enumerate(systems):
        check(s, b.atoms(k), b.thermo(k), b.neighbors(k, True, RC), precision)
    b.close()
