"""Checkpoint / restore: a simulation restored from a snapshot continues bit for bit.

The snapshot (gbmd_*_checkpoint_save) holds the complete device state — atoms in device
order, Verlet lists, rebuild clocks and displacement references, thermo log — and the host
counters, so the restored run takes the same rebuild decisions and sums in the same order.
"""
import numpy as np
import pytest

from helpers import load_golden
from lpmd2_gb300 import inputs as I

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def make_sim(g, precision, cm_args=None):
    sim = gbmd.Simulation(len(g["pos_in"]), g["L"])
    sim.set_atoms(g["pos_in"], g["vel_in"], Z=g["Z"], mass=g["mass"])
    sim.set_cell_manager(gbmd.Plugin(str(g["cm"]), cm_args or str(g["cm_args"])))
    for name, args, spc in zip(g["pot_names"], g["pot_args"], g["pot_species"]):
        sim.add_potential(gbmd.Plugin(str(name), str(args)), int(spc[0]), int(spc[1]))
    sim.set_integrator(gbmd.Plugin("velocityverlet", f"dt {float(g['dt'])!r}"))
    sim.set_precision(precision)
    return sim


def state(sim):
    p, v, a = sim.atoms()
    return p, v, a, sim.thermo_log()


@pytest.mark.parametrize("case", ["lj_liquid_vl", "sc_cu"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_restored_simulation_continues_bitwise(case, precision, tmp_path):
    g = load_golden(case)
    a = make_sim(g, precision)
    a.update_forces()
    a.do_steps(31)
    path = tmp_path / "run.ckpt"
    path.write_bytes(a.checkpoint())
    a.do_steps(37)
    want = state(a)
    b = make_sim(g, precision)
    b.restore(path.read_bytes())
    b.do_steps(37)
    got = state(b)
    for x, y in zip(want, got):
        np.testing.assert_array_equal(x, y)
    assert b.stats()["steps"] == a.stats()["steps"]


def test_batch_checkpoint_continues_bitwise():
    systems = [I.lj_system(4, 0.9, 1.5, seed=61), I.lj_system(6, 0.75, 1.0, seed=62)]
    sigma = I.LJ_AR["sigma"]
    rc = 2.5 * sigma

    def make():
        b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
        for k, s in enumerate(systems):
            b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
        b.set_cell_manager(gbmd.Plugin("verletlist", f"cutoff {rc!r} skin {0.3 * sigma!r} maxneighbors 256"))
        b.add_potential(gbmd.Plugin("lennardjones", f"sigma {sigma} epsilon {I.LJ_AR['epsilon']} cutoff {rc!r}"))
        b.set_integrator(gbmd.Plugin("velocityverlet", "dt 10.0"))
        b.set_precision("mixed")
        return b

    a = make()
    a.update_forces()
    a.do_steps(20)
    ck = a.checkpoint()
    a.do_steps(15)
    b = make()
    b.restore(ck)
    b.do_steps(15)
    for k in range(len(systems)):
        for x, y in zip(a.atoms(k), b.atoms(k)):
            np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(a.thermo(k)["raw"], b.thermo(k)["raw"])


def test_checkpoint_needs_the_same_configuration():
    g = load_golden("lj_liquid_vl")
    a = make_sim(g, "mixed")
    a.update_forces()
    a.do_steps(5)
    ck = a.checkpoint()
    b = make_sim(g, "fp64")
    with pytest.raises(gbmd.GbmdError, match="differ"):
        b.restore(ck)
    with pytest.raises(gbmd.GbmdError, match="gbmd checkpoint|truncated|size"):
        b.restore(ck[:100])


def test_lcbinary_checkpoint_after_the_grid_grew():
    # lj_lcbinary_grow starts from a 4x4x4 sub-cell grid that grows until no sub-cell holds two
    # atoms; a fresh simulation restoring the snapshot adopts the grown grid
    g = load_golden("lj_lcbinary_grow")
    a = make_sim(g, "fp64")
    a.update_forces()
    a.do_steps(7)
    grown = a.stats()["cell_grid"]
    assert min(grown) > 4
    data = a.checkpoint()
    a.do_steps(9)
    want = state(a)
    b = make_sim(g, "fp64")
    b.restore(data)
    assert b.stats()["cell_grid"] == grown
    b.do_steps(9)
    for x, y in zip(want, state(b)):
        np.testing.assert_array_equal(x, y)
