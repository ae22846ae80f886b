"""Failure paths on the GPU that fault, trap and hang nothing.

A kernel wait that nothing completes must end by its bound and report it, leaving the device
usable; device-side limits (list capacity, positions far outside the box) come back as status
codes through the error word, and the simulation can be set up again afterwards.
"""
import numpy as np
import pytest

from helpers import load_golden

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def small_sim(g, cm_args=None):
    sim = gbmd.Simulation(len(g["pos_in"]), g["L"])
    sim.set_atoms(g["pos_in"], g["vel_in"], Z=g["Z"], mass=g["mass"])
    sim.set_cell_manager(gbmd.Plugin(str(g["cm"]), cm_args or str(g["cm_args"])))
    for name, args, spc in zip(g["pot_names"], g["pot_args"], g["pot_species"]):
        sim.add_potential(gbmd.Plugin(str(name), str(args)), int(spc[0]), int(spc[1]))
    sim.set_integrator(gbmd.Plugin("velocityverlet", f"dt {float(g['dt'])!r}"))
    return sim


def test_bounded_wait_gives_up_and_device_stays_usable():
    assert gbmd.selftest_bounded_wait(1000) is True
    with pytest.raises(gbmd.GbmdError):
        gbmd.selftest_bounded_wait(0)
    g = load_golden("lj_liquid_vl")
    sim = small_sim(g)
    sim.set_precision("mixed")
    sim.update_forces()
    sim.do_steps(10)
    assert np.isfinite(sim.thermo()["total_energy"])


def test_capacity_error_then_recovery():
    g = load_golden("lj_liquid_vl")
    sim = small_sim(g, "cutoff 8.5 maxneighbors 20")
    with pytest.raises(gbmd.PluginError, match="maxneighbors"):
        sim.update_forces()
    sim.close()
    sim = small_sim(g)
    sim.update_forces()
    sim.do_steps(5)
    assert np.isfinite(sim.thermo()["total_energy"])


def test_far_outside_position_is_a_runtime_error():
    g = load_golden("lj_liquid_vl")
    pos = g["pos_in"].copy()
    pos[7] = [1e12, 0.0, 0.0]
    sim = gbmd.Simulation(len(pos), g["L"])
    sim.set_atoms(pos, g["vel_in"], Z=g["Z"], mass=g["mass"])
    sim.set_cell_manager(gbmd.Plugin(str(g["cm"]), str(g["cm_args"])))
    sim.add_potential(gbmd.Plugin(str(g["pot_names"][0]), str(g["pot_args"][0])))
    sim.set_integrator(gbmd.Plugin("velocityverlet", "dt 1.0"))
    with pytest.raises(gbmd.GbmdError, match="outside"):
        sim.update_forces()
