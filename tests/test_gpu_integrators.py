"""The integrators other than velocityverlet (euler, leapfrog, verlet, beeman, nosehoover)
against trajectories of the reference's own plugins (tests/golden/lj_integ_*.npz,
sc_integ_beeman.npz; see make_golden.py and ref_driver.cpp for the runtime context the
harness supplies to leapfrog / beeman / nosehoover, without which the reference stops at
their first step).

FP64: positions and velocities after 20-30 steps within 1e-9, per-step energies and
temperature within 1e-9 (the forces differ from the reference's only in summation order;
the integrator formulas keep its operation order).  Mixed: the same trajectories within the
error the FP32 pair forces leave after that many steps.
"""
import numpy as np
import pytest

from helpers import INTEG_CASES, load_golden, rel_norm_err

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def make_sim(g, precision="fp64", integ=None):
    sim = gbmd.Simulation(len(g["pos_in"]), g["L"])
    sim.set_atoms(g["pos_in"], g["vel_in"], Z=g["Z"], mass=g["mass"])
    sim.set_cell_manager(gbmd.Plugin(str(g["cm"]), str(g["cm_args"])))
    for name, args, spc in zip(g["pot_names"], g["pot_args"], g["pot_species"]):
        sim.add_potential(gbmd.Plugin(str(name), str(args)), int(spc[0]), int(spc[1]))
    name, args = (str(g["integ_name"]), str(g["integ_args"])) if integ is None else integ
    sim.set_integrator(gbmd.Plugin(name, f"dt {float(g['dt'])!r} {args}".strip()))
    sim.set_precision(precision)
    return sim


def wrapped_max(a, b, L):
    d = a - b
    d -= L * np.round(d / L)
    return float(np.abs(d).max())


@pytest.mark.parametrize("case", INTEG_CASES)
def test_fp64_trajectory_matches_reference(case):
    g = load_golden(case)
    sim = make_sim(g)
    sim.update_forces()
    n = int(g["nsteps"])
    sim.do_steps(n)
    pos, vel, acc = sim.atoms()
    log = sim.thermo_log()
    assert log.shape == (n, 22)
    L = np.asarray(g["L"], float)
    assert wrapped_max(pos, g["pos"], L) <= 1e-9 * L.max()
    assert rel_norm_err(vel, g["vel"]) <= 1e-9
    assert rel_norm_err(acc, g["acc"]) <= 1e-9
    for col in (1, 2, 4, 5):  # Epot, Ekin, T, virial per step
        np.testing.assert_allclose(log[:, col], g["thermo"][:, col], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("case", INTEG_CASES)
def test_mixed_trajectory_tracks_reference(case):
    g = load_golden(case)
    sim = make_sim(g, precision="mixed")
    sim.update_forces()
    sim.do_steps(int(g["nsteps"]))
    pos, vel, _ = sim.atoms()
    log = sim.thermo_log()
    L = np.asarray(g["L"], float)
    assert wrapped_max(pos, g["pos"], L) <= 1e-5 * L.max()
    assert rel_norm_err(vel, g["vel"]) <= 1e-4
    np.testing.assert_allclose(log[:, 1], g["thermo"][:, 1], rtol=1e-5)
    np.testing.assert_allclose(log[:, 4], g["thermo"][:, 4], rtol=1e-4)


@pytest.mark.parametrize("name", ["euler", "leapfrog", "verlet", "beeman", "nosehoover"])
def test_tagged_atoms(name):
    g = load_golden("lj_integ_" + name)
    n = len(g["pos_in"])
    flags = np.zeros(n, np.uint8)
    flags[::9] = gbmd.FLAG_FIXEDPOS
    flags[4::13] = gbmd.FLAG_FIXEDVEL
    fixedpos = flags == gbmd.FLAG_FIXEDPOS
    sim = make_sim(g)
    sim.set_flags(flags)
    sim.update_forces()
    p0, v0, _ = sim.atoms()
    sim.do_steps(2)
    _, v2, _ = sim.atoms()
    sim.do_steps(10)
    p1, v1, _ = sim.atoms()
    # fixedpos: Advance is not called for them (onestepintegrator.cc:30-37)
    np.testing.assert_array_equal(p1[fixedpos], p0[fixedpos])
    np.testing.assert_array_equal(v1[fixedpos], v0[fixedpos])
    moved = ~fixedpos
    assert np.abs(p1[moved] - p0[moved]).max() > 0
    fv = flags == gbmd.FLAG_FIXEDVEL
    if name == "euler":  # zero acceleration from the first step on: the velocity stays
        np.testing.assert_array_equal(v1[fv], v0[fv])
    if name == "beeman":
        # the first AdvanceVelocity still subtracts (1/6) a_b dt, a_b from the bare
        # UpdateForces of the backed-up configuration (fixedvel not zeroed there); from then on
        # every acceleration term is zero and the velocity stays
        assert not np.array_equal(v2[fv], v0[fv])
        np.testing.assert_array_equal(v1[fv], v2[fv])


@pytest.mark.parametrize("name", ["leapfrog", "nosehoover"])
def test_checkpoint_keeps_the_integrator_history(name, tmp_path):
    g = load_golden("lj_integ_" + name)
    a = make_sim(g)
    a.update_forces()
    a.do_steps(9)
    data = a.checkpoint()
    a.do_steps(11)
    want = a.atoms()
    b = make_sim(g)
    b.restore(data)
    b.do_steps(11)
    for x, y in zip(want, b.atoms()):
        np.testing.assert_array_equal(x, y)


def test_switching_back_to_velocityverlet():
    g = load_golden("lj_integ_beeman")
    sim = make_sim(g)
    sim.update_forces()
    sim.do_steps(5)
    sim.set_integrator(gbmd.Plugin("velocityverlet", f"dt {float(g['dt'])!r}"))
    sim.do_steps(5)
    th = sim.thermo_log()
    assert th.shape == (10, 22) and np.isfinite(th).all()
    np.testing.assert_array_equal(th[:, 0], np.arange(1, 11))


@pytest.mark.parametrize("name", ["beeman", "nosehoover", "leapfrog"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_systems_match_their_runs_alone(name, precision):
    # per-system history, Nose-Hoover friction and ranks: a batch of two liquids under the
    # integrator gives each system the trajectory it has alone, bit for bit
    from lpmd2_gb300 import inputs as I

    systems = [I.lj_system(4, 0.85, 1.3, seed=91), I.lj_system(5, 0.8, 1.0, seed=92)]
    sigma = I.LJ_AR["sigma"]
    rc = 2.5 * sigma
    args = "dt 5.0" + (" fmass 1e9 t 100" if name == "nosehoover" else "")

    def setup(obj):
        obj.set_cell_manager(gbmd.Plugin("verletlist", f"cutoff {rc!r} skin {0.3 * sigma!r} maxneighbors 256"))
        obj.add_potential(gbmd.Plugin("lennardjones", f"sigma {sigma} epsilon {I.LJ_AR['epsilon']} cutoff {rc!r}"))
        obj.set_integrator(gbmd.Plugin(name, args))
        obj.set_precision(precision)
        obj.update_forces()
        obj.do_steps(23)

    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
    for k, s in enumerate(systems):
        b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    setup(b)
    for k, s in enumerate(systems):
        alone = gbmd.Batch([s["natoms"]], [s["L"]])
        alone.set_atoms(0, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
        setup(alone)
        for x, y in zip(b.atoms(k), alone.atoms(0)):
            np.testing.assert_array_equal(x, y)
        alone.close()
    b.close()
