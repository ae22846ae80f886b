"""Batched ensembles: every system of a batch must evolve exactly as it does alone.

Systems in a batch share kernel launches but no data: per-atom sums run over the atom's own
list, energies and virials are per-system fixed-point (mixed) or per-system tile sums in a
fixed order (FP64), and list rebuilds are decided per system.  So positions, velocities,
accelerations and thermo records are compared bit for bit, in both precisions, for Lennard-
Jones and Sutton-Chen systems of different sizes, densities and temperatures.
"""
import numpy as np
import pytest

from lpmd2_gb300 import inputs as I

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")

SIGMA = I.LJ_AR["sigma"]
RC_LJ = 2.5 * SIGMA
DT_LJ = 0.005 * I.lj_reduced_units(SIGMA, I.LJ_AR["epsilon"], I.LJ_AR["mass"])["tau_fs"]
SC_ARGS = "e 0.012382 a 3.61 n 9 m 6 c 39.432 cutoff 7.22"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def plugins(kind):
    if kind == "lj":
        return (gbmd.Plugin("verletlist", f"cutoff {RC_LJ!r} skin {0.3 * SIGMA!r} maxneighbors 256"),
                gbmd.Plugin("lennardjones", f"sigma {SIGMA} epsilon {I.LJ_AR['epsilon']} cutoff {RC_LJ!r}"),
                gbmd.Plugin("velocityverlet", f"dt {DT_LJ!r}"))
    return (gbmd.Plugin("verletlist", "cutoff 7.22 skin 0.5 maxneighbors 256"),
            gbmd.Plugin("suttonchen", SC_ARGS),
            gbmd.Plugin("velocityverlet", "dt 2.0"))


def setup(obj, kind, precision):
    cm, pot, integ = plugins(kind)
    obj.set_cell_manager(cm)
    obj.add_potential(pot)
    obj.set_integrator(integ)
    obj.set_precision(precision)
    obj.set_option("graph_block", 10)


def run_batch(systems, kind, precision, nsteps):
    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
    for k, s in enumerate(systems):
        b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    setup(b, kind, precision)
    b.update_forces()
    b.do_steps(nsteps)
    out = [(b.atoms(k), b.thermo(k)["raw"]) for k in range(len(systems))]
    b.close()
    return out


def run_alone(s, kind, precision, nsteps):
    sim = gbmd.Simulation(s["natoms"], s["L"])
    sim.set_atoms(s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    setup(sim, kind, precision)
    sim.update_forces()
    sim.do_steps(nsteps)
    out = (sim.atoms(), sim.thermo()["raw"])
    sim.close()
    return out


def lj_systems():
    return [I.lj_system(4, 0.95, 1.8, seed=41), I.lj_system(6, 0.80, 0.9, seed=42),
            I.lj_system(5, 0.72, 1.2, seed=43), I.lj_system(8, 0.88, 2.0, seed=44),
            I.lj_system(7, 0.70, 0.7, seed=45)]


def sc_systems():
    return [I.sc_cu_system(5, seed=51), I.sc_cu_system(7, seed=52), I.sc_cu_system(6, seed=53)]


def assert_same(a, b):
    (pa, va, aa), ta = a
    (pb, vb, ab), tb = b
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(va, vb)
    np.testing.assert_array_equal(aa, ab)
    np.testing.assert_array_equal(ta, tb)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("kind", ["lj", "sc"])
def test_batch_matches_alone_bitwise(kind, precision):
    systems = lj_systems() if kind == "lj" else sc_systems()
    nsteps = 25  # first step + two 10-step graph blocks + four direct steps
    batched = run_batch(systems, kind, precision, nsteps)
    for s, got in zip(systems, batched):
        assert_same(got, run_alone(s, kind, precision, nsteps))


def test_inactive_system_is_frozen_and_others_run_on():
    systems = lj_systems()[:3]
    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
    for k, s in enumerate(systems):
        b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    setup(b, "lj", "mixed")
    b.update_forces()
    b.do_steps(10)
    b.set_active(1, False)
    frozen = (b.atoms(1), b.thermo(1)["raw"])
    b.do_steps(13)  # odd: the position buffers end flipped
    assert_same((b.atoms(1), b.thermo(1)["raw"]), frozen)
    for k in (0, 2):
        assert_same((b.atoms(k), b.thermo(k)["raw"]), run_alone(systems[k], "lj", "mixed", 23))
    b.close()


@pytest.mark.parametrize("lanes", [2, 4, 8, 16, 32])
def test_lanes_per_atom_give_the_same_trajectory(lanes):
    # the list groups of an atom are summed exactly as with one lane, and the lanes' fixed-point
    # partials combine exactly: forces, positions, energies and virials are bitwise those of
    # one lane per atom; only the stress components (FP32 per lane) move by summation order
    systems = [I.lj_system(4, 0.9, 1.5, seed=81), I.lj_system(7, 0.8, 1.0, seed=82)]
    sigma = I.LJ_AR["sigma"]
    rc = 2.5 * sigma
    out = []
    for ln in (1, lanes):
        b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
        for k, s in enumerate(systems):
            b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
        b.set_cell_manager(gbmd.Plugin("verletlist", f"cutoff {rc!r} skin {0.3 * sigma!r} maxneighbors 256"))
        b.add_potential(gbmd.Plugin("lennardjones", f"sigma {sigma} epsilon {I.LJ_AR['epsilon']} cutoff {rc!r}"))
        b.set_integrator(gbmd.Plugin("velocityverlet", "dt 5.0"))
        b.set_precision("mixed")
        b.set_option("lanes_per_atom", ln)
        b.update_forces()
        b.do_steps(37)
        out.append(([b.atoms(k) for k in range(2)], [b.thermo(k) for k in range(2)]))
        b.close()
    (a_atoms, a_th), (b_atoms, b_th) = out
    for x, y in zip(a_atoms, b_atoms):
        for u, v in zip(x, y):
            np.testing.assert_array_equal(u, v)
    for x, y in zip(a_th, b_th):
        assert x["potential_energy"] == y["potential_energy"]
        assert x["virial"] == y["virial"]
        np.testing.assert_allclose(x["stress"], y["stress"], rtol=1e-6, atol=1e-9 * np.abs(y["stress"]).max())


@pytest.mark.parametrize("kind", ["lj", "sc"])
def test_list_feeds_agree_bitwise(kind):
    """The mixed passes read their list rows through registers (list_feed 1, the default for a
    single system) or through the shared-memory ring of bulk copies (list_feed 2, the default
    for a batch).  Both feed the same entries to the same arithmetic: a batch run with either
    ends bit for bit the same."""
    systems = lj_systems()[:3] if kind == "lj" else sc_systems()[:2]
    runs = []
    for feed in (1, 2):
        b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
        for k, s in enumerate(systems):
            b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
        setup(b, kind, "mixed")
        b.set_option("list_feed", feed)
        b.update_forces()
        b.do_steps(30)
        runs.append([(b.atoms(k), b.thermo(k)["raw"]) for k in range(len(systems))])
        b.close()
    for (a1, t1), (a2, t2) in zip(runs[0], runs[1]):
        for x, y in zip(a1, a2):
            np.testing.assert_array_equal(x, y)
        np.testing.assert_array_equal(t1, t2)
