"""GPU parity at the benchmark's own sizes, through checks that do not need a full oracle run.

* The 256,000-atom LJ liquid (FCC 40^3 at rho* 0.8442, jittered, T* 1.5, rc 2.5 sigma): one
  force evaluation in the oracle (linkedcell, the reference algorithm) against the FP64 path
  (forces/energy/virial <= 1e-12 relative, neighbour multisets exact) and the mixed Verlet-list
  path (force RMS <= 1e-5, energy <= 1e-6, virial <= 1e-5 relative).
* The 495,000-atom Sutton-Chen copper (FCC 50^3 minus 1 % of the sites) after 20 FP64 steps
  from the lattice: the same comparison for the two-pass EAM force, virial <= 1e-5 included.
  Near the lattice constant pair repulsion and many-body attraction cancel in the virial to
  about 1/20 of either, so a consistent bias of the FP32 functionals would be amplified ~100
  times; the mixed kernels refine the hardware reciprocal square root by a Newton step for
  that reason, and sum energy and virial per list group in int64 fixed point.
* Total momentum of the 256k liquid after 200 steps of either path: the pair forces cancel
  (Newton's third law in the reference's full-list sum), so it stays at its initial value up to
  rounding.
* The 512-system ensemble (3.2 M atoms): sample systems advance bit for bit as they do alone.
"""
import numpy as np
import pytest

import oracle
from helpers import neighbor_hashes, rel_norm_err

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")
from lpmd2_gb300 import inputs as I  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists() or not oracle.PORT_LIB.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


SIGMA, EPS = I.LJ_AR["sigma"], I.LJ_AR["epsilon"]
RC = 2.5 * SIGMA
LJ = f"sigma {SIGMA} epsilon {EPS} cutoff {RC!r}"


@pytest.fixture(scope="module")
def liquid():
    return I.lj_system(40, 0.8442, 1.5, seed=2)


def lj_cells(L) -> str:
    n = int(np.floor(float(L[0]) / RC))
    return f"cutoff {RC!r} nx {n} ny {n} nz {n}"


@pytest.fixture(scope="module")
def liquid_oracle(liquid):
    w = liquid
    sim = oracle.PortSim(w["pos"], w["L"], np.full(w["natoms"], w["Z"]), w["mass"], w["vel"])
    sim.set_cell_manager("linkedcell", lj_cells(w["L"]))
    sim.add_potential("lennardjones", LJ)
    sim.update_forces()
    _, _, acc = sim.atoms()
    counts, idx = sim.neighbors(True, RC)
    return dict(acc=acc, energy=sim.energy(), virial=sim.virial(), counts=counts, hash=neighbor_hashes(counts, idx))


def lj_sim(w, precision, cm, cm_args):
    sim = gbmd.Simulation(w["natoms"], w["L"])
    sim.set_atoms(w["pos"], w["vel"], Z=w["Z"], mass=w["mass"])
    sim.set_cell_manager(gbmd.Plugin(cm, cm_args))
    sim.add_potential(gbmd.Plugin("lennardjones", LJ))
    sim.set_integrator(gbmd.Plugin("velocityverlet", "dt 10.0"))
    sim.set_precision(precision)
    return sim


def test_lj_liquid_256k_fp64_matches_oracle(liquid, liquid_oracle):
    sim = lj_sim(liquid, "fp64", "linkedcell", lj_cells(liquid["L"]))
    sim.update_forces()
    _, _, acc = sim.atoms()
    th = sim.thermo_raw()
    ref = liquid_oracle
    assert rel_norm_err(acc, ref["acc"]) <= 1e-12
    assert abs(th[1] - ref["energy"]) <= 1e-12 * abs(ref["energy"])
    assert abs(th[5] - ref["virial"]) <= 1e-11 * abs(ref["virial"])
    counts, idx = sim.neighbors(True, RC)
    np.testing.assert_array_equal(counts, ref["counts"])
    np.testing.assert_array_equal(neighbor_hashes(counts, idx), ref["hash"])
    sim.close()


def test_lj_liquid_256k_mixed_matches_oracle(liquid, liquid_oracle):
    sim = lj_sim(liquid, "mixed", "verletlist", f"cutoff {RC!r} skin {0.3 * SIGMA!r} maxneighbors 256")
    sim.update_forces()
    _, _, acc = sim.atoms()
    th = sim.thermo_raw()
    ref = liquid_oracle
    assert rel_norm_err(acc, ref["acc"]) <= 1e-5
    assert abs(th[1] - ref["energy"]) <= 1e-6 * abs(ref["energy"])
    assert abs(th[5] - ref["virial"]) <= 1e-5 * abs(ref["virial"])
    # the pairs inside the cutoff, exactly the oracle's: the FP32 distance decides, and the
    # exact FP64 test takes over inside the guard band around rc^2 (shared with the force kernel)
    counts, idx = sim.neighbors(True, RC)
    np.testing.assert_array_equal(counts, ref["counts"])
    np.testing.assert_array_equal(neighbor_hashes(counts, idx), ref["hash"])
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lj_liquid_256k_momentum_is_conserved(liquid, precision):
    cm, args = (("linkedcell", lj_cells(liquid["L"])) if precision == "fp64" else
                ("verletlist", f"cutoff {RC!r} skin {0.3 * SIGMA!r} maxneighbors 256"))
    sim = lj_sim(liquid, precision, cm, args)
    sim.update_forces()
    _, v0, _ = sim.atoms()
    sim.do_steps(200 if precision == "mixed" else 20)
    _, v1, _ = sim.atoms()
    m = liquid["mass"][:, None]
    p0, p1 = (m * v0).sum(axis=0), (m * v1).sum(axis=0)
    scale = np.sqrt(np.sum(m * m * v0 * v0))  # the momentum a random sum of the atoms' would have
    # full-list gathers evaluate each pair twice, once from each side: in FP64 the two forces are
    # exact negatives; the FP32 pair maths of the mixed path leaves a rounding-level residue
    tol = 1e-12 if precision == "fp64" else 1e-5
    assert np.abs(p1 - p0).max() <= tol * scale
    sim.close()


def test_sc_cu_495k_matches_oracle():
    w = I.sc_cu_system(50, seed=3)
    c = I.SC_CU
    n = int(round(float(w["L"][0]) / (2 * c["a"])))
    cm_args = f"cutoff {2 * c['a']!r} nx {n} ny {n} nz {n}"
    sc = f"e {c['e']} a {c['a']} n {c['n']} m {c['m']} c {c['c']} cutoff {2 * c['a']!r}"

    def make(precision):
        sim = gbmd.Simulation(w["natoms"], w["L"])
        sim.set_atoms(w["pos"], w["vel"], Z=w["Z"], mass=w["mass"])
        sim.set_cell_manager(gbmd.Plugin("linkedcell", cm_args))
        sim.add_potential(gbmd.Plugin("suttonchen", sc))
        sim.set_integrator(gbmd.Plugin("velocityverlet", "dt 2.0"))
        sim.set_precision(precision)
        return sim

    # a thermalised state: 20 FP64 steps from the lattice (on the lattice the forces are zero
    # but for the vacancies' neighbours)
    run = make("fp64")
    run.update_forces()
    run.do_steps(20)
    pos, vel, _ = run.atoms()
    run.close()
    ref = oracle.PortSim(pos, w["L"], np.full(w["natoms"], w["Z"]), w["mass"], vel)
    ref.set_cell_manager("linkedcell", cm_args)
    ref.add_potential("suttonchen", sc)
    ref.update_forces()
    _, _, acc_ref = ref.atoms()
    e_ref, w_ref = ref.energy(), ref.virial()
    for precision, (tf, te, tw) in (("fp64", (1e-12, 1e-12, 1e-11)), ("mixed", (1e-5, 1e-6, 1e-5))):
        sim = make(precision)
        sim.set_atoms(pos, vel, Z=w["Z"], mass=w["mass"])
        sim.update_forces()
        _, _, acc = sim.atoms()
        th = sim.thermo_raw()
        assert rel_norm_err(acc, acc_ref) <= tf, precision
        assert abs(th[1] - e_ref) <= te * abs(e_ref), precision
        assert abs(th[5] - w_ref) <= tw * abs(w_ref), precision
        sim.close()


def test_ensemble_512_systems_match_their_runs_alone():
    systems = I.lj_ensemble(512, seed=4)
    skin = 0.3 * SIGMA

    def setup(obj):
        obj.set_cell_manager(gbmd.Plugin("verletlist", f"cutoff {RC!r} skin {skin!r} maxneighbors 512"))
        obj.add_potential(gbmd.Plugin("lennardjones", LJ))
        obj.set_integrator(gbmd.Plugin("velocityverlet", "dt 10.0"))
        obj.set_precision("mixed")
        obj.update_forces()
        obj.do_steps(30)

    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
    for k, s in enumerate(systems):
        b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    setup(b)
    sizes = np.array([s["natoms"] for s in systems])
    for k in sorted({int(np.argmin(sizes)), int(np.argmax(sizes)), 255}):
        s = systems[k]
        alone = gbmd.Batch([s["natoms"]], [s["L"]])
        alone.set_atoms(0, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
        setup(alone)
        for x, y in zip(b.atoms(k), alone.atoms(0)):
            np.testing.assert_array_equal(x, y)
        alone.close()
    b.close()
