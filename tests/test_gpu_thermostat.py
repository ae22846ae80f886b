"""Thermostats between steps (gbmd_*_scale_velocities) against host arithmetic on the velocities
read back from the device.

SetTemperature (liblpmd/simulation/simulationbuilder.cc:53-72, the tempscaling and temperature
modifiers) measures T over the atoms without fixedvel/fixedpos when any atom has one of them
and scales only those atoms by sqrt(target/T); Berendsen (plugins/berendsen.cc:72-99) measures
T over all atoms and scales every atom by sqrt(1 + dt/tau (target/T - 1)).  The step's thermo
record is left as the step reported it, and the next step continues from the rescaled
velocities exactly as a fresh run started from them does.
"""
import numpy as np
import pytest

from helpers import load_golden, rel_norm_err
from lpmd2_gb300 import inputs as I

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")
from lpmd2_gb300 import control as C  # noqa: E402

KIN2EV, KB = 103.64269, 8.6173422e-05
# The device sums kinetic energy in int64 units of 2^-44 amu A^2/fs^2 (each warp's FP64 sum
# rounded once): for the small systems here that is ~1e-12 of the total, which bounds the
# relative error of T and of the scaling factor.
TOL = 1e-11


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def make_sim(g, precision, pos=None, vel=None):
    sim = gbmd.Simulation(len(g["pos_in"]), g["L"])
    sim.set_atoms(g["pos_in"] if pos is None else pos, g["vel_in"] if vel is None else vel, Z=g["Z"], mass=g["mass"])
    sim.set_cell_manager(gbmd.Plugin(str(g["cm"]), str(g["cm_args"])))
    for name, args, spc in zip(g["pot_names"], g["pot_args"], g["pot_species"]):
        sim.add_potential(gbmd.Plugin(str(name), str(args)), int(spc[0]), int(spc[1]))
    sim.set_integrator(gbmd.Plugin("velocityverlet", f"dt {float(g['dt'])!r}"))
    sim.set_precision(precision)
    return sim


def temperature(v, m, mask=None):
    """lpmd::Temperature (liblpmd/lpmd/properties.h:40-53) over the atoms in mask."""
    if mask is None:
        mask = np.ones(len(v), bool)
    ke = 0.5 * np.sum(m[mask] * np.sum(v[mask] ** 2, axis=1)) * KIN2EV
    return (2.0 / 3.0) * ke / (KB * mask.sum())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["lj_liquid_vl", "sc_cu"])
def test_set_temperature_factor(case, precision):
    g = load_golden(case)
    m = np.asarray(g["mass"], float) * np.ones(len(g["pos_in"]))
    sim = make_sim(g, precision)
    sim.update_forces()
    sim.do_steps(7)
    th = sim.thermo_raw().copy()
    p0, v0, a0 = sim.atoms()
    target = 0.5 * temperature(v0, m)
    sim.set_temperature(target)
    p1, v1, a1 = sim.atoms()
    f = np.sqrt(target / temperature(v0, m))
    assert rel_norm_err(v1, f * v0) < TOL
    assert abs(temperature(v1, m) / target - 1.0) < TOL
    np.testing.assert_array_equal(p1, p0)
    np.testing.assert_array_equal(a1, a0)
    # the step's record is what the step reported (lpmd's monitor prints those tags)
    np.testing.assert_array_equal(sim.thermo_raw(), th)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_set_temperature_skips_tagged_atoms_and_berendsen_does_not(precision):
    g = load_golden("lj_liquid_vl")
    n = len(g["pos_in"])
    m = np.asarray(g["mass"], float) * np.ones(n)
    flags = np.zeros(n, np.uint8)
    flags[::7] = gbmd.FLAG_FIXEDVEL
    flags[3::11] = gbmd.FLAG_FIXEDPOS
    tagged = flags != 0
    sim = make_sim(g, precision)
    sim.set_flags(flags)
    sim.update_forces()
    sim.do_steps(5)
    _, v0, _ = sim.atoms()
    t_free = temperature(v0, m, ~tagged)
    sim.set_temperature(120.0)
    _, v1, _ = sim.atoms()
    np.testing.assert_array_equal(v1[tagged], v0[tagged])
    assert rel_norm_err(v1[~tagged], np.sqrt(120.0 / t_free) * v0[~tagged]) < TOL
    # Berendsen: T over all atoms, every atom scaled
    dt_over_tau = 1.0 / 40.0
    t_all = temperature(v1, m)
    sim.berendsen(300.0, dt_over_tau)
    _, v2, _ = sim.atoms()
    xi = np.sqrt(1.0 + dt_over_tau * (300.0 / t_all - 1.0))
    assert rel_norm_err(v2, xi * v1) < TOL
    assert not np.array_equal(v2[tagged], v1[tagged])


def test_rescaled_run_continues_as_a_fresh_run():
    # linked cells: the FP64 force sums depend on positions only, not on a list's history
    g = load_golden("lj_ar_fcc10")
    a = make_sim(g, "fp64")
    a.update_forces()
    a.do_steps(10)
    a.set_temperature(250.0)
    p, v, _ = a.atoms()
    a.do_steps(15)
    b = make_sim(g, "fp64", pos=p, vel=v)
    b.update_forces()
    b.do_steps(15)
    pa, va, _ = a.atoms()
    pb, vb, _ = b.atoms()
    L = np.asarray(g["L"], float)
    d = pa - pb
    d -= L * np.round(d / L)
    assert np.abs(d).max() < 1e-10
    assert rel_norm_err(va, vb) < 1e-10


def test_batch_scales_one_system_or_all():
    systems = [I.lj_system(4, 0.9, 1.5, seed=71), I.lj_system(5, 0.8, 1.0, seed=72)]
    sigma = I.LJ_AR["sigma"]
    rc = 2.5 * sigma
    b = gbmd.Batch([s["natoms"] for s in systems], [s["L"] for s in systems])
    for k, s in enumerate(systems):
        b.set_atoms(k, s["pos"], s["vel"], Z=s["Z"], mass=s["mass"])
    b.set_cell_manager(gbmd.Plugin("verletlist", f"cutoff {rc!r} skin {0.3 * sigma!r} maxneighbors 256"))
    b.add_potential(gbmd.Plugin("lennardjones", f"sigma {sigma} epsilon {I.LJ_AR['epsilon']} cutoff {rc!r}"))
    b.set_integrator(gbmd.Plugin("velocityverlet", "dt 5.0"))
    b.set_precision("mixed")
    b.update_forces()
    b.do_steps(6)
    v0 = [b.atoms(k)[1] for k in range(2)]
    b.set_temperature(60.0, sys=1)
    v1 = [b.atoms(k)[1] for k in range(2)]
    np.testing.assert_array_equal(v1[0], v0[0])
    m1 = systems[1]["mass"]
    assert abs(temperature(v1[1], m1) / 60.0 - 1.0) < TOL
    b.berendsen(90.0, 0.1)
    v2 = [b.atoms(k)[1] for k in range(2)]
    for k in range(2):
        t = temperature(v1[k], systems[k]["mass"])
        assert rel_norm_err(v2[k], np.sqrt(1.0 + 0.1 * (90.0 / t - 1.0)) * v1[k]) < TOL
    b.do_steps(4)
    assert all(np.isfinite(b.atoms(k)[0]).all() for k in range(2))


def test_control_file_thermostat(tmp_path):
    g = load_golden("lj_ar_fcc10")
    L = float(np.asarray(g["L"])[0])
    text = f"""
cell cubic {L!r}
input crystal3d type=fcc symbol=Ar nx=10 ny=10 nz=10
prepare temperature t=100.0 seed=1
steps 20
monitor step,temperature each=1 output=monitor.dat
use lennardjones
    sigma 3.405
    epsilon 0.0103
    cutoff 8.5
enduse
use linkedcell
    cutoff 8.5
    nx 6
    ny 6
    nz 6
enduse
use velocityverlet
    dt 1.0
enduse
use temperature
    t 150.0
enduse
cellmanager linkedcell
potential lennardjones Ar Ar
integrator velocityverlet
apply temperature start=10 each=10
"""
    ctl = C.parse(text, strict=True)
    assert [s for s, *_ in C.modifier_schedule(ctl, 1.0)] == [10, 20]
    out = C.run(ctl, precision="fp64", workdir=tmp_path)
    m = np.full(out["natoms"], C.STANDARD_MASS["Ar"])
    # the run ends with a rescaling to 150 K ...
    assert abs(temperature(out["vel"], m) / 150.0 - 1.0) < TOL
    # ... while the monitor shows the temperatures the steps reported, before the modifier
    rows = np.asarray(out["rows"])
    assert rows[-1][0] == 20 and abs(rows[-1][1] / 150.0 - 1.0) > 1e-6
    # after the step-10 rescaling the system starts from 150 K
    assert abs(rows[10][1] - 150.0) < 0.2 * 150.0
