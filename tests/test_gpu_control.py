"""The control file of the small Lennard-Jones argon case, run by the control-file runner on the
GPU, against the reference's own run of the same system (golden fixture lj_ar_fcc10: FCC 10^3,
linkedcell nx 6, velocityverlet dt 1 fs, 100 steps, FP64)."""
import numpy as np
import pytest

from helpers import load_golden, rel_norm_err

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")
from lpmd2_gb300 import control as C  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0:
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def control_text(L: float) -> str:
    return f"""
cell cubic {L!r}
input crystal3d type=fcc symbol=Ar nx=10 ny=10 nz=10
prepare temperature t=100.0 seed=1
steps 100
monitor step,potential-energy,kinetic-energy,temperature each=1 output=monitor.dat
output xyz last.xyz each=100 level=1
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
cellmanager linkedcell
potential lennardjones Ar Ar
integrator velocityverlet
"""


def test_ar_fcc10_control_file_matches_reference_run(tmp_path):
    g = load_golden("lj_ar_fcc10")
    L = g["L"]
    ctl = C.parse(control_text(float(L[0])), strict=True)
    out = C.run(ctl, precision="fp64", workdir=tmp_path)
    assert out["natoms"] == len(g["pos_in"])
    d = out["pos"] - g["pos"]
    d -= L * np.round(d / L)
    assert np.max(np.abs(d)) <= 1e-9 * L.max()
    assert rel_norm_err(out["vel"], g["vel"]) <= 1e-9
    rows = np.array(out["rows"])
    assert rows.shape == (100, 4)
    np.testing.assert_array_equal(rows[:, 0], np.arange(1, 101))
    for k, col in ((1, 1), (2, 2), (3, 4)):  # Epot, Ekin, T against the reference's per-step values
        np.testing.assert_allclose(rows[:, k], g["thermo"][:, col], rtol=1e-9, atol=1e-12)
    assert len((tmp_path / "monitor.dat").read_text().splitlines()) == 100
    xyz = (tmp_path / "last.xyz").read_text().splitlines()
    assert int(xyz[0]) == 4000 and len(xyz) == 4002 and xyz[2].startswith("Ar ")


CU_TEXT = """
cell crystal 14.44
input crystal3d type=fcc symbol=Cu nx=4 ny=4 nz=4
output module=lpmd file=cu.zlp level=2 each=50
output xyz cu.xyz level=1 each=100
monitor step,temperature,total-energy start=0 each=10 end=-1 output=props.dat
prepare temperature t=300
steps 100
use velocityverlet
 dt 1.0
enduse
use suttonchen
 e 0.015713
 n 9.0
 m 6.0
 a 3.61
 c 39.755
 cutoff 6.0
enduse
use linkedcell
 cutoff 7.0
 mode auto
enduse
use tempscaling
 from 300.0
 to 300.0
enduse
potential suttonchen Cu Cu
integrator velocityverlet
cellmanager linkedcell
apply tempscaling start=0 end=100 each=20
"""


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sutton_chen_control_file_with_thermostat_and_frames(precision, tmp_path):
    from lpmd2_gb300 import formats as F

    ctl = C.parse(CU_TEXT, strict=True)
    np.testing.assert_array_equal(ctl.cell, [14.44, 14.44, 14.44])  # `cell crystal a` is cubic
    out = C.run(ctl, precision=precision, workdir=tmp_path)
    n = out["natoms"]
    m = np.full(n, C.STANDARD_MASS["Cu"])
    ke = 0.5 * np.sum(m * np.sum(out["vel"] ** 2, axis=1)) * 103.64269
    assert abs((2.0 / 3.0) * ke / (8.6173422e-05 * n) / 300.0 - 1.0) < 1e-11  # rescaled at step 100
    frames = F.read_lpmd(tmp_path / "cu.zlp")
    assert len(frames) == 2 and all(f["symbols"] == ["Cu"] * n for f in frames)
    last = frames[-1]
    assert np.abs(last["pos"] - out["pos"]).max() <= 0.5e-6 * 14.44 * (1 + 1e-9)
    # the frame is written after the modifier (SaveCurrentConfiguration follows RunModifiers)
    assert np.abs(last["vel"] - out["vel"]).max() <= 0.5e-6 * (1 + 1e-9)
    assert np.abs(last["acc"] - out["acc"]).max() <= 0.5e-6 * (1 + 1e-9)
    xyz = F.read_xyz(tmp_path / "cu.xyz")
    assert len(xyz) == 1 and xyz[0]["level"] == 1
    assert np.abs(xyz[0]["pos"] - out["pos"]).max() <= 0.5e-8 * 16
    rows = np.loadtxt(tmp_path / "props.dat")
    assert list(rows[:, 0]) == list(range(10, 101, 10))


def test_input_from_an_lpmd_file(tmp_path):
    from lpmd2_gb300 import formats as F

    g = load_golden("lj_ar_fcc10")
    L = np.asarray(g["L"], float)
    w = F.LPMDWriter(tmp_path / "start.lpmd", level=1)
    w.write_header()
    w.write_frame("Ar", L, g["pos_in"], g["vel_in"])
    w.close()
    text = control_text(float(L[0])).replace("input crystal3d type=fcc symbol=Ar nx=10 ny=10 nz=10",
                                             "input module=lpmd file=start.lpmd")
    text = text.replace("prepare temperature t=100.0 seed=1\n", "")
    out = C.run(C.parse(text, strict=True), precision="fp64", workdir=tmp_path)
    fr = F.read_lpmd(tmp_path / "start.lpmd")[0]
    sim = gbmd.Simulation(len(fr["pos"]), L)
    sim.set_atoms(fr["pos"], fr["vel"], Z=g["Z"], mass=g["mass"])
    sim.set_cell_manager(gbmd.Plugin("linkedcell", "cutoff 8.5 nx 6 ny 6 nz 6"))
    sim.add_potential(gbmd.Plugin("lennardjones", "sigma 3.405 epsilon 0.0103 cutoff 8.5"), 18, 18)
    sim.set_integrator(gbmd.Plugin("velocityverlet", "dt 1.0"))
    sim.set_precision("fp64")
    sim.update_forces()
    sim.do_steps(100)
    p, v, _ = sim.atoms()
    np.testing.assert_array_equal(out["pos"], p)
    np.testing.assert_array_equal(out["vel"], v)


def test_control_file_with_sibling_plugins_matches_the_api(tmp_path):
    # gupta + lcbinary + beeman from a control file = the same plugins through the API
    text = """
cell cubic 16.32
input crystal3d type=fcc symbol=Au nx=4 ny=4 nz=4
prepare temperature t=300.0 seed=3
steps 25
use gupta
 A 0.2061
 r0 2.884
 p 10.229
 B 1.790
 q 4.036
 cutoff 6.0
enduse
use lcbinary
 cutoff 6.0
 mode auto
enduse
use beeman
 dt 2.0
enduse
potential gupta Au Au
cellmanager lcbinary
integrator beeman
"""
    ctl = C.parse(text, strict=True)
    out = C.run(ctl, precision="fp64", workdir=tmp_path)
    from lpmd2_gb300 import inputs as I

    L = np.full(3, 16.32)
    pos = C.crystal3d("fcc", 4, 4, 4, L)
    n = len(pos)
    mass = np.full(n, C.STANDARD_MASS["Au"])
    vel = I.maxwell_boltzmann(mass, 300.0, seed=3)
    sim = gbmd.Simulation(n, L)
    sim.set_atoms(pos, vel, Z=np.full(n, 79, dtype=np.int32), mass=mass)
    sim.set_cell_manager(gbmd.Plugin("lcbinary", "cutoff 6.0 mode auto"))
    sim.add_potential(gbmd.Plugin("gupta", "A 0.2061 r0 2.884 p 10.229 B 1.790 q 4.036 cutoff 6.0"), 79, 79)
    sim.set_integrator(gbmd.Plugin("beeman", "dt 2.0"))
    sim.set_precision("fp64")
    sim.update_forces()
    sim.do_steps(25)
    p, v, _ = sim.atoms()
    np.testing.assert_array_equal(out["pos"], p)
    np.testing.assert_array_equal(out["vel"], v)


def test_dump_restore_continues_from_the_dumped_step(tmp_path):
    from lpmd2_gb300 import formats as F

    g = load_golden("lj_ar_fcc10")
    L = float(np.asarray(g["L"])[0])
    base = control_text(L).replace("steps 100", "steps 20").replace("output xyz last.xyz each=100 level=1\n", "")
    base = base.replace("monitor step,potential-energy,kinetic-energy,temperature each=1 output=monitor.dat",
                        "monitor step,temperature each=1 output=monitor.dat")
    first = C.run(C.parse(base + "set dumping-each 8\nset dumping-file every8.dump\n", strict=True),
                  precision="fp64", workdir=tmp_path)
    d = F.read_dump(tmp_path / "lastconfig.dump")
    assert d["step"] == 20
    np.testing.assert_allclose(d["pos"], first["pos"], rtol=5e-6)
    assert F.read_dump(tmp_path / "every8.dump")["step"] == 16  # Stepper(0, 20, 8): 8, 16
    # a second control file restores the dump and runs on to step 35
    second = base.replace("steps 20", "steps 35") + "set restore-file lastconfig.dump\nset lastconfig final.dump\n"
    out = C.run(C.parse(second, strict=True), precision="fp64", workdir=tmp_path)
    rows = np.loadtxt(tmp_path / "monitor.dat")
    assert list(rows[:, 0]) == list(range(21, 36))
    assert F.read_dump(tmp_path / "final.dump")["step"] == 35
    sim = gbmd.Simulation(len(d["pos"]), d["L"])
    sim.set_atoms(d["pos"], d["vel"], Z=d["Z"], mass=g["mass"])
    sim.set_cell_manager(gbmd.Plugin("linkedcell", "cutoff 8.5 nx 6 ny 6 nz 6"))
    sim.add_potential(gbmd.Plugin("lennardjones", "sigma 3.405 epsilon 0.0103 cutoff 8.5"), 18, 18)
    sim.set_integrator(gbmd.Plugin("velocityverlet", "dt 1.0"))
    sim.set_precision("fp64")
    sim.update_forces()
    sim.do_steps(15)
    p, v, _ = sim.atoms()
    np.testing.assert_array_equal(out["pos"], p)
    np.testing.assert_array_equal(out["vel"], v)


@pytest.mark.parametrize("name", ["argon_liquid.control", "copper_thermostat.control"])
def test_example_control_files_run(name, tmp_path):
    from pathlib import Path

    text = (Path(__file__).resolve().parents[1] / "examples" / name).read_text()
    text = "\n".join("steps 60" if ln.startswith("steps ") else ln for ln in text.splitlines())
    ctl = C.parse(text, strict=True)
    out = C.run(ctl, workdir=tmp_path)
    assert np.isfinite(out["pos"]).all() and np.isfinite(out["thermo"]["total_energy"])
    assert (tmp_path / ctl.options.get("lastconfig", "lastconfig.dump")).exists()
