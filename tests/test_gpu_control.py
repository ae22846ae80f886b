"""The control file of the small Lennard-Jones argon case, run by the control-file runner on the
GPU, against the reference's own run of the same system (golden fixture lj_config1: FCC 10^3,
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


def test_config1_control_file_matches_reference_run(tmp_path):
    g = load_golden("lj_config1")
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
