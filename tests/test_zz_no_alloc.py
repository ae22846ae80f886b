"""gbmd_pair_forces_static (pair forces without device allocation) against the simulation path.

Both go through the C ABI.  The simulation path (gbmd_sim_* with the minimumimage cell
manager, FP64) is the existing entry point; the static entry point must agree with it to
1e-12 relative on forces, pair energy, virial and stress, on two calls in a row with
different positions (the second call must not see anything the first one left behind).
The file sorts last so that it also runs after every other GPU test in one session.
"""
import re
from pathlib import Path

import numpy as np
import pytest

from helpers import LJ_AR, rel_norm_err
from lpmd2_gb300 import inputs as I

pytestmark = pytest.mark.gpu

gbmd = pytest.importorskip("lpmd2_gb300.gbmd")
torch = pytest.importorskip("torch")

FORCEFACTOR = 0.00964853  # eV/A/amu -> A/fs^2, the session's "forcefactor"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0 or not torch.cuda.is_available():
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def _system(seed):
    a = (4.0 / 0.8442) ** (1.0 / 3.0) * 3.405
    pos, L = I.fcc_fast(6, 6, 6, a)
    pos = np.mod(I.jitter(pos, 0.35, seed=seed), L)
    return pos, L


def _simulation_path(pos, L, pot):
    """Forces (eV/A), pair energy, virial and stress from gbmd_sim_* (minimumimage, FP64)."""
    n = len(pos)
    mass = np.full(n, I.MASSES["Ar"])
    sim = gbmd.Simulation(n, L)
    sim.set_atoms(pos, np.zeros_like(pos), Z=np.full(n, 18), mass=mass)
    sim.set_cell_manager(gbmd.Plugin("minimumimage", "cutoff 8.5"))
    sim.add_potential(pot)
    sim.set_integrator(gbmd.Plugin("velocityverlet", "dt 1.0"))
    sim.set_precision("fp64")
    sim.update_forces()
    _, _, acc = sim.atoms()
    th = sim.thermo()
    sim.close()
    force = acc / (FORCEFACTOR / mass)[:, None]
    return force, th["potential_energy"], th["virial"], th["stress"].ravel()


def _static_path(pos, L, pot, force_d, out_d, stream):
    pos_d = torch.from_numpy(np.ascontiguousarray(pos)).to("cuda")
    force_d.fill_(float("nan"))  # every entry must be written by the call
    out_d.fill_(float("nan"))
    gbmd.pair_forces_static(pot, pos_d.data_ptr(), len(pos), L, force_d.data_ptr(), out_d.data_ptr(),
                            stream.cuda_stream)
    stream.synchronize()
    return force_d.cpu().numpy().reshape(-1, 3).copy(), out_d.cpu().numpy().copy()


def test_static_matches_simulation_on_two_calls():
    pot = gbmd.Plugin("lennardjones", LJ_AR)
    stream = torch.cuda.Stream()
    n = 864
    force_d = torch.empty(3 * n, dtype=torch.float64, device="cuda")
    out_d = torch.empty(11, dtype=torch.float64, device="cuda")
    for seed in (11, 12):
        pos, L = _system(seed)
        assert len(pos) == n
        f_ref, e_ref, w_ref, s_ref = _simulation_path(pos, L, pot)
        f, out = _static_path(pos, L, pot, force_d, out_d, stream)
        assert np.all(np.isfinite(f)) and np.all(np.isfinite(out))
        assert rel_norm_err(f, f_ref) <= 1e-12
        assert abs(out[0] - e_ref) <= 1e-12 * abs(e_ref)
        assert abs(out[1] - w_ref) <= 1e-12 * abs(w_ref)
        assert np.max(np.abs(out[2:] - s_ref)) <= 1e-12 * np.max(np.abs(s_ref))


def _static_max() -> int:
    text = (Path(__file__).resolve().parents[1] / "include" / "gbmd.h").read_text()
    return int(re.search(r"#define GBMD_STATIC_MAX_ATOMS (\d+)", text).group(1))


def test_static_rejects_sizes_beyond_its_scratch():
    pot = gbmd.Plugin("lennardjones", LJ_AR)
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    L = np.array([100.0, 100.0, 100.0])
    for n in (0, _static_max() + 1):
        # rejected on the host before anything is launched, so the small buffers are never read
        with pytest.raises(gbmd.GbmdError, match="capacity of its fixed scratch array"):
            gbmd.pair_forces_static(pot, buf.data_ptr(), n, L, buf.data_ptr(), buf.data_ptr())


def test_static_rejects_many_body_potentials():
    pot = gbmd.Plugin("suttonchen", "e 0.012382 a 3.61 n 9 m 6 c 39.432 cutoff 7.22")
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    with pytest.raises(gbmd.GbmdError, match="only pair potentials"):
        gbmd.pair_forces_static(pot, buf.data_ptr(), 10, [20.0, 20.0, 20.0], buf.data_ptr(), buf.data_ptr())
