"""gbmd_pair_forces_static: pair forces for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc at the point where they need forces: a host program that
hands its whole device memory budget to its own pool allocator up front, or a latency-bound
loop that cannot afford an allocation's implicit synchronisation.  The static entry point
takes positions, forces and sums in buffers the caller owns and keeps its only scratch in a
fixed array inside the library.

Checked through the C ABI, on two calls in a row, against (1) the existing simulation entry
point (gbmd_sim_* with the minimumimage cell manager, FP64) to 1e-12 relative, and (2) the
oracle's restatement of the reference's minimum-image pair forces on the same positions, to
1e-12 relative.  The second call of each pair must not see anything the first one left in the
shared scratch array: the calls differ in positions and, in the second test, in size (16,384
atoms, the array's capacity, then 864).  The file sorts last so that it also runs after every
other GPU test in one session; it needs nothing from them and passes alone in a fresh process.
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
oracle = pytest.importorskip("oracle")

FORCEFACTOR = 0.00964853  # eV/A/amu -> A/fs^2, the session's "forcefactor"
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists() or not oracle.PORT_LIB.exists():
        import __graft_entry__

        __graft_entry__.build()
    if gbmd.device_count() == 0 or not torch.cuda.is_available():
        pytest.fail("no CUDA device: the GPU tests need a GB300")


def _system(k, seed):
    """FCC k^3 argon at liquid density, jittered by up to 0.35 A (4k^3 atoms)."""
    a = (4.0 / 0.8442) ** (1.0 / 3.0) * 3.405
    pos, L = I.fcc_fast(k, k, k, a)
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


def _oracle_path(pos, L):
    """The same quantities from the oracle's minimum-image restatement of the reference."""
    n = len(pos)
    mass = np.full(n, I.MASSES["Ar"])
    ref = oracle.run_port(pos, L, np.full(n, 18), mass, np.zeros_like(pos), "minimumimage", "cutoff 8.5",
                          [("lennardjones", LJ_AR, -1, -1)], 1.0, 0)
    th = ref["thermo0"]
    force = ref["acc0"] / (FORCEFACTOR / mass)[:, None]
    return force, th[1], th[5], th[13:22]


def _static_path(pos, L, pot, force_d, out_d, stream):
    n = len(pos)
    pos_d = torch.from_numpy(np.ascontiguousarray(pos).ravel()).to("cuda")
    force_d[: 3 * n].fill_(float("nan"))  # every entry the call owns must be written by it
    out_d.fill_(float("nan"))
    # the upload and the fills above were queued on torch's current stream; the library's
    # kernels go to `stream`, which must not start before them
    stream.wait_stream(torch.cuda.current_stream())
    gbmd.pair_forces_static(pot, pos_d.data_ptr(), n, L, force_d.data_ptr(), out_d.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    return force_d[: 3 * n].cpu().numpy().reshape(-1, 3).copy(), out_d.cpu().numpy().copy()


def _check(f, out, expect):
    f_ref, e_ref, w_ref, s_ref = expect
    assert np.all(np.isfinite(f)) and np.all(np.isfinite(out))
    assert rel_norm_err(f, f_ref) <= TOL
    assert abs(out[0] - e_ref) <= TOL * abs(e_ref)
    assert abs(out[1] - w_ref) <= TOL * abs(w_ref)
    assert np.max(np.abs(out[2:] - s_ref)) <= TOL * np.max(np.abs(s_ref))


def _static_max() -> int:
    text = (Path(__file__).resolve().parents[1] / "include" / "gbmd.h").read_text()
    return int(re.search(r"#define GBMD_STATIC_MAX_ATOMS (\d+)", text).group(1))


def _run_calls(cases):
    pot = gbmd.Plugin("lennardjones", LJ_AR)
    stream = torch.cuda.Stream()
    nmax = max(4 * k ** 3 for k, _ in cases)
    force_d = torch.empty(3 * nmax, dtype=torch.float64, device="cuda")
    out_d = torch.empty(11, dtype=torch.float64, device="cuda")
    for k, seed in cases:
        pos, L = _system(k, seed)
        f, out = _static_path(pos, L, pot, force_d, out_d, stream)
        _check(f, out, _simulation_path(pos, L, pot))
        _check(f, out, _oracle_path(pos, L))


def test_static_matches_simulation_and_oracle_on_two_calls():
    _run_calls([(6, 11), (6, 12)])  # 864 atoms, two different configurations


def test_static_at_capacity_then_small():
    # 16^3 FCC = 16,384 atoms fills the scratch array (128 blocks); the 864-atom call after it
    # reduces over 7 blocks and must not pick up the larger call's partial sums
    assert 4 * 16 ** 3 == _static_max()
    _run_calls([(16, 13), (6, 14)])


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
