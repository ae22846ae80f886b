"""CPU tests of the C ABI and the host-side plugin logic (no GPU needed).

The library must load without a GPU, export every entry point declared in include/gbmd.h,
parse plugin arguments with LPMD's Module semantics (liblpmd/plugins/module.cc:77-103) and
evaluate the potential functionals on the host exactly as the reference plugins do.
"""
import math
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from helpers import FS_FE, FSX_MO, GUPTA_AU, LJ_AR, SC_CU
from lpmd2_gb300 import gbmd

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not gbmd.LIB_PATH.exists():
        import __graft_entry__

        __graft_entry__.build()
    if not oracle.PORT_LIB.exists():
        oracle.build()


def _declared():
    text = (ROOT / "include" / "gbmd.h").read_text()
    return sorted(set(re.findall(r"^[a-z_ ]+?\**\s*(gbmd_[a-z_0-9]+)\(", text, flags=re.M)))


def test_exports_every_declared_symbol():
    import ctypes

    lib = ctypes.CDLL(str(gbmd.LIB_PATH))
    declared = _declared()
    assert len(declared) >= 40
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(gbmd.exported_symbols()) == declared


def test_abi_version_and_no_gpu_behaviour():
    lib = gbmd.load()
    assert lib.gbmd_abi_version() == 1
    if gbmd.device_count() == 0:
        with pytest.raises(gbmd.GbmdError) as e:
            gbmd.Simulation(10, [10.0, 10.0, 10.0])
        assert e.value.status == gbmd.ERR_CUDA
        assert "no CUDA device" in str(e.value)


def test_plugin_arguments_and_defaults():
    lc = gbmd.Plugin("linkedcell", "cutoff 8.5 nx 6 ny 6 nz 6")
    assert lc.kind == gbmd.KIND_CELLMANAGER
    assert lc["nx"] == "6" and lc["mode"] == "noauto" and lc["warn-outside"] == "true"
    assert lc.cutoff() == 8.5
    vl = gbmd.Plugin("verletlist", "cutoff 8.5")
    assert vl["maxneighbors"] == "80" and vl["each"] == "5" and vl["extcutoff"] == "0.0"
    vv = gbmd.Plugin("velocityverlet", "")
    assert vv["dt"] == "1.0" and vv.kind == gbmd.KIND_INTEGRATOR
    sc = gbmd.Plugin("suttonchen", SC_CU)
    assert sc["corrections"] == "false" and sc.cutoff() == 7.22
    fs = gbmd.Plugin("finnissinclair", FS_FE)
    assert fs.cutoff() == 3.569745  # max(c, d), plugins/finnissinclair.cc:27-30
    # a keyword given twice keeps the last value (ParamList assignment order)
    assert gbmd.Plugin("lennardjones", "sigma 1 sigma 2 epsilon 1 cutoff 3")["sigma"] == "2"
    # missing keywords read as empty -> 0
    assert gbmd.Plugin("lennardjones", "cutoff 3")["sigma"] == ""


def test_plugin_errors():
    with pytest.raises(SyntaxError, match="Unexpected end of input"):
        gbmd.Plugin("linkedcell", "cutoff 8.5 nx")
    with pytest.raises(gbmd.PluginError):
        gbmd.Plugin("ewald", "")
    with pytest.raises(gbmd.PluginError):
        gbmd.Plugin("lennardjones", LJ_AR + " precision half")


def _two_atom_force(name, args, r, mass=39.948):
    """Force on atom 0 from atom 1 at distance r along x, from the oracle (acc * m / ff)."""
    L = [60.0, 60.0, 60.0]
    pos = np.array([[10.0, 10.0, 10.0], [10.0 + r, 10.0, 10.0]])
    out = oracle.run_port(pos, L, [1, 1], [mass, mass], None, "minimumimage", "cutoff 20",
                          [(name, args, -1, -1)], 1.0, 0)
    return out["acc0"][0] * mass / 0.00964853, out["thermo0"][1]


@pytest.mark.parametrize("r", [3.2, 3.8, 5.0, 8.4])
def test_lj_functionals_match_oracle(r):
    p = gbmd.Plugin("lennardjones", LJ_AR)
    f, e = _two_atom_force("lennardjones", LJ_AR, r)
    assert p.pair_energy(r) == pytest.approx(e, rel=1e-14)
    np.testing.assert_allclose(p.pair_force([r, 0.0, 0.0]), f, rtol=1e-13)


@pytest.mark.parametrize("spec", [("suttonchen", SC_CU, 2.6), ("suttonchen", SC_CU, 5.1),
                                  ("finnissinclair", FS_FE, 2.5), ("finnissinclair-ext", FSX_MO, 2.9),
                                  ("gupta", GUPTA_AU, 2.7), ("gupta", GUPTA_AU, 4.9)])
def test_metal_functionals_match_oracle(spec):
    name, args, r = spec
    p = gbmd.Plugin(name, args)
    f, e = _two_atom_force(name, args, r)
    rho = p.rhoij(r)
    # E = V(r) + 2 F(rho(r)); force = PairForce + ManyBodies(rho, rho)
    assert p.pair_energy(r) + 2.0 * p.F(rho) == pytest.approx(e, rel=1e-13)
    fv = p.pair_force([r, 0.0, 0.0]) + p.many_bodies([r, 0.0, 0.0], rho, rho)
    np.testing.assert_allclose(fv, f, rtol=1e-12, atol=1e-14)


def test_sutton_chen_closed_form():
    p = gbmd.Plugin("suttonchen", SC_CU)
    e, a, n, m, c = 0.012382, 3.61, 9, 6, 39.432
    r = 3.0
    assert p.pair_energy(r) == pytest.approx(e * (a / r) ** n, rel=1e-14)
    assert p.rhoij(r) == pytest.approx((a / r) ** m, rel=1e-14)
    assert p.F(2.0) == pytest.approx(-c * e * math.sqrt(2.0), rel=1e-15)


def test_gupta_closed_form():
    # plugins/gupta.cc:52-70 (Cleri-Rosato second-moment form)
    A, r0, pp, B, q = 0.2061, 2.884, 10.229, 1.790, 4.036
    p = gbmd.Plugin("gupta", GUPTA_AU)
    assert p.cutoff() == 6.0
    r = 3.1
    assert p.pair_energy(r) == pytest.approx(A * math.exp(-pp * (r / r0 - 1)), rel=1e-14)
    assert p.rhoij(r) == pytest.approx(math.exp(-2 * q * (r / r0 - 1)), rel=1e-14)
    assert p.F(2.0) == pytest.approx(-B * math.sqrt(2.0), rel=1e-15)
    f = p.pair_force([r, 0.0, 0.0])
    assert f[0] == pytest.approx(-(A * pp / r0) * math.exp(-pp * (r / r0 - 1)), rel=1e-14)
    mb = p.many_bodies([0.0, r, 0.0], 2.0, 3.0)
    want = (B * q / r0) * (1 / math.sqrt(2.0) + 1 / math.sqrt(3.0)) * math.exp(-2 * q * (r / r0 - 1))
    assert mb[1] == pytest.approx(want, rel=1e-14) and mb[0] == 0.0
    with pytest.raises(SyntaxError, match="Unexpected end of input"):
        gbmd.Plugin("gupta", "A 1 r0 2 p 3 B 4 q")  # a keyword without a value


@pytest.mark.parametrize("r", [3.3, 3.81, 6.0, 8.49])
def test_fastlj_functionals_are_the_table_steps(r):
    # plugins/fastlj.cc:38-73: LJ at the lower edge of bin floor(bins r / cutoff)
    sigma, eps, rc, bins = 3.405, 0.0103, 8.5, 500
    p = gbmd.Plugin("fastlj", f"sigma {sigma} epsilon {eps} cutoff {rc}")
    assert p["bins"] == "500" and p.cutoff() == rc
    rk = rc * math.floor(bins * r / rc) / bins
    r6 = (sigma / rk) ** 6
    assert p.pair_energy(r) == pytest.approx(4 * eps * (r6 * r6 - r6), rel=1e-14)
    f = p.pair_force([0.0, 0.0, r])
    assert f[2] == pytest.approx(r * -48 * (eps / rk ** 2) * (r6 * r6 - 0.5 * r6), rel=1e-14)
    lj = gbmd.Plugin("lennardjones", f"sigma {sigma} epsilon {eps} cutoff {rc}")
    assert p.pair_energy(r) == pytest.approx(lj.pair_energy(rk), rel=1e-13)
