"""Pins the C restatement (oracle/oracle.c) against the reference.

The golden fixtures were produced by the reference plugins themselves (tests/golden/make_golden.py);
the geometry vectors and the 108-atom neighbour known-answer test come from the reference's own
unit tests (liblpmd/tests/orthogonalcelltest.unit:100-170, liblpmd/tests/simulationtest.unit:58-67)
and its linked-cell demo (liblpmd/demos/linkedcell.cc:66-121).  CPU only.
"""
import platform

import numpy as np
import pytest

import oracle
from helpers import GOLDEN_CASES, INTEG_CASES, load_golden, neighbor_hashes
from lpmd2_gb300 import inputs as I

EXACT = platform.machine() in ("x86_64", "AMD64")


@pytest.fixture(scope="module", autouse=True)
def _build():
    if not oracle.PORT_LIB.exists():
        oracle.build()


def _same(a, b, rtol=1e-12):
    if EXACT:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=1e-300)


def _replay(g):
    pots = [(str(n), str(a), int(s[0]), int(s[1]))
            for n, a, s in zip(g["pot_names"], g["pot_args"], g["pot_species"])]
    integ = (str(g["integ_name"]), str(g["integ_args"])) if "integ_name" in g else None
    return oracle.run_port(g["pos_in"], g["L"], g["Z"], g["mass"], g["vel_in"], str(g["cm"]),
                           str(g["cm_args"]), pots, float(g["dt"]), int(g["nsteps"]),
                           neigh=(bool(g["neigh_full"]), float(g["neigh_rcut"])), integrator=integ)


@pytest.mark.parametrize("case", GOLDEN_CASES + INTEG_CASES)
def test_port_matches_reference(case):
    g = load_golden(case)
    out = _replay(g)
    # neighbour sets: exact, as multisets, in the reference's per-atom order when stored
    np.testing.assert_array_equal(out["neigh_counts"], g["neigh_counts"])
    np.testing.assert_array_equal(neighbor_hashes(out["neigh_counts"], out["neigh_idx"]), g["neigh_hash"])
    if "neigh_idx" in g:
        np.testing.assert_array_equal(out["neigh_idx"], g["neigh_idx"])
    _same(out["acc0"], g["acc0"])
    pinned = ~np.isnan(g["thermo0"])
    _same(out["thermo0"][pinned], g["thermo0"][pinned])
    if int(g["nsteps"]):
        pinned = ~np.isnan(g["thermo"])
        _same(out["thermo"][pinned], g["thermo"][pinned])
        _same(out["pos"], g["pos"])
        _same(out["vel"], g["vel"])
        _same(out["acc"], g["acc"])


def test_kat108_neighbors():
    """liblpmd/demos/linkedcell.cc:66-121: 108-atom Ar FCC, L = 17.1191, linkedcell nx 1,
    rcut 4.15: every atom has 12 neighbours at 4.03501 +- 1e-4 and full = 2 x half."""
    L = 17.1191
    pos = I.fcc_centered(3, L)
    n = len(pos)
    sim = oracle.PortSim(pos, [L, L, L], np.full(n, 18), np.full(n, 39.948))
    sim.set_cell_manager("linkedcell", "cutoff 8.5 nx 1 ny 1 nz 1")
    full_c, full_i = sim.neighbors(True, 4.15)
    half_c, half_i = sim.neighbors(False, 4.15)
    assert np.all(full_c == 12)
    assert full_c.sum() == 2 * half_c.sum()
    owner = np.repeat(np.arange(n), full_c)
    d = np.array([np.linalg.norm(oracle.displacement([L] * 3, pos[i], pos[j])) for i, j in zip(owner, full_i)])
    assert np.all(np.abs(d - 4.03501) < 1e-4)
    assert np.all(owner != full_i)
    g = load_golden("kat108")
    np.testing.assert_array_equal(full_c, g["neigh_counts"])
    np.testing.assert_array_equal(full_i, g["neigh_idx"])


def test_fitted_inside_vectors():
    """liblpmd/tests/orthogonalcelltest.unit:100-121."""
    L = [20.0, 20.0, 20.0]
    for a, want in [((10.0, 10.0, 10.0), (10.0, 10.0, 10.0)), ((22.0, 23.0, 24.0), (2.0, 3.0, 4.0)),
                    ((-3.0, -7.0, -4.0), (17.0, 13.0, 16.0)), ((63.0, 65.0, 61.0), (3.0, 5.0, 1.0)),
                    ((-83.0, -87.0, -84.0), (17.0, 13.0, 16.0))]:
        assert np.linalg.norm(oracle.fitted_inside(L, a) - np.array(want)) < 1e-10


def test_displacement_vectors():
    """liblpmd/tests/orthogonalcelltest.unit:130-162, with a seeded RandomVector."""
    L = [10.0, 10.0, 10.0]
    rng = I.uniform(11, 6000).reshape(-1, 2, 3) * 2.0 - 1.0
    center = np.array([5.0, 5.0, 5.0])
    for w in rng[:1000]:
        a = center + 4.95 * w[0] / np.linalg.norm(w[0])
        b = center + 4.95 * w[1] / np.linalg.norm(w[1])
        d = oracle.displacement(L, a, b)
        # a + d equals b up to a lattice vector (the unit test's "a + d - b = 0" holds
        # whenever no component of b - a reaches half a box length)
        r = a + d - b
        assert np.all(np.abs(r - 10.0 * np.round(r / 10.0)) < 1e-10)
        assert np.all(np.abs(d) <= 5.0)
        if np.all(np.abs(b - a) < 5.0):
            assert np.linalg.norm(r) < 1e-10
        assert abs(np.linalg.norm(oracle.displacement(L, center, a)) - 4.95) < 1e-10
    for w in rng[:1000]:
        a = np.array([1.5] * 3) + w[0] / np.linalg.norm(w[0])
        b = np.array([8.5] * 3) + w[1] / np.linalg.norm(w[1])
        d = oracle.displacement(L, a, b)
        for q in range(3):
            assert abs(d[q]) <= 5.0 and d[q] < 0.0
            assert abs(abs(d[q]) + abs((b - a)[q]) - 10.0) < 1e-10


def test_temperature_round_trip():
    """liblpmd/tests/simulationtest.unit:58-67: set T, read T back to 1e-10."""
    m = np.full(108, I.MASSES["Cu"])
    for T in (300.0, 150.0):
        v = I.maxwell_boltzmann(m, T, seed=4)
        assert abs(I.temperature(v, m) - T) < 1e-10
        assert np.all(np.abs((v * m[:, None]).sum(axis=0)) < 1e-12)


def test_verletlist_maxneighbors_error():
    """plugins/verletlist.cc:96-97 throws PluginError("maxneighbors is too small!")."""
    g = load_golden("lj_liquid_vl")
    sim = oracle.PortSim(g["pos_in"], g["L"], g["Z"], g["mass"], g["vel_in"])
    with pytest.raises(oracle.OracleError, match="maxneighbors is too small"):
        sim.set_cell_manager("verletlist", "cutoff 8.5125 maxneighbors 40 each 5")


def test_module_argument_syntax():
    """liblpmd/plugins/module.cc:99-103: a keyword without a value is a SyntaxError."""
    with pytest.raises(SyntaxError):
        oracle.parse_args("cutoff 8.5 nx")


def test_linkedcell_stencil_quirks():
    """plugins/linkedcell.cc:216-222: side = ceil(rc/d - 0.5); auto mode picks d ~ rc/2.5."""
    L = [52.6] * 3
    assert oracle.linkedcell_geometry(L, 8.5, 6, 6, 6) == ((6, 6, 6), 1, 27)
    n, side, ci = oracle.linkedcell_geometry(L, 8.5, 0, 0, 0, mode_auto=True)
    assert side == 2 and ci == 125 and n[0] % 2 == 0
    g = load_golden("lj_auto")
    full = load_golden("lj_ar_fcc10")
    # auto mode drops pairs: fewer neighbours than the complete 27-cell stencil
    assert g["neigh_counts"].sum() < full["neigh_counts"].sum()
