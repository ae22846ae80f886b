"""Shared helpers for the test suite: workload builders and neighbour-set fingerprints."""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from lpmd2_gb300 import inputs as I

GOLDEN = Path(__file__).resolve().parent / "golden"

LJ_AR = "sigma 3.405 epsilon 0.0103 cutoff 8.5"
SC_CU = "e 0.012382 a 3.61 n 9 m 6 c 39.432 cutoff 7.22"
# Finnis-Sinclair alpha-Fe (Finnis & Sinclair 1984) and an extended (quartic) variant.
FS_FE = "c0 1.2371147 c1 -0.3592185 c2 -0.0385607 A 1.828905 B 1.8 c 3.40 d 3.569745"
# Gupta / tight-binding second-moment gold (Cleri and Rosato, Phys. Rev. B 48, 22 (1993))
GUPTA_AU = "A 0.2061 r0 2.884 p 10.229 B 1.790 q 4.036 cutoff 6.0"
FSX_MO = "c0 47.1346499 c1 -33.7665655 c2 6.2541999 c3 -0.0122 c4 0.0001 A 1.848 B 0.5 c 3.25 d 4.1"


def mix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser applied elementwise (a 64-bit mixing function)."""
    with np.errstate(over="ignore"):
        z = x.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def neighbor_hashes(counts: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """Order-independent per-atom fingerprint of each neighbour multiset:
    sum over the atom's neighbours j of mix64(j), modulo 2^64."""
    counts = np.asarray(counts, dtype=np.int64)
    owner = np.repeat(np.arange(len(counts)), counts)
    h = np.zeros(len(counts), dtype=np.uint64)
    with np.errstate(over="ignore"):
        np.add.at(h, owner, mix64(np.asarray(idx, dtype=np.int64)))
    return h


def workload(name: str) -> dict:
    """Seeded inputs of the golden cases (positions, box, species, velocities, plugins)."""
    if name == "kat108":
        L = 17.1191
        pos = I.fcc_centered(3, L)
        n = len(pos)
        return dict(pos=pos, L=np.array([L, L, L]), symbol="Ar", Z=18, vel=np.zeros((n, 3)),
                    cm="linkedcell", cm_args="cutoff 8.5 nx 1 ny 1 nz 1",
                    pots=[("lennardjones", "sigma 3.405 epsilon 0.0103 cutoff 4.15", -1, -1)],
                    dt=1.0, nsteps=0, neigh=(1, 4.15))
    if name == "lj_ar_fcc10":
        pos, L = I.fcc_crystal3d(10, 10, 10, 5.26)
        m = np.full(len(pos), I.MASSES["Ar"])
        return dict(pos=pos, L=L, symbol="Ar", Z=18, vel=I.maxwell_boltzmann(m, 100.0, seed=1),
                    cm="linkedcell", cm_args="cutoff 8.5 nx 6 ny 6 nz 6",
                    pots=[("lennardjones", LJ_AR, -1, -1)], dt=1.0, nsteps=100, neigh=(1, 8.5))
    if name == "lj_liquid_vl":
        sigma, eps = 3.405, 0.0103
        a = (4.0 / 0.8442) ** (1.0 / 3.0) * sigma
        pos, L = I.fcc_fast(6, 6, 6, a)
        pos = I.jitter(pos, 0.05 * sigma, seed=2)
        m = np.full(len(pos), I.MASSES["Ar"])
        T = 1.5 * eps / I.KBOLTZMANN
        tau = I.lj_reduced_units(sigma, eps, I.MASSES["Ar"])["tau_fs"]
        rc = 2.5 * sigma
        return dict(pos=pos, L=L, symbol="Ar", Z=18, vel=I.maxwell_boltzmann(m, T, seed=2),
                    cm="verletlist", cm_args=f"cutoff {rc!r} maxneighbors 128 each 5",
                    pots=[("lennardjones", f"sigma {sigma} epsilon {eps} cutoff {rc!r}", -1, -1)],
                    dt=0.005 * tau, nsteps=20, neigh=(1, rc))
    if name == "sc_cu":
        pos, L = I.fcc_fast(6, 6, 6, 3.61)
        pos = I.remove_sites(pos, 0.01, seed=3)
        m = np.full(len(pos), I.MASSES["Cu"])
        return dict(pos=pos, L=L, symbol="Cu", Z=29, vel=I.maxwell_boltzmann(m, 300.0, seed=3),
                    cm="linkedcell", cm_args="cutoff 7.22 nx 3 ny 3 nz 3",
                    pots=[("suttonchen", SC_CU, -1, -1)], dt=2.0, nsteps=20, neigh=(1, 7.22))
    if name == "fs_fe":
        pos, L = I.fcc_fast(5, 5, 5, 3.6)
        pos = I.jitter(pos, 0.05, seed=5)
        m = np.full(len(pos), I.MASSES["Fe"])
        return dict(pos=pos, L=L, symbol="Fe", Z=26, vel=I.maxwell_boltzmann(m, 300.0, seed=5),
                    cm="linkedcell", cm_args="cutoff 3.6 nx 5 ny 5 nz 5",
                    pots=[("finnissinclair", FS_FE, -1, -1)], dt=1.0, nsteps=10, neigh=(1, 3.569745))
    if name == "fsx_mo":
        pos, L = I.fcc_fast(5, 5, 5, 3.6)
        pos = I.jitter(pos, 0.05, seed=6)
        m = np.full(len(pos), I.MASSES["Mo"])
        return dict(pos=pos, L=L, symbol="Mo", Z=42, vel=I.maxwell_boltzmann(m, 300.0, seed=6),
                    cm="linkedcell", cm_args="cutoff 4.1 nx 4 ny 4 nz 4",
                    pots=[("finnissinclair-ext", FSX_MO, -1, -1)], dt=1.0, nsteps=10, neigh=(1, 4.1))
    if name == "gupta_au":
        pos, L = I.fcc_fast(6, 6, 6, 4.08)
        pos = I.remove_sites(pos, 0.01, seed=8)
        m = np.full(len(pos), I.MASSES["Au"])
        return dict(pos=pos, L=L, symbol="Au", Z=79, vel=I.maxwell_boltzmann(m, 400.0, seed=8),
                    cm="linkedcell", cm_args="cutoff 6.0 nx 4 ny 4 nz 4",
                    pots=[("gupta", GUPTA_AU, -1, -1)], dt=2.0, nsteps=20, neigh=(1, 6.0))
    if name.startswith("lj_integ_"):
        # the same argon liquid under each integrator other than velocityverlet
        kind = name[len("lj_integ_"):]
        s_ = I.lj_system(5, 0.8, 1.2, seed=21)
        integ = (kind, "fmass 2e9 t 120.0" if kind == "nosehoover" else "")
        return dict(pos=s_["pos"], L=s_["L"], symbol="Ar", Z=18, vel=s_["vel"], cm="linkedcell",
                    cm_args="cutoff 8.5 nx 3 ny 3 nz 3", pots=[("lennardjones", LJ_AR, -1, -1)], dt=2.0,
                    nsteps=30, neigh=(1, 8.5), integ=integ)
    if name == "sc_integ_beeman":
        # three cells per axis: with two, the reference's LinkedCell stencil visits a cell twice
        pos, L = I.fcc_fast(6, 6, 6, 3.61)
        pos = I.remove_sites(pos, 0.01, seed=23)
        m = np.full(len(pos), I.MASSES["Cu"])
        return dict(pos=pos, L=L, symbol="Cu", Z=29, vel=I.maxwell_boltzmann(m, 600.0, seed=23),
                    cm="linkedcell", cm_args="cutoff 7.22 nx 3 ny 3 nz 3",
                    pots=[("suttonchen", SC_CU, -1, -1)], dt=2.0, nsteps=20, neigh=(1, 7.22),
                    integ=("beeman", ""))
    if name.startswith("lj_lcbinary"):
        # automatic grid (sub-cells of about cutoff/5: the stencil stops short of the cutoff), or
        # a coarse 4x4x4 grid that has to grow until no sub-cell holds two atoms
        s_ = I.lj_system(5, 0.8, 1.2, seed=27)
        args = "cutoff 8.5 mode auto" if name == "lj_lcbinary" else "cutoff 8.5 nx 4 ny 4 nz 4"
        return dict(pos=s_["pos"], L=s_["L"], symbol="Ar", Z=18, vel=s_["vel"], cm="lcbinary", cm_args=args,
                    pots=[("lennardjones", LJ_AR, -1, -1)], dt=2.0, nsteps=30, neigh=(1, 8.5))
    if name == "lj_fastlj":
        s_ = I.lj_system(5, 0.8, 1.2, seed=25)
        return dict(pos=s_["pos"], L=s_["L"], symbol="Ar", Z=18, vel=s_["vel"], cm="linkedcell",
                    cm_args="cutoff 8.5 nx 3 ny 3 nz 3", pots=[("fastlj", LJ_AR + " bins 500", -1, -1)], dt=2.0,
                    nsteps=30, neigh=(1, 8.5))
    if name == "lj_auto":
        pos, L = I.fcc_crystal3d(10, 10, 10, 5.26)
        m = np.full(len(pos), I.MASSES["Ar"])
        return dict(pos=pos, L=L, symbol="Ar", Z=18, vel=I.maxwell_boltzmann(m, 100.0, seed=1),
                    cm="linkedcell", cm_args="cutoff 8.5 mode auto",
                    pots=[("lennardjones", LJ_AR, -1, -1)], dt=1.0, nsteps=5, neigh=(1, 8.5))
    if name == "lj_nx2":
        pos, L = I.fcc_crystal3d(4, 4, 4, 5.26)
        m = np.full(len(pos), I.MASSES["Ar"])
        return dict(pos=pos, L=L, symbol="Ar", Z=18, vel=I.maxwell_boltzmann(m, 100.0, seed=1),
                    cm="linkedcell", cm_args="cutoff 8.5 nx 2 ny 2 nz 2",
                    pots=[("lennardjones", LJ_AR, -1, -1)], dt=1.0, nsteps=5, neigh=(1, 8.5))
    raise KeyError(name)


GOLDEN_CASES = ["kat108", "lj_ar_fcc10", "lj_liquid_vl", "sc_cu", "fs_fe", "fsx_mo", "gupta_au", "lj_fastlj", "lj_auto",
                "lj_nx2", "lj_lcbinary", "lj_lcbinary_grow"]
FP64_ONLY_CASES = {"lj_fastlj"}  # fastlj has no mixed-precision form
# integrators other than velocityverlet (fixtures from the reference's own plugins)
INTEG_CASES = ["lj_integ_euler", "lj_integ_leapfrog", "lj_integ_verlet", "lj_integ_beeman", "lj_integ_nosehoover",
               "sc_integ_beeman"]


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz", allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def rel_norm_err(a: np.ndarray, b: np.ndarray) -> float:
    """sqrt(sum |a-b|^2) / sqrt(sum |b|^2): the force RMS relative error definition."""
    den = math.sqrt(float(np.sum(np.asarray(b, dtype=np.float64) ** 2)))
    num = math.sqrt(float(np.sum((np.asarray(a, dtype=np.float64) - b) ** 2)))
    return num / den if den > 0 else num
