"""Seeded synthetic inputs for the MD timestep: lattices, vacancies, jitter, velocities.

All randomness comes from SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom
number generators", OOPSLA 2014) so that the same seed gives the same stream everywhere.
Lattice generation mirrors the ``crystal3d`` generator plugin (plugins/crystal3d.cc:62-130),
including its +0.01 fractional x offset for FCC sites, which leaves the last column of atoms
just outside the box.  Units are the reference's: angstrom, fs, amu, eV.
"""
from __future__ import annotations

import math

import numpy as np

KIN2EV = 103.64269  # liblpmd/lpmd/properties.h:10
KBOLTZMANN = 8.6173422e-05  # liblpmd/lpmd/properties.h:11
FORCEFACTOR = 0.00964853  # session string "0.00964853", liblpmd/runtime/session.cc:17-31

# Masses of the species used by the standard workloads (liblpmd/support/elements.cc:20-24).
MASSES = {"Ar": 39.948, "Cu": 63.546, "Fe": 55.847, "Mo": 95.94, "Au": 196.967}
ATOMIC_NUMBERS = {"Ar": 18, "Cu": 29, "Fe": 26, "Mo": 42, "Au": 79}

_M64 = (1 << 64) - 1


def splitmix64(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n successive SplitMix64 outputs for (seed, stream), as uint64."""
    with np.errstate(over="ignore"):
        gamma = np.uint64(0x9E3779B97F4A7C15)
        start = np.uint64((seed * 0x632BE59BD9B4E019 + stream * 0xD1B54A32D192ED03) & _M64)
        z = start + gamma * np.arange(1, n + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n doubles uniform in [0, 1) (top 53 bits of SplitMix64)."""
    return (splitmix64(seed, n, stream) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n standard normals by the Box-Muller transform."""
    m = (n + 1) // 2
    u = uniform(seed, 2 * m, stream)
    u1 = 1.0 - u[0::2]  # (0, 1]
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2.0 * math.pi * u2), r * np.sin(2.0 * math.pi * u2)])
    return z[:n]


def fcc_crystal3d(nx: int, ny: int, nz: int, a: float) -> tuple[np.ndarray, np.ndarray]:
    """FCC sites as crystal3d generates them; returns (positions[N,3], box[3]).

    Site order is k (z) outer, j, i inner, four sites per unit cell, each position being
    Cartesian(frac) = frac * L (plugins/crystal3d.cc:84-104).
    """
    L = np.array([nx * a, ny * a, nz * a], dtype=np.float64)
    ax, ay, az = 1.0 / nx, 1.0 / ny, 1.0 / nz
    pos = np.empty((4 * nx * ny * nz, 3), dtype=np.float64)
    c = 0
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                for f in (
                    ((i + 0.51) * ax, (j + 0.5) * ay, (k + 0.5) * az),
                    ((i + 0.51) * ax, j * ay, (k + 1.0) * az),
                    ((i + 1.01) * ax, j * ay, (k + 0.5) * az),
                    ((i + 1.01) * ax, (j + 0.5) * ay, (k + 1.0) * az),
                ):
                    pos[c] = (f[0] * L[0], f[1] * L[1], f[2] * L[2])
                    c += 1
    return pos, L


def fcc_fast(nx: int, ny: int, nz: int, a: float, offset: float = 0.01) -> tuple[np.ndarray, np.ndarray]:
    """Vectorised crystal3d FCC (identical site order and arithmetic) for large lattices."""
    L = np.array([nx * a, ny * a, nz * a], dtype=np.float64)
    k, j, i = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    ax, ay, az = 1.0 / nx, 1.0 / ny, 1.0 / nz
    o5, o10 = 0.5 + offset, 1.0 + offset
    fr = [
        ((i + o5) * ax, (j + 0.5) * ay, (k + 0.5) * az),
        ((i + o5) * ax, j * ay, (k + 1.0) * az),
        ((i + o10) * ax, j * ay, (k + 0.5) * az),
        ((i + o10) * ax, (j + 0.5) * ay, (k + 1.0) * az),
    ]
    pos = np.empty((len(i), 4, 3), dtype=np.float64)
    for s, f in enumerate(fr):
        for q in range(3):
            pos[:, s, q] = f[q] * L[q]
    return pos.reshape(-1, 3), L


def fcc_centered(n: int, L: float, masses: np.ndarray | None = None) -> np.ndarray:
    """The 108-atom (n=3) FCC of liblpmd/demos/linkedcell.cc:35-53 (ScaleByCell then
    CenterByCenterOfMass, liblpmd/lpmd/manipulations.h:31-37)."""
    a = 1.0 / n
    pos = []
    for k in range(n):
        for j in range(n):
            for i in range(n):
                pos.append(((i + 0.5) * a * L, (j + 0.5) * a * L, (k + 0.5) * a * L))
                pos.append(((i + 0.5) * a * L, j * a * L, (k + 1.0) * a * L))
                pos.append(((i + 1.0) * a * L, j * a * L, (k + 0.5) * a * L))
                pos.append(((i + 1.0) * a * L, (j + 0.5) * a * L, (k + 1.0) * a * L))
    pos = np.array(pos, dtype=np.float64)
    m = np.ones(len(pos)) if masses is None else masses
    com = (pos * m[:, None]).sum(axis=0) / m.sum()
    return pos - (com - 0.5 * L)


def remove_sites(pos: np.ndarray, fraction: float, seed: int) -> np.ndarray:
    """Removes round(fraction * N) sites chosen uniformly without replacement (vacancies)."""
    n = len(pos)
    k = int(round(fraction * n))
    keys = splitmix64(seed, n, stream=7)
    drop = np.argsort(keys, kind="stable")[:k]
    keep = np.ones(n, dtype=bool)
    keep[drop] = False
    return pos[keep]


def jitter(pos: np.ndarray, amplitude: float, seed: int) -> np.ndarray:
    """Adds independent uniform displacements in [-amplitude, amplitude) per coordinate."""
    u = uniform(seed, pos.size, stream=3).reshape(pos.shape)
    return pos + (2.0 * u - 1.0) * amplitude


def kinetic_energy(vel: np.ndarray, mass: np.ndarray) -> float:
    """KineticEnergy (liblpmd/lpmd/properties.h:22-37) in eV."""
    return float(np.sum(0.5 * mass * np.sum(vel * vel, axis=1)) * KIN2EV)


def temperature(vel: np.ndarray, mass: np.ndarray) -> float:
    """Temperature (liblpmd/lpmd/properties.h:39-53): N, not 3N-3, in the denominator."""
    return (2.0 / 3.0) * kinetic_energy(vel, mass) / (KBOLTZMANN * len(vel))


def maxwell_boltzmann(mass: np.ndarray, T: float, seed: int) -> np.ndarray:
    """Gaussian velocities at temperature T (K), zero total momentum, rescaled so that the
    reference's Temperature() of the result is T."""
    n = len(mass)
    if n == 0:
        return np.zeros((0, 3))
    sd = np.sqrt(KBOLTZMANN * T / (mass * KIN2EV))  # angstrom/fs per component
    v = normal(seed, 3 * n, stream=1).reshape(n, 3) * sd[:, None]
    p = (v * mass[:, None]).sum(axis=0) / mass.sum()
    v -= p
    t = temperature(v, mass)
    if t > 0:
        v *= math.sqrt(T / t)
    return v


def lj_reduced_units(sigma: float, epsilon: float, mass: float) -> dict:
    """tau = sqrt(m sigma^2 / (eps * forcefactor)) fs; T* -> K; rho* -> atoms/A^3."""
    tau = math.sqrt(mass * sigma * sigma / (epsilon * FORCEFACTOR))
    return {"tau_fs": tau, "T_per_Tstar": epsilon / KBOLTZMANN, "rho_per_rhostar": 1.0 / sigma**3}


# ---------------------------------------------------------------------------------------------
# Ensembles and job streams (seeded; every array is a pure function of the seed)
# ---------------------------------------------------------------------------------------------

LJ_AR = dict(sigma=3.405, epsilon=0.0103, mass=39.948, Z=18)
SC_CU = dict(e=0.012382, a=3.61, n=9, m=6, c=39.432, mass=63.546, Z=29)


def fcc_count_k(n_target: float, kmin: int, kmax: int) -> int:
    """FCC cells per edge k with 4k^3 atoms closest (in k) to n_target, clamped to [kmin, kmax]."""
    return int(min(kmax, max(kmin, round((n_target / 4.0) ** (1.0 / 3.0)))))


def lj_system(k: int, rho_star: float, t_star: float, seed: int) -> dict:
    """Argon FCC k^3 cells (4k^3 atoms) at reduced density rho*, jittered by +-0.05 sigma, with
    Maxwell-Boltzmann velocities at T*.  Real units (A, fs, amu, eV)."""
    sigma, eps, mass = LJ_AR["sigma"], LJ_AR["epsilon"], LJ_AR["mass"]
    a = (4.0 / rho_star) ** (1.0 / 3.0) * sigma
    pos, L = fcc_fast(k, k, k, a)
    pos = np.mod(jitter(pos, 0.05 * sigma, seed=seed), L)
    m = np.full(len(pos), mass)
    vel = maxwell_boltzmann(m, t_star * eps / KBOLTZMANN, seed=seed)
    return dict(kind="lj", pos=pos, vel=vel, mass=m, Z=LJ_AR["Z"], L=L, natoms=len(pos), k=k, rho_star=rho_star,
                t_star=t_star, seed=seed)


def sc_cu_system(k: int, seed: int, T: float = 300.0, vacancies: float = 0.01) -> dict:
    """Sutton-Chen copper: FCC k^3 cells at a = 3.61 A with a fraction of sites removed, velocities
    at T (K)."""
    pos, L = fcc_fast(k, k, k, SC_CU["a"])
    if vacancies > 0:
        pos = remove_sites(pos, vacancies, seed=seed)
    m = np.full(len(pos), SC_CU["mass"])
    vel = maxwell_boltzmann(m, T, seed=seed)
    return dict(kind="sc", pos=pos, vel=vel, mass=m, Z=SC_CU["Z"], L=L, natoms=len(pos), k=k, seed=seed)


def log_uniform(u: np.ndarray, lo: float, hi: float) -> np.ndarray:
    return np.exp(math.log(lo) + u * (math.log(hi) - math.log(lo)))


def lj_ensemble(nsys: int = 512, seed: int = 4, nmin: int = 256, nmax: int = 32000) -> list[dict]:
    """Independent LJ systems: N log-uniform in [nmin, nmax] rounded to 4k^3 (k in [4, 20]),
    rho* uniform in [0.70, 0.95], T* uniform in [0.7, 2.0]."""
    u = uniform(seed, 3 * nsys, stream=11).reshape(nsys, 3)
    n_target = log_uniform(u[:, 0], nmin, nmax)
    out = []
    for s in range(nsys):
        k = fcc_count_k(n_target[s], 4, 20)
        out.append(lj_system(k, 0.70 + 0.25 * u[s, 1], 0.7 + 1.3 * u[s, 2], seed=seed * 100003 + s))
    return out


def job_stream(njobs: int, rate: float, seed: int = 5, nmin: int = 500, nmax: int = 200000,
               smin: int = 1000, smax: int = 20000, lj_fraction: float = 0.7) -> list[dict]:
    """MD jobs with Poisson arrivals at `rate` jobs/s: 70 % LJ (rho*, T* as the ensemble), 30 %
    Sutton-Chen Cu at 300 K; N log-uniform in [nmin, nmax] rounded to 4k^3; steps uniform in
    [smin, smax].  Systems are generated lazily by materialize_job()."""
    u = uniform(seed, 6 * njobs, stream=13).reshape(njobs, 6)
    gaps = -np.log1p(-u[:, 0]) / rate
    t = np.cumsum(gaps) - gaps[0]
    n_target = log_uniform(u[:, 2], nmin, nmax)
    jobs = []
    for j in range(njobs):
        kind = "lj" if u[j, 1] < lj_fraction else "sc"
        k = fcc_count_k(n_target[j], 5, 36)
        steps = int(smin + min(smax - smin, int(u[j, 3] * (smax - smin + 1))))
        jobs.append(dict(id=j, kind=kind, k=k, steps=steps, arrival=float(t[j]), rho_star=0.70 + 0.25 * u[j, 4],
                         t_star=0.7 + 1.3 * u[j, 5], seed=seed * 1000003 + j))
    return jobs


def materialize_job(job: dict) -> dict:
    """Positions, velocities and box of a job from job_stream()."""
    if job["kind"] == "lj":
        return lj_system(job["k"], job["rho_star"], job["t_star"], seed=job["seed"])
    return sc_cu_system(job["k"], seed=job["seed"])
