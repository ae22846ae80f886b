"""Python binding of libgbmd (include/gbmd.h) through ctypes.

The classes mirror LPMD's host API for the MD timestep so that code written against the
reference reads the same:

    Plugin("linkedcell", "cutoff 8.5 nx 6 ny 6 nz 6")    PluginManager::LoadPlugin + create()
    sim = Simulation(natoms, cell)                        SimulationBuilder::CreateFixedOrthogonal
    sim.set_cell_manager(cm)                              Configuration::SetCellManager
    sim.add_potential(pot, s1, s2)                        Potentials().Append + SetValidSpecies
    sim.set_integrator(vv)                                Simulation::SetIntegrator
    sim.update_forces()                                   CombinedPotential::UpdateForces
    sim.do_steps(n)                                       Simulation::DoSteps

Every call goes to the CUDA library; there is no CPU code path.  Loading fails loudly when
libgbmd.so has not been built.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libgbmd.so"

OK = 0
ERR_INVALID, ERR_SYNTAX, ERR_PLUGIN, ERR_MISSING, ERR_CUDA, ERR_NOMEM, ERR_OVERFLOW, ERR_RUNTIME, ERR_CAPACITY = range(1, 10)
PRECISION = {"fp64": 0, "mixed": 1}
KIND_CELLMANAGER, KIND_POTENTIAL, KIND_INTEGRATOR = 1, 2, 3
FLAG_FIXEDVEL, FLAG_FIXEDPOS = 1, 2
THERMO_FIELDS = ["step", "potential_energy", "kinetic_energy", "total_energy", "temperature", "virial",
                 "px", "py", "pz", "volume", "virial_pressure", "kinetic_pressure", "pressure"]
MODES = {0: "allpairs", 1: "cells", 2: "verlet"}


class GbmdError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


class PluginError(GbmdError):
    pass


class MissingComponent(GbmdError):
    pass


class Thermo(ctypes.Structure):
    _fields_ = [("v", ctypes.c_double * 22)]


class Stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("force_evaluations", ctypes.c_int64),
                ("list_rebuilds", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
                ("max_neighbors", ctypes.c_int64), ("list_capacity", ctypes.c_int64),
                ("neighbor_mode", ctypes.c_int64), ("cell_grid", ctypes.c_int64 * 3),
                ("list_radius", ctypes.c_double), ("device_bytes", ctypes.c_int64),
                ("fp_guard_rechecks", ctypes.c_int64),
                ("force_ms", ctypes.c_double), ("force_launches", ctypes.c_int64),
                ("drift_ms", ctypes.c_double), ("drift_launches", ctypes.c_int64),
                ("rebuild_ms", ctypes.c_double), ("rebuild_launches", ctypes.c_int64)]


_D = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.POINTER(ctypes.c_int64)
_I32 = ctypes.POINTER(ctypes.c_int32)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_VP = ctypes.c_void_p

_SIGS = {
    "gbmd_last_error": (ctypes.c_char_p, []),
    "gbmd_abi_version": (ctypes.c_int, []),
    "gbmd_device_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    "gbmd_plugin_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "gbmd_plugin_destroy": (None, [_VP]),
    "gbmd_plugin_kind": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_int)]),
    "gbmd_plugin_param": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]),
    "gbmd_plugin_cutoff": (ctypes.c_int, [_VP, _D]),
    "gbmd_potential_eval": (ctypes.c_int, [_VP, ctypes.c_int, _D, _D]),
    "gbmd_sim_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, _D, ctypes.POINTER(_VP)]),
    "gbmd_sim_destroy": (None, [_VP]),
    "gbmd_sim_set_atoms": (ctypes.c_int, [_VP, _D, _D, _D, _I32, _D]),
    "gbmd_sim_set_flags": (ctypes.c_int, [_VP, _U8]),
    "gbmd_sim_get_atoms": (ctypes.c_int, [_VP, _D, _D, _D]),
    "gbmd_sim_set_cell_manager": (ctypes.c_int, [_VP, _VP]),
    "gbmd_sim_add_potential": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.c_int]),
    "gbmd_sim_set_integrator": (ctypes.c_int, [_VP, _VP]),
    "gbmd_sim_set_precision": (ctypes.c_int, [_VP, ctypes.c_int]),
    "gbmd_sim_set_option": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_char_p]),
    "gbmd_sim_update_forces": (ctypes.c_int, [_VP]),
    "gbmd_sim_do_steps": (ctypes.c_int, [_VP, ctypes.c_int64]),
    "gbmd_sim_synchronize": (ctypes.c_int, [_VP]),
    "gbmd_sim_thermo": (ctypes.c_int, [_VP, ctypes.POINTER(Thermo)]),
    "gbmd_sim_thermo_log": (ctypes.c_int, [_VP, ctypes.POINTER(Thermo), ctypes.c_int64, _I64]),
    "gbmd_sim_stats": (ctypes.c_int, [_VP, ctypes.POINTER(Stats)]),
    "gbmd_sim_stream": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "gbmd_sim_neighbors": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_double, _I64, _I64, ctypes.c_int64, _I64]),
    "gbmd_sim_cell_sort": (ctypes.c_int, [_VP, _I32, _I64, _I64]),
    "gbmd_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _I64, _D, ctypes.POINTER(_VP)]),
    "gbmd_batch_destroy": (None, [_VP]),
    "gbmd_batch_set_atoms": (ctypes.c_int, [_VP, ctypes.c_int, _D, _D, _I32, _D]),
    "gbmd_batch_get_atoms": (ctypes.c_int, [_VP, ctypes.c_int, _D, _D, _D]),
    "gbmd_batch_set_cell_manager": (ctypes.c_int, [_VP, _VP]),
    "gbmd_batch_add_potential": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.c_int]),
    "gbmd_batch_set_integrator": (ctypes.c_int, [_VP, _VP]),
    "gbmd_batch_set_precision": (ctypes.c_int, [_VP, ctypes.c_int]),
    "gbmd_batch_set_option": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_char_p]),
    "gbmd_batch_update_forces": (ctypes.c_int, [_VP]),
    "gbmd_batch_do_steps": (ctypes.c_int, [_VP, ctypes.c_int64]),
    "gbmd_batch_synchronize": (ctypes.c_int, [_VP]),
    "gbmd_batch_thermo": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.POINTER(Thermo)]),
    "gbmd_batch_stats": (ctypes.c_int, [_VP, ctypes.POINTER(Stats)]),
    "gbmd_batch_stream": (ctypes.c_int, [_VP, ctypes.POINTER(_VP)]),
    "gbmd_batch_neighbors": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_double, _I64, _I64,
                                            ctypes.c_int64, _I64]),
    "gbmd_batch_set_active": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int]),
    "gbmd_sim_scale_velocities": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_double, ctypes.c_double]),
    "gbmd_batch_scale_velocities": (ctypes.c_int, [_VP, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                    ctypes.c_double]),
    "gbmd_sim_checkpoint_size": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_size_t)]),
    "gbmd_sim_checkpoint_save": (ctypes.c_int, [_VP, ctypes.c_void_p, ctypes.c_size_t]),
    "gbmd_sim_checkpoint_load": (ctypes.c_int, [_VP, ctypes.c_void_p, ctypes.c_size_t]),
    "gbmd_batch_checkpoint_size": (ctypes.c_int, [_VP, ctypes.POINTER(ctypes.c_size_t)]),
    "gbmd_batch_checkpoint_save": (ctypes.c_int, [_VP, ctypes.c_void_p, ctypes.c_size_t]),
    "gbmd_batch_checkpoint_load": (ctypes.c_int, [_VP, ctypes.c_void_p, ctypes.c_size_t]),
    "gbmd_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]),
    "gbmd_pair_forces_static": (ctypes.c_int, [_VP, ctypes.c_void_p, ctypes.c_int, _D, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p]),
}

_LIB = None


def load(path: Path | str | None = None):
    """Loads libgbmd.so (built by __graft_entry__.build() or ``make -C lpmd2_gb300/csrc``).

    The environment variable GBMD_LIBRARY names another build of the library (for example a
    variant compiled with different tuning flags) to load instead of the in-tree one.
    """
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else Path(os.environ.get("GBMD_LIBRARY", LIB_PATH))
    if not p.exists():
        raise ImportError(f"libgbmd.so not built ({p}); run __graft_entry__.build()")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def _check(rc: int):
    if rc == OK:
        return
    msg = load().gbmd_last_error().decode()
    if rc == ERR_SYNTAX:
        raise SyntaxError(msg)
    if rc == ERR_PLUGIN:
        raise PluginError(rc, msg)
    if rc == ERR_MISSING:
        raise MissingComponent(rc, msg)
    raise GbmdError(rc, msg)


def _p(a, t=_D):
    return None if a is None else a.ctypes.data_as(t)


def _out3(out, n):
    if out is None:
        return tuple(np.zeros((n, 3)) for _ in range(3))
    if len(out) != 3:
        raise ValueError("out: three (n, 3) arrays")
    for x in out:
        if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.shape == (n, 3) and x.flags.c_contiguous):
            raise ValueError("out arrays must be C-contiguous float64 of shape (n, 3)")
    return tuple(out)


def _vec(a, n):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (n, 3):
        raise ValueError(f"expected shape ({n}, 3), got {a.shape}")
    return a


def device_count() -> int:
    c = ctypes.c_int(0)
    _check(load().gbmd_device_count(ctypes.byref(c)))
    return c.value


def selftest_bounded_wait(polls: int = 1000, device: int = 0) -> bool:
    """True if a kernel wait that nothing completes ended by its poll bound (see gbmd.h)."""
    g = ctypes.c_int(-1)
    _check(load().gbmd_selftest_bounded_wait(device, int(polls), ctypes.byref(g)))
    return g.value == 1


def pair_forces_static(plugin: "Plugin", pos_ptr: int, n: int, box, force_ptr: int, out_ptr: int,
                       stream: int = 0) -> None:
    """gbmd_pair_forces_static: pair forces of one small system from device pointers.

    pos_ptr (3n doubles), force_ptr (3n doubles) and out_ptr (11 doubles) are device
    addresses owned by the caller; nothing is allocated.  The work is queued on ``stream``.
    """
    b = np.ascontiguousarray(box, dtype=np.float64)
    if b.shape != (3,):
        raise ValueError("box must hold 3 edge lengths")
    _check(load().gbmd_pair_forces_static(plugin.h, pos_ptr, int(n), _p(b), force_ptr, out_ptr, stream or None))


class Plugin:
    """A GPU plugin created from its LPMD name and argument string."""

    def __init__(self, name: str, args: str = ""):
        self.lib = load()
        self.name = name
        self.args = args
        h = _VP()
        _check(self.lib.gbmd_plugin_create(name.encode(), args.encode(), ctypes.byref(h)))
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.gbmd_plugin_destroy(h)
            self.h = None

    @property
    def kind(self) -> int:
        k = ctypes.c_int(0)
        _check(self.lib.gbmd_plugin_kind(self.h, ctypes.byref(k)))
        return k.value

    def __getitem__(self, key: str) -> str:
        buf = ctypes.create_string_buffer(512)
        _check(self.lib.gbmd_plugin_param(self.h, key.encode(), buf, 512))
        return buf.value.decode()

    def cutoff(self) -> float:
        c = ctypes.c_double(0.0)
        _check(self.lib.gbmd_plugin_cutoff(self.h, ctypes.byref(c)))
        return c.value

    def _eval(self, what: int, args, nout: int) -> np.ndarray:
        a = np.ascontiguousarray(args, dtype=np.float64)
        out = np.zeros(nout)
        _check(self.lib.gbmd_potential_eval(self.h, what, _p(a), _p(out)))
        return out

    def pair_energy(self, r: float) -> float:
        return float(self._eval(0, [r], 1)[0])

    def pair_force(self, rij) -> np.ndarray:
        return self._eval(1, rij, 3)

    def rhoij(self, r: float) -> float:
        return float(self._eval(2, [r], 1)[0])

    def F(self, rho: float) -> float:
        return float(self._eval(3, [rho], 1)[0])

    def many_bodies(self, rij, rhoi: float, rhoj: float) -> np.ndarray:
        return self._eval(4, list(rij) + [rhoi, rhoj], 3)


def _thermo_dict(t: np.ndarray) -> dict:
    d = {k: float(t[i]) for i, k in enumerate(THERMO_FIELDS)}
    d["stress"] = t[13:22].reshape(3, 3).copy()
    d["raw"] = t.copy()
    return d


def _stats_dict(s: Stats) -> dict:
    return {
        "steps": s.steps, "force_evaluations": s.force_evaluations, "list_rebuilds": s.list_rebuilds,
        "kernel_launches": s.kernel_launches, "max_neighbors": s.max_neighbors,
        "list_capacity": s.list_capacity, "neighbor_mode": MODES.get(s.neighbor_mode, s.neighbor_mode),
        "cell_grid": tuple(s.cell_grid), "list_radius": s.list_radius, "device_bytes": s.device_bytes,
        "fp_guard_rechecks": s.fp_guard_rechecks,
        "force_ms": s.force_ms, "force_launches": s.force_launches,
        "drift_ms": s.drift_ms, "drift_launches": s.drift_launches,
        "rebuild_ms": s.rebuild_ms, "rebuild_launches": s.rebuild_launches,
    }


def _kernel_times(st: dict) -> dict:
    """Average device ms per launch of each kernel class (option time_kernels=1, graph_mode=0)."""
    avg = lambda t, n: (t / n) if n else None
    return {"force_ms": avg(st["force_ms"], st["force_launches"]), "force_launches": st["force_launches"],
            "drift_ms": avg(st["drift_ms"], st["drift_launches"]), "drift_launches": st["drift_launches"],
            "rebuild_chain_ms": avg(st["rebuild_ms"], st["rebuild_launches"]),
            "rebuild_chain_launches": st["rebuild_launches"], "list_rebuilds": st["list_rebuilds"]}


def _checkpoint(lib, kind: str, h) -> bytes:
    n = ctypes.c_size_t(0)
    _check(getattr(lib, f"gbmd_{kind}_checkpoint_size")(h, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value)
    _check(getattr(lib, f"gbmd_{kind}_checkpoint_save")(h, buf, n.value))
    return buf.raw


def _restore(lib, kind: str, h, data: bytes):
    buf = ctypes.create_string_buffer(bytes(data), len(data))
    _check(getattr(lib, f"gbmd_{kind}_checkpoint_load")(h, buf, len(data)))


class Simulation:
    """One periodic orthogonal system on one GPU."""

    def __init__(self, natoms: int, cell, device: int = 0):
        self.lib = load()
        self.n = int(natoms)
        c = np.ascontiguousarray(cell, dtype=np.float64)
        h = _VP()
        _check(self.lib.gbmd_sim_create(device, self.n, _p(c), ctypes.byref(h)))
        self.h = h
        self._plugins = []

    def close(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.gbmd_sim_destroy(h)
            self.h = None

    def __del__(self):
        self.close()

    def set_atoms(self, pos, vel=None, acc=None, Z=None, mass=None):
        pos, vel, acc = _vec(pos, self.n), _vec(vel, self.n), _vec(acc, self.n)
        Zc = None if Z is None else np.ascontiguousarray(np.broadcast_to(Z, (self.n,)), dtype=np.int32)
        mc = None if mass is None else np.ascontiguousarray(np.broadcast_to(mass, (self.n,)), dtype=np.float64)
        _check(self.lib.gbmd_sim_set_atoms(self.h, _p(pos), _p(vel), _p(acc), _p(Zc, _I32), _p(mc)))

    def set_temperature(self, target: float):
        """SetTemperature (tempscaling, temperature): v *= sqrt(target / T) for untagged atoms."""
        _check(self.lib.gbmd_sim_scale_velocities(self.h, 0, float(target), 0.0))

    def berendsen(self, target: float, dt_over_tau: float):
        """One Berendsen rescaling: v *= sqrt(1 + dt/tau (target / T - 1))."""
        _check(self.lib.gbmd_sim_scale_velocities(self.h, 1, float(target), float(dt_over_tau)))

    def checkpoint(self) -> bytes:
        """Lossless snapshot of the whole state (gbmd_sim_checkpoint_save)."""
        return _checkpoint(self.lib, "sim", self.h)

    def restore(self, data: bytes):
        """Loads a snapshot into this identically configured simulation."""
        _restore(self.lib, "sim", self.h, data)

    def set_flags(self, flags):
        f = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
        _check(self.lib.gbmd_sim_set_flags(self.h, _p(f, _U8)))

    def atoms(self, out=None):
        """Positions, velocities, accelerations (n x 3, original atom order).  `out`: three
        C-contiguous float64 (n, 3) arrays to fill instead (e.g. pinned host memory, which the
        copies then reach by DMA without staging)."""
        p, v, a = _out3(out, self.n)
        _check(self.lib.gbmd_sim_get_atoms(self.h, _p(p), _p(v), _p(a)))
        return p, v, a

    def set_cell_manager(self, plugin: Plugin):
        self._plugins.append(plugin)
        _check(self.lib.gbmd_sim_set_cell_manager(self.h, plugin.h))

    def add_potential(self, plugin: Plugin, s1: int = -1, s2: int = -1):
        self._plugins.append(plugin)
        _check(self.lib.gbmd_sim_add_potential(self.h, plugin.h, s1, s2))

    def set_integrator(self, plugin: Plugin):
        self._plugins.append(plugin)
        _check(self.lib.gbmd_sim_set_integrator(self.h, plugin.h))

    def set_precision(self, precision: str):
        _check(self.lib.gbmd_sim_set_precision(self.h, PRECISION[precision]))

    def set_option(self, key: str, value):
        _check(self.lib.gbmd_sim_set_option(self.h, key.encode(), str(value).encode()))

    def update_forces(self):
        _check(self.lib.gbmd_sim_update_forces(self.h))

    def do_steps(self, n: int):
        _check(self.lib.gbmd_sim_do_steps(self.h, int(n)))

    def synchronize(self):
        _check(self.lib.gbmd_sim_synchronize(self.h))

    def thermo_raw(self) -> np.ndarray:
        t = Thermo()
        _check(self.lib.gbmd_sim_thermo(self.h, ctypes.byref(t)))
        return np.array(t.v[:])

    def thermo(self) -> dict:
        return _thermo_dict(self.thermo_raw())

    def thermo_log(self, cap: int = 100000) -> np.ndarray:
        buf = (Thermo * cap)()
        c = ctypes.c_int64(0)
        _check(self.lib.gbmd_sim_thermo_log(self.h, buf, cap, ctypes.byref(c)))
        return np.array([buf[k].v[:] for k in range(c.value)]).reshape(-1, 22)

    def stats(self) -> dict:
        s = Stats()
        _check(self.lib.gbmd_sim_stats(self.h, ctypes.byref(s)))
        return _stats_dict(s)

    def kernel_times(self) -> dict:
        return _kernel_times(self.stats())

    @property
    def stream(self) -> int:
        p = _VP()
        _check(self.lib.gbmd_sim_stream(self.h, ctypes.byref(p)))
        return p.value or 0

    def neighbors(self, full: bool, rcut: float):
        counts = np.zeros(self.n, dtype=np.int64)
        total = ctypes.c_int64(0)
        _check(self.lib.gbmd_sim_neighbors(self.h, int(full), float(rcut), _p(counts, _I64), None, 0, ctypes.byref(total)))
        idx = np.zeros(max(total.value, 1), dtype=np.int64)
        _check(self.lib.gbmd_sim_neighbors(self.h, int(full), float(rcut), _p(counts, _I64), _p(idx, _I64),
                                           total.value, ctypes.byref(total)))
        return counts, idx[: total.value]

    def cell_sort(self, n3):
        n = np.ascontiguousarray(n3, dtype=np.int32)
        cell = np.zeros(self.n, dtype=np.int64)
        order = np.zeros(self.n, dtype=np.int64)
        _check(self.lib.gbmd_sim_cell_sort(self.h, _p(n, _I32), _p(cell, _I64), _p(order, _I64)))
        return cell, order


class Batch:
    """Many independent systems advanced together by the same kernels."""

    def __init__(self, natoms, cells, device: int = 0):
        self.lib = load()
        self.natoms = np.ascontiguousarray(natoms, dtype=np.int64)
        c = np.ascontiguousarray(cells, dtype=np.float64).reshape(-1, 3)
        self.nsys = len(self.natoms)
        h = _VP()
        _check(self.lib.gbmd_batch_create(device, self.nsys, _p(self.natoms, _I64), _p(c), ctypes.byref(h)))
        self.h = h
        self._plugins = []

    def close(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.gbmd_batch_destroy(h)
            self.h = None

    def __del__(self):
        self.close()

    def set_atoms(self, sys: int, pos, vel=None, Z=None, mass=None):
        n = int(self.natoms[sys])
        pos, vel = _vec(pos, n), _vec(vel, n)
        Zc = None if Z is None else np.ascontiguousarray(np.broadcast_to(Z, (n,)), dtype=np.int32)
        mc = None if mass is None else np.ascontiguousarray(np.broadcast_to(mass, (n,)), dtype=np.float64)
        _check(self.lib.gbmd_batch_set_atoms(self.h, sys, _p(pos), _p(vel), _p(Zc, _I32), _p(mc)))

    def checkpoint(self) -> bytes:
        return _checkpoint(self.lib, "batch", self.h)

    def restore(self, data: bytes):
        _restore(self.lib, "batch", self.h, data)

    def set_active(self, sys: int, active: bool):
        _check(self.lib.gbmd_batch_set_active(self.h, sys, 1 if active else 0))

    def set_temperature(self, target: float, sys: int = -1):
        """Simulation.set_temperature for one system (-1: every active system)."""
        _check(self.lib.gbmd_batch_scale_velocities(self.h, sys, 0, float(target), 0.0))

    def berendsen(self, target: float, dt_over_tau: float, sys: int = -1):
        """Simulation.berendsen for one system (-1: every active system)."""
        _check(self.lib.gbmd_batch_scale_velocities(self.h, sys, 1, float(target), float(dt_over_tau)))

    def atoms(self, sys: int, out=None):
        n = int(self.natoms[sys])
        p, v, a = _out3(out, n)
        _check(self.lib.gbmd_batch_get_atoms(self.h, sys, _p(p), _p(v), _p(a)))
        return p, v, a

    def set_cell_manager(self, plugin: Plugin):
        self._plugins.append(plugin)
        _check(self.lib.gbmd_batch_set_cell_manager(self.h, plugin.h))

    def add_potential(self, plugin: Plugin, s1: int = -1, s2: int = -1):
        self._plugins.append(plugin)
        _check(self.lib.gbmd_batch_add_potential(self.h, plugin.h, s1, s2))

    def set_integrator(self, plugin: Plugin):
        self._plugins.append(plugin)
        _check(self.lib.gbmd_batch_set_integrator(self.h, plugin.h))

    def set_precision(self, precision: str):
        _check(self.lib.gbmd_batch_set_precision(self.h, PRECISION[precision]))

    def set_option(self, key: str, value):
        _check(self.lib.gbmd_batch_set_option(self.h, key.encode(), str(value).encode()))

    def update_forces(self):
        _check(self.lib.gbmd_batch_update_forces(self.h))

    def do_steps(self, n: int):
        _check(self.lib.gbmd_batch_do_steps(self.h, int(n)))

    def synchronize(self):
        _check(self.lib.gbmd_batch_synchronize(self.h))

    def thermo(self, sys: int) -> dict:
        t = Thermo()
        _check(self.lib.gbmd_batch_thermo(self.h, sys, ctypes.byref(t)))
        return _thermo_dict(np.array(t.v[:]))

    def stats(self) -> dict:
        s = Stats()
        _check(self.lib.gbmd_batch_stats(self.h, ctypes.byref(s)))
        return _stats_dict(s)

    def kernel_times(self) -> dict:
        """Simulation.kernel_times for the batch (set_option("time_kernels", 1) first)."""
        return _kernel_times(self.stats())

    @property
    def stream(self) -> int:
        p = _VP()
        _check(self.lib.gbmd_batch_stream(self.h, ctypes.byref(p)))
        return p.value or 0

    def neighbors(self, sys: int, full: bool, rcut: float):
        """Simulation.neighbors for system `sys` (indices local to the system)."""
        n = int(self.natoms[sys])
        counts = np.zeros(n, dtype=np.int64)
        total = ctypes.c_int64(0)
        _check(self.lib.gbmd_batch_neighbors(self.h, sys, int(full), float(rcut), _p(counts, _I64), None, 0,
                                             ctypes.byref(total)))
        idx = np.zeros(max(total.value, 1), dtype=np.int64)
        _check(self.lib.gbmd_batch_neighbors(self.h, sys, int(full), float(rcut), _p(counts, _I64), _p(idx, _I64),
                                             total.value, ctypes.byref(total)))
        return counts, idx[: total.value]
