"""Python access to the oracle: the C restatement (liboracle.so) and, where the reference
sources were compiled here, the reference itself (_ref/libref_driver.so).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py; never by the product package.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref_driver.so"
THERMO_LEN = 22
THERMO_FIELDS = ["step", "epot", "ekin", "etot", "temperature", "virial", "px", "py", "pz",
                 "volume", "virial_pressure", "kinetic_pressure", "pressure"]

INTEG_KIND = {"velocityverlet": 0, "euler": 1, "leapfrog": 2, "verlet": 3, "beeman": 4, "nosehoover": 5}
CM_KIND = {"linkedcell": 1, "verletlist": 2, "minimumimage": 3}
POT_KIND = {"lennardjones": 1, "suttonchen": 2, "finnissinclair": 3, "finnissinclair-ext": 4, "gupta": 5,
            "fastlj": 6}
POT_KEYS = {
    "lennardjones": ["sigma", "epsilon", "cutoff"],
    "suttonchen": ["e", "a", "n", "m", "c", "cutoff"],
    "finnissinclair": ["c0", "c1", "c2", "A", "B", "c", "d"],
    "finnissinclair-ext": ["c0", "c1", "c2", "c3", "c4", "A", "B", "c", "d"],
    "gupta": ["A", "r0", "p", "B", "q", "cutoff"],
    "fastlj": ["sigma", "epsilon", "cutoff", "bins"],
}
ERRORS = {1: "invalid argument", 2: "maxneighbors is too small!", 3: "out of memory",
          4: "missing component", 5: "capacity"}

_D = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.POINTER(ctypes.c_int64)


def reference_source() -> Path | None:
    """The lpmd2 checkout to compile the reference from: $LPMD_REFERENCE, else the checkout the
    last `make ref` was built from (recorded in _ref/REFERENCE); None when neither names an
    existing checkout."""
    env = os.environ.get("LPMD_REFERENCE")
    rec = HERE / "_ref" / "REFERENCE"
    cand = Path(env) if env else (Path(rec.read_text().strip()) if rec.exists() else None)
    return cand if cand is not None and (cand / "liblpmd").is_dir() else None


def build(quiet: bool = True) -> None:
    """Compiles the oracle (and the reference driver when reference_source() names a checkout)."""
    import subprocess

    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", str(HERE), "liboracle.so"], check=True, stdout=out)
    ref = reference_source()
    if ref is not None:
        subprocess.run(["make", "-C", str(HERE), "-j8", "ref", f"REF={ref}"], check=True, stdout=out)


def _ptr(a, t=_D):
    return None if a is None else a.ctypes.data_as(t)


def parse_args(args: str) -> dict:
    """Module::ProcessArguments (liblpmd/plugins/module.cc:77-97): whitespace-separated
    key/value pairs; a key without a value is a SyntaxError."""
    words = args.split()
    if len(words) % 2:
        raise SyntaxError("Unexpected end of input while reading module arguments")
    return {words[i]: words[i + 1] for i in range(0, len(words), 2)}


def _port():
    lib = ctypes.CDLL(str(PORT_LIB))
    lib.orc_sim_create.restype = ctypes.c_void_p
    lib.orc_sim_create.argtypes = [ctypes.c_int64, _D]
    lib.orc_sim_destroy.argtypes = [ctypes.c_void_p]
    lib.orc_sim_set_atoms.argtypes = [ctypes.c_void_p, _D, _D, _D, ctypes.POINTER(ctypes.c_int32), _D]
    lib.orc_sim_set_flags.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8)]
    lib.orc_sim_get_atoms.argtypes = [ctypes.c_void_p, _D, _D, _D]
    lib.orc_sim_set_linkedcell.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.orc_sim_set_verletlist.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int64, ctypes.c_int64]
    lib.orc_sim_set_minimumimage.argtypes = [ctypes.c_void_p, ctypes.c_double]
    lib.orc_sim_set_lcbinary.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int]
    lib.orc_sim_add_potential.argtypes = [ctypes.c_void_p, ctypes.c_int, _D, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int]
    lib.orc_sim_set_velocityverlet.argtypes = [ctypes.c_void_p, ctypes.c_double]
    lib.orc_sim_set_integrator.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_double]
    lib.orc_sim_update_forces.argtypes = [ctypes.c_void_p]
    lib.orc_sim_do_steps.argtypes = [ctypes.c_void_p, ctypes.c_int64, _D]
    lib.orc_sim_thermo.argtypes = [ctypes.c_void_p, _D]
    lib.orc_sim_energy.restype = ctypes.c_double
    lib.orc_sim_energy.argtypes = [ctypes.c_void_p]
    lib.orc_sim_virial.restype = ctypes.c_double
    lib.orc_sim_virial.argtypes = [ctypes.c_void_p]
    lib.orc_sim_stress.argtypes = [ctypes.c_void_p, _D]
    lib.orc_sim_neighbors.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, _I64, _I64,
                                      ctypes.c_int64, _I64]
    lib.orc_sim_update_cell_calls.restype = ctypes.c_int64
    lib.orc_sim_update_cell_calls.argtypes = [ctypes.c_void_p]
    lib.orc_displacement.argtypes = [_D, _D, _D, _D]
    lib.orc_fitted_inside.argtypes = [_D, _D, _D]
    lib.orc_linkedcell_geometry.argtypes = [_D, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
    return lib


_PORT = None


def port_lib():
    global _PORT
    if _PORT is None:
        _PORT = _port()
    return _PORT


class OracleError(RuntimeError):
    pass


def _check(rc: int):
    if rc:
        raise OracleError(ERRORS.get(rc, f"oracle error {rc}"))


class PortSim:
    """One simulation in the C restatement, driven like a reference Simulation."""

    def __init__(self, pos, L, Z, mass, vel=None, flags=None):
        self.lib = port_lib()
        self.n = len(pos)
        self.L = np.ascontiguousarray(L, dtype=np.float64)
        self.h = self.lib.orc_sim_create(self.n, _ptr(self.L))
        if not self.h:
            raise OracleError("orc_sim_create failed")
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        self._Z = np.ascontiguousarray(Z, dtype=np.int32)
        self._m = np.ascontiguousarray(mass, dtype=np.float64)
        _check(self.lib.orc_sim_set_atoms(self.h, _ptr(pos), _ptr(vel), None,
                                          _ptr(self._Z, ctypes.POINTER(ctypes.c_int32)), _ptr(self._m)))
        if flags is not None:
            f = np.ascontiguousarray(flags, dtype=np.uint8)
            _check(self.lib.orc_sim_set_flags(self.h, _ptr(f, ctypes.POINTER(ctypes.c_uint8))))

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.orc_sim_destroy(h)
            self.h = None

    def set_cell_manager(self, name: str, args: str):
        kw = parse_args(args)
        if name == "linkedcell":
            auto = kw.get("mode", "noauto") in ("auto", "AUTO")
            _check(self.lib.orc_sim_set_linkedcell(self.h, float(kw.get("cutoff", 7.0)), int(kw.get("nx", 0)),
                                                   int(kw.get("ny", 0)), int(kw.get("nz", 0)), int(auto)))
        elif name == "verletlist":
            _check(self.lib.orc_sim_set_verletlist(self.h, float(kw.get("cutoff", 0.0)),
                                                   int(kw.get("maxneighbors", 80)), int(kw.get("each", 5))))
        elif name == "minimumimage":
            _check(self.lib.orc_sim_set_minimumimage(self.h, float(kw.get("cutoff", 0.0))))
        elif name == "lcbinary":
            auto = kw.get("mode", "noauto") in ("auto", "AUTO")
            _check(self.lib.orc_sim_set_lcbinary(self.h, float(kw.get("cutoff", 7.0)), int(kw.get("nx", 0)),
                                                 int(kw.get("ny", 0)), int(kw.get("nz", 0)), int(auto)))
        else:
            raise OracleError(f"unknown cell manager {name}")

    def add_potential(self, name: str, args: str, s1: int = -1, s2: int = -1):
        kw = parse_args(args)
        defaults = {"bins": 500.0} if name == "fastlj" else {}  # plugins/fastlj.cc:19
        p = np.array([float(kw.get(k, defaults.get(k, 0.0))) for k in POT_KEYS[name]], dtype=np.float64)
        _check(self.lib.orc_sim_add_potential(self.h, POT_KIND[name], _ptr(p), len(p), s1, s2))

    def set_integrator(self, dt: float, name: str = "velocityverlet", args: str = ""):
        kw = parse_args(args)
        _check(self.lib.orc_sim_set_integrator(self.h, INTEG_KIND[name], float(dt), float(kw.get("fmass", 0.0)),
                                               float(kw.get("t", 300.0))))

    def update_forces(self):
        _check(self.lib.orc_sim_update_forces(self.h))

    def do_steps(self, n: int) -> np.ndarray:
        th = np.zeros((max(n, 1), THERMO_LEN))
        _check(self.lib.orc_sim_do_steps(self.h, n, _ptr(th)))
        return th[:n]

    def thermo(self) -> np.ndarray:
        th = np.zeros(THERMO_LEN)
        _check(self.lib.orc_sim_thermo(self.h, _ptr(th)))
        return th

    def energy(self) -> float:
        return self.lib.orc_sim_energy(self.h)

    def virial(self) -> float:
        return self.lib.orc_sim_virial(self.h)

    def stress(self) -> np.ndarray:
        s = np.zeros(9)
        self.lib.orc_sim_stress(self.h, _ptr(s))
        return s.reshape(3, 3)

    def atoms(self):
        p = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        a = np.zeros((self.n, 3))
        self.lib.orc_sim_get_atoms(self.h, _ptr(p), _ptr(v), _ptr(a))
        return p, v, a

    def neighbors(self, full: bool, rcut: float):
        counts = np.zeros(self.n, dtype=np.int64)
        total = ctypes.c_int64(0)
        _check(self.lib.orc_sim_neighbors(self.h, int(full), rcut, _ptr(counts, _I64), None, 0,
                                          ctypes.byref(total)))
        idx = np.zeros(max(total.value, 1), dtype=np.int64)
        _check(self.lib.orc_sim_neighbors(self.h, int(full), rcut, _ptr(counts, _I64), _ptr(idx, _I64),
                                          total.value, ctypes.byref(total)))
        return counts, idx[: total.value]

    def update_cell_calls(self) -> int:
        return self.lib.orc_sim_update_cell_calls(self.h)


def displacement(L, a, b):
    lib = port_lib()
    L = np.ascontiguousarray(L, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    out = np.zeros(3)
    lib.orc_displacement(_ptr(L), _ptr(a), _ptr(b), _ptr(out))
    return out


def fitted_inside(L, a):
    lib = port_lib()
    L = np.ascontiguousarray(L, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = np.zeros(3)
    lib.orc_fitted_inside(_ptr(L), _ptr(a), _ptr(out))
    return out


def linkedcell_geometry(L, cutoff, nx, ny, nz, mode_auto=False):
    lib = port_lib()
    L = np.ascontiguousarray(L, dtype=np.float64)
    n = (ctypes.c_int * 3)()
    side = ctypes.c_int(0)
    ci = ctypes.c_int(0)
    _check(lib.orc_linkedcell_geometry(_ptr(L), cutoff, nx, ny, nz, int(mode_auto), n,
                                       ctypes.byref(side), ctypes.byref(ci)))
    return tuple(n), side.value, ci.value


def run_port(pos, L, Z, mass, vel, cm, cm_args, pots, dt, nsteps, neigh=None, flags=None, integrator=None):
    """Same protocol as run_reference, on the C restatement."""
    sim = PortSim(pos, L, Z, mass, vel, flags)
    sim.set_cell_manager(cm, cm_args)
    for name, args, s1, s2 in pots:
        sim.add_potential(name, args, s1, s2)
    if nsteps > 0:
        sim.set_integrator(dt, *(integrator or ("velocityverlet", "")))
    sim.update_forces()
    out = {"acc0": sim.atoms()[2], "thermo0": sim.thermo()}
    if neigh is not None:
        out["neigh_counts"], out["neigh_idx"] = sim.neighbors(*neigh)
    out["thermo"] = sim.do_steps(nsteps) if nsteps > 0 else np.zeros((0, THERMO_LEN))
    out["pos"], out["vel"], out["acc"] = sim.atoms()
    return out


# --------------------------------------------------------------------------------------------
# The reference itself (only where oracle/_ref was built from the reference sources)
# --------------------------------------------------------------------------------------------

_REF = None


def reference_available() -> bool:
    return REF_LIB.exists()


def _ref():
    global _REF
    if _REF is None:
        lib = ctypes.CDLL(str(REF_LIB))
        lib.ref_last_error.restype = ctypes.c_char_p
        lib.ref_run.restype = ctypes.c_int
        lib.ref_write_frames.restype = ctypes.c_int
        _REF = lib
    return _REF


def run_reference(pos, L, symbol, vel, cm, cm_args, pots, dt, nsteps, neigh=None, integrator=None):
    """Runs the reference plugins (see ref_driver.cpp) and returns its outputs.

    pots: list of (name, args, s1, s2).  neigh: (full, rcut) to export neighbour lists after
    the initial force evaluation.  integrator: (name, extra args) of the integrator plugin
    (velocityverlet when None); "dt" is added.
    """
    lib = _ref()
    if integrator is not None:
        # these three need the runtime context supplied to the backed-up configuration (the
        # unmodified reference throws MissingComponent at their first step; ref_driver.cpp)
        supply = integrator[0] in ("leapfrog", "beeman", "nosehoover")
        lib.ref_set_integrator(integrator[0].encode(), integrator[1].encode(), ctypes.c_int(int(supply)))
    n = len(pos)
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
    L = np.ascontiguousarray(L, dtype=np.float64)
    names = (ctypes.c_char_p * len(pots))(*[p[0].encode() for p in pots])
    args = (ctypes.c_char_p * len(pots))(*[p[1].encode() for p in pots])
    spc = np.array([[p[2], p[3]] for p in pots], dtype=np.int32).ravel()
    mass = np.zeros(n)
    acc0 = np.zeros((n, 3))
    th0 = np.zeros(THERMO_LEN)
    th = np.zeros((max(nsteps, 1), THERMO_LEN))
    pf, vf, af = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    counts = np.zeros(n, dtype=np.int64)
    total = ctypes.c_int64(0)
    cap = 0
    idx = None
    full, rcut = (0, 0.0) if neigh is None else (int(neigh[0]), float(neigh[1]))
    if neigh is not None:
        cap = n * 512
        idx = np.zeros(cap, dtype=np.int64)
    rc = lib.ref_run(
        ctypes.c_int64(n), _ptr(L), symbol.encode(), _ptr(pos), _ptr(vel), cm.encode(), cm_args.encode(),
        ctypes.c_int(len(pots)), names, args, _ptr(spc, ctypes.POINTER(ctypes.c_int32)),
        ctypes.c_double(dt), ctypes.c_int64(nsteps), _ptr(mass), _ptr(acc0), _ptr(th0),
        ctypes.c_int(full), ctypes.c_double(rcut),
        _ptr(counts, _I64) if neigh is not None else None, _ptr(idx, _I64) if neigh is not None else None,
        ctypes.c_int64(cap), ctypes.byref(total) if neigh is not None else None,
        _ptr(th), _ptr(pf), _ptr(vf), _ptr(af))
    if rc:
        raise OracleError("reference: " + lib.ref_last_error().decode())
    out = {"mass": mass, "acc0": acc0, "thermo0": th0, "thermo": th[:nsteps], "pos": pf, "vel": vf, "acc": af}
    if neigh is not None:
        out["neigh_counts"] = counts
        out["neigh_idx"] = idx[: total.value]
    return out


def write_reference_dump(path, L, Z, pos, vel, acc, flags=None) -> None:
    """Simulation::Dump of the reference (see ref_driver.cpp) for these atoms at step 0."""
    lib = _ref()
    n = len(pos)
    arr = [np.ascontiguousarray(x, dtype=np.float64) for x in (L, pos, vel, acc)]
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    fl = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
    rc = lib.ref_dump(ctypes.c_int64(n), _ptr(arr[0]), _ptr(Z, ctypes.POINTER(ctypes.c_int32)), _ptr(arr[1]),
                      _ptr(arr[2]), _ptr(arr[3]), None if fl is None else fl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                      str(path).encode())
    if rc:
        raise OracleError("reference: " + lib.ref_last_error().decode())


def write_reference_frames(path, module: str, args: str, L, Z, pos, vel=None, acc=None) -> None:
    """Writes frames [nframes, n, 3] through the reference's own output plugin (lpmd / xyz,
    see ref_driver.cpp); `args` must name `path` with its `file` keyword."""
    lib = _ref()
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    nf, n = pos.shape[0], pos.shape[1]
    vel = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
    acc = None if acc is None else np.ascontiguousarray(acc, dtype=np.float64)
    L = np.ascontiguousarray(L, dtype=np.float64)
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    rc = lib.ref_write_frames(ctypes.c_int64(n), _ptr(L), _ptr(Z, ctypes.POINTER(ctypes.c_int32)), ctypes.c_int64(nf),
                              _ptr(pos), _ptr(vel), _ptr(acc), module.encode(), args.encode(), str(path).encode())
    if rc:
        raise OracleError("reference: " + lib.ref_last_error().decode())
