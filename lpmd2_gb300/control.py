"""LPMD control files on the GPU.

    python -m lpmd2_gb300.control run.control [--precision fp64|mixed] [--strict] [--device N]

Reads the control-file language of the lpmd program (lpmd/controlparser.cc: statements with
positional and key=value arguments, `use <plugin> [as <id>] ... enduse` blocks) and runs the
simulation it describes through libgbmd:

  cell cubic a [scale] | cell crystal a b c 90 90 90 [scale]    orthogonal periodic box
  input crystal3d type=fcc|bcc|sc|hcp symbol=X nx= ny= nz=     initial lattice (crystal3d)
  input module=lpmd|xyz file=F                                 first configuration of a file
  prepare temperature t=T [seed=S]                             velocities (see below)
  use linkedcell|verletlist|minimumimage|lcbinary|lennardjones|fastlj|suttonchen|gupta|finnissinclair|
      finnissinclair-ext|velocityverlet|euler|leapfrog|verlet|
      beeman|nosehoover [as id] ... enduse                     the timestep's plugins
  cellmanager <id> / potential <id> A B / integrator <id>      wiring (ids of use blocks)
  steps N                                                      velocity-Verlet steps
  monitor p1,p2,... [start= end= each= output=]                thermo columns (monitor.cc)
  use tempscaling|temperature|berendsen ... enduse; apply <id>  thermostats between steps
  output xyz <file> [each= start= end= level= precout=]        XYZ frames (xyz.cc)
  output module=lpmd file=F [level= type=lpmd|zlp blocksize= compression= extra=TYPE]
                                                               lpmd / zlp frames (lpmd.cc)
  mass <symbol> <value>, set <option> <value>, periodic x y z
  set restore-file F / dumping-each N / dumping-file F / lastconfig F   text dumps (Dump/Restore)

Thermo comes from the device's per-step record, so monitored steps cost no extra
synchronisation; positions are copied back only for the output frames.  Thermostats
(tempscaling, temperature, berendsen) rescale velocities on the device between steps, on the
schedule of their `apply` statements.  Statements of modules outside the timestep (property,
visualize, filter, average, other plugins' use blocks and applies) are reported and skipped,
or rejected with --strict.

`prepare temperature` draws seeded Maxwell-Boltzmann velocities with zero total momentum,
rescaled to exactly T (seed 1 unless `seed=` is given): the reference's modifier is seeded from
the clock and gives every atom the same speed, so no run of it can be reproduced anyway.
"""
from __future__ import annotations

import argparse
import dataclasses
import math
import sys
from pathlib import Path
from typing import TextIO

import numpy as np

from . import formats as F
from . import inputs as I

TIMESTEP_PLUGINS = {"linkedcell", "verletlist", "minimumimage", "lcbinary", "lennardjones", "fastlj", "suttonchen", "gupta",
                    "finnissinclair",
                    "finnissinclair-ext", "velocityverlet", "euler", "leapfrog", "verlet", "beeman", "nosehoover"}
MODIFIER_PLUGINS = {"tempscaling", "temperature", "berendsen"}
SKIPPED_STATEMENTS = {"property", "visualize", "filter", "average", "bond", "charge", "plugindir"}

# Element symbols in order of atomic number (the periodic table up to Rn).
_SYMBOLS = ("H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
            "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm "
            "Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn").split()
ATOMIC_NUMBER = {s: k + 1 for k, s in enumerate(_SYMBOLS)}
# Standard atomic weights (amu) of common MD species; the values the reference uses where it
# is the source (inputs.MASSES) take precedence.  Others need a `mass` statement.
STANDARD_MASS = {"H": 1.008, "He": 4.0026, "Ne": 20.180, "Kr": 83.798, "Xe": 131.29, "Al": 26.982, "Ni": 58.693,
                 "Ag": 107.87, "Au": 196.97, "Pt": 195.08, "Pd": 106.42, "W": 183.84, "Ta": 180.95, "Nb": 92.906,
                 "V": 50.942, "Cr": 51.996, "Ti": 47.867, "Zr": 91.224, **I.MASSES}


class ControlError(ValueError):
    pass


@dataclasses.dataclass
class Control:
    cell: np.ndarray | None = None
    input: dict | None = None
    prepares: list[dict] = dataclasses.field(default_factory=list)
    outputs: list[dict] = dataclasses.field(default_factory=list)
    monitors: list[dict] = dataclasses.field(default_factory=list)
    uses: dict[str, tuple[str, str]] = dataclasses.field(default_factory=dict)  # id -> (plugin, args)
    modifiers: dict[str, tuple[str, str]] = dataclasses.field(default_factory=dict)  # id -> (plugin, args)
    applies: list[tuple[str, dict]] = dataclasses.field(default_factory=list)  # (id, statement args)
    cellmanager: str | None = None
    potentials: list[tuple[str, str, str]] = dataclasses.field(default_factory=list)
    integrator: str | None = None
    steps: int = 0
    masses: dict[str, float] = dataclasses.field(default_factory=dict)
    options: dict[str, str] = dataclasses.field(default_factory=dict)
    periodic: tuple[bool, bool, bool] = (True, True, True)
    skipped: list[str] = dataclasses.field(default_factory=list)


def _args(words: list[str], positional: list[str]) -> dict:
    """Positional values fill `positional` in order; key=value words set keys."""
    out: dict[str, str] = {}
    k = 0
    for w in words:
        if "=" in w:
            key, val = w.split("=", 1)
            out[key] = val
        else:
            if k >= len(positional):
                raise ControlError(f"unexpected argument {w!r}")
            out[positional[k]] = w
            k += 1
    return out


def _true(v: str) -> bool:
    return v.lower() in ("true", "yes", "1", "on")


def parse(text: str, strict: bool = False) -> Control:
    ctl = Control()
    lines = [ln.split("#", 1)[0].strip() for ln in text.splitlines()]
    i = 0
    while i < len(lines):
        ln = lines[i]
        i += 1
        if not ln:
            continue
        w = ln.split()
        name = w[0]
        if name == "use":
            if len(w) < 2:
                raise ControlError("use without a plugin name")
            plugin, uid = w[1], w[1]
            if len(w) >= 4 and w[2] == "as":
                uid = w[3]
            body = []
            while i < len(lines) and lines[i] != "enduse":
                if lines[i]:
                    body.append(lines[i])
                i += 1
            if i >= len(lines):
                raise ControlError(f"use {plugin}: missing enduse")
            i += 1
            if plugin in TIMESTEP_PLUGINS:
                ctl.uses[uid] = (plugin, " ".join(body))
            elif plugin in MODIFIER_PLUGINS:
                ctl.modifiers[uid] = (plugin, " ".join(body))
            else:
                ctl.skipped.append(f"use {plugin}")
            continue
        rest = w[1:]
        if name == "cell":
            if not rest:
                raise ControlError("cell without a type")
            kind = rest[0]
            if kind == "cubic":
                a = _args(rest[1:], ["a", "scale"])
                L = float(a["a"]) * float(a.get("scale", 1.0))
                ctl.cell = np.array([L, L, L])
            elif kind == "crystal":
                a = _args(rest[1:], ["a", "b", "c", "alpha", "beta", "gamma", "scale"])
                if "b" not in a:  # a crystal cell given by `a` alone is cubic (lpmd/controlparser.cc:81-87)
                    a["b"] = a["c"] = a["a"]
                if any(abs(float(a.get(k, 90.0)) - 90.0) > 1e-12 for k in ("alpha", "beta", "gamma")):
                    raise ControlError("only orthogonal cells run on the GPU path")
                sc = float(a.get("scale", 1.0))
                ctl.cell = np.array([float(a["a"]) * sc, float(a["b"]) * sc, float(a["c"]) * sc])
            else:
                raise ControlError(f"cell {kind}: only cubic and orthogonal crystal cells are supported")
        elif name == "input":
            a = _args(rest, ["module"])
            ctl.input = a
        elif name == "prepare":
            ctl.prepares.append(_args(rest, ["module"]))
        elif name == "output":
            ctl.outputs.append(_args(rest, ["module", "file"]))
        elif name == "monitor":
            ctl.monitors.append(_args(rest, ["properties", "start", "end", "each", "output"]))
        elif name == "steps":
            ctl.steps = int(rest[0])
        elif name == "cellmanager":
            ctl.cellmanager = rest[0]
        elif name == "potential":
            a = _args(rest, ["module", "a", "b"])
            ctl.potentials.append((a["module"], a["a"], a["b"]))
        elif name == "integrator":
            ctl.integrator = rest[0]
        elif name == "mass":
            ctl.masses[rest[0]] = float(rest[1])
        elif name == "set":
            ctl.options[rest[0]] = rest[1] if len(rest) > 1 else ""
        elif name == "periodic":
            ctl.periodic = tuple(_true(x) for x in rest[:3])
        elif name == "apply":
            a = _args(rest, ["module"]) if "over" not in rest else {}
            if a.get("module") in ctl.modifiers:
                ctl.applies.append((a.pop("module"), a))
            else:
                ctl.skipped.append(ln)
        elif name in SKIPPED_STATEMENTS:
            ctl.skipped.append(ln)
        else:
            raise ControlError(f"unknown statement {name!r}")
    if strict and ctl.skipped:
        raise ControlError("outside the GPU timestep path: " + "; ".join(ctl.skipped))
    return ctl


def _species(symbol: str, ctl: Control) -> tuple[int, float]:
    if symbol not in ATOMIC_NUMBER:
        raise ControlError(f"unknown element {symbol!r}")
    mass = ctl.masses.get(symbol, STANDARD_MASS.get(symbol))
    if mass is None:
        raise ControlError(f"no mass for {symbol}: add a `mass {symbol} <amu>` statement")
    return ATOMIC_NUMBER[symbol], mass


def crystal3d(kind: str, nx: int, ny: int, nz: int, L: np.ndarray) -> np.ndarray:
    """Sites of crystal3d's lattices (plugins/crystal3d.cc:62-131) in the cell L: k outer, then
    j, then i, with the plugin's fractional offsets."""
    ax, ay, az = 1.0 / nx, 1.0 / ny, 1.0 / nz
    basis = {"fcc": ((0.51, 0.5, 0.5), (0.51, 0.0, 1.0), (1.01, 0.0, 0.5), (1.01, 0.5, 1.0)),
             "bcc": ((0.0, 0.0, 0.0), (0.5, 0.5, 0.5)), "sc": ((0.0, 0.0, 0.0),),
             "hcp": ((2.0 / 3.0, 1.0 / 3.0, 3.0 / 4.0), (1.0 / 3.0, 2.0 / 3.0, 1.0 / 4.0))}.get(kind)
    if basis is None:
        raise ControlError(f"crystal3d type {kind!r} is not supported")
    out = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                for b in basis:
                    out.append(((i + b[0]) * ax * L[0], (j + b[1]) * ay * L[1], (k + b[2]) * az * L[2]))
    return np.array(out, dtype=np.float64)


def _active(step: int, start: int, end: int, each: int) -> bool:
    """Stepper::IsActiveInStep (liblpmd/lpmd/stepper.h:17-25)."""
    if step < start or (end != -1 and step > end):
        return False
    return (step - start) % each == 0


def _kv(args: str) -> dict:
    w = args.split()
    return {w[k]: w[k + 1] for k in range(0, len(w) - 1, 2)}


def modifier_schedule(ctl: Control, dt: float, first_step: int = 0) -> list[tuple[int, int, float, float]]:
    """The velocity rescalings the applied modifiers make, as (step, mode, target T, dt/tau)
    after that step, in the order lpmd runs them (Application::RunModifiers after DoStep,
    lpmd/application.cc:403-464).  Stepper activity and the linear ramp follow
    liblpmd/lpmd/stepper.h:17-31, with `end` -1 replaced by the step count; tempscaling and
    temperature call SetTemperature (plugins/tempscaling.cc:66-71, plugins/temperature.cc:35-39);
    berendsen (plugins/berendsen.cc:72-99) switches itself on at its first active step (no
    rescaling then), applies every step until tau/dt steps later, and switches off on the
    step after."""
    out = []
    mods = []
    for uid, extra in ctl.applies:
        plugin, body = ctl.modifiers[uid]
        kw = {"start": "0", "end": "-1", "each": "1", "from": "300.0", "to": "300.0", "t": "300.0", "tau": "400.0"}
        kw.update(_kv(body))
        kw.update(extra)
        if int(kw["each"]) == 0:
            kw.update(start="0", end="-1", each="1")
        st = dict(plugin=plugin, start=int(kw["start"]), end=int(kw["end"]), each=int(kw["each"]),
                  frm=float(kw["from"]), to=float(kw["to"]), t=float(kw["t"]), tau=float(kw["tau"]), stop=-1,
                  old_each=None)
        if st["end"] == -1:
            st["end"] = ctl.steps
        mods.append(st)

    def ramp(m, k):
        if m["start"] == m["end"]:
            return m["frm"]
        return m["frm"] + float(k - m["start"]) / float(m["end"] - m["start"]) * (m["to"] - m["frm"])

    for k in range(first_step + 1, ctl.steps + 1):  # a restored run starts after its dump's step
        for m in mods:
            if not _active(k, m["start"], m["end"], m["each"]):
                continue
            if m["plugin"] == "tempscaling":
                out.append((k, 0, ramp(m, k), 0.0))
            elif m["plugin"] == "temperature":
                out.append((k, 0, m["t"], 0.0))
            else:  # berendsen
                if m["stop"] == -1:
                    m["stop"] = int(float(k) + m["tau"] / dt)
                    m["old_each"], m["each"] = m["each"], 1
                elif k <= m["stop"]:
                    out.append((k, 1, ramp(m, k), dt / m["tau"]))
                else:
                    m["stop"] = -1
                    m["each"] = m["old_each"]
    return out


def _tags(rec: np.ndarray, natoms: int, L: np.ndarray, masses: np.ndarray) -> dict:
    """The numeric tags SetSimulationTags sets (liblpmd/simulation/simulationbuilder.cc:84-124)
    from one thermo record."""
    vol = rec[9]
    p = rec[6:9]
    t = {"step": int(round(rec[0])), "potential-energy": rec[1], "kinetic-energy": rec[2], "total-energy": rec[3],
         "temperature": rec[4], "virial": rec[5], "px": p[0], "py": p[1], "pz": p[2],
         "momentum": float(np.sqrt(np.sum(p * p))), "volume": vol, "volume-per-atom": vol / natoms,
         "cell-a": L[0], "cell-b": L[1], "cell-c": L[2], "particle-density": natoms / vol,
         "density": 1.66054 * float(masses.sum()) / vol, "virial-pressure": rec[10], "kinetic-pressure": rec[11],
         "pressure": rec[12]}
    comp = "xyz"
    for q in range(3):
        for r in range(3):  # tag s<q><r> = pressfactor / V * stress[q][r]
            t["s" + comp[q] + comp[r]] = (160217.65 / vol) * rec[13 + 3 * q + r]
    return t


def _fmt(v) -> str:
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    return f"{float(v):g}"  # a tag holds the value as text with 6 significant digits


def run(ctl: Control, device: int = 0, precision: str | None = None, out: TextIO = sys.stdout,
        workdir: Path | str = ".") -> dict:
    """Runs the control file's simulation; returns the final state and the monitored rows."""
    from . import gbmd

    workdir = Path(workdir)
    if ctl.cell is None:
        raise ControlError("no cell statement")
    if not all(ctl.periodic):
        raise ControlError("the GPU path runs fully periodic cells only")
    inp = ctl.input or {}
    cell = np.asarray(ctl.cell, dtype=np.float64)
    step0 = 0
    flags = None
    restore = ctl.options.get("restore-file")
    if restore:
        # LPMD::RestoreSimulation -> Simulation::Restore (lpmd/lpmd.cc:32-50,
        # liblpmd/simulation/simulationbuilder.cc:240-293): atoms, cell and step from a dump; no
        # input module and no prepares (lpmd/application.cc:59); the run continues from the step
        path = Path(restore)
        path = path if path.is_absolute() else workdir / path
        try:
            d = F.read_dump(path)
        except (OSError, ValueError, IndexError) as e:
            raise ControlError(f"restore-file: {e}") from None
        cell = np.asarray(d["L"], dtype=np.float64)
        pos, vel, Z = d["pos"], d["vel"], d["Z"]
        n = len(pos)
        syms = [_SYMBOLS[int(z) - 1] for z in Z]
        table = {sy: _species(sy, ctl) for sy in set(syms)}
        masses = np.array([table[sy][1] for sy in syms])
        symbols = syms[0] if len(table) == 1 else syms
        step0 = d["step"]
        flags = d["flags"] if d["flags"].any() else None
    elif inp.get("module") == "crystal3d":
        symbols = inp.get("symbol", "H")
        Z, mass = _species(symbols, ctl)
        pos = crystal3d(inp.get("type", "fcc"), int(inp.get("nx", 1)), int(inp.get("ny", 1)), int(inp.get("nz", 1)),
                        cell)
        n = len(pos)
        masses = np.full(n, mass)
        vel = np.zeros((n, 3))
    elif inp.get("module") in ("lpmd", "xyz"):
        # CellReader::ReadCell of the first configuration (Application::FillAtomsFromCellReader,
        # lpmd/application.cc:207-237); accelerations are recomputed before the first step
        path = Path(inp.get("file", ""))
        path = path if path.is_absolute() else workdir / path
        try:
            fr = (F.read_lpmd(path) if inp["module"] == "lpmd" else F.read_xyz(path))[0]
        except (OSError, ValueError, IndexError, KeyError) as e:
            raise ControlError(f"input {inp['module']}: {e}") from None
        if inp["module"] == "lpmd" and _true(ctl.options.get("replacecell", "false")):
            cell = np.asarray(fr["L"], dtype=np.float64)
        pos, vel = fr["pos"], fr["vel"]
        if inp["module"] == "xyz" and not ((pos >= 0.0) & (pos < cell)).all():
            raise ControlError("input xyz: an atom was found outside the cell")  # external=consider
        n = len(pos)
        table = {s: _species(s, ctl) for s in set(fr["symbols"])}
        Z = np.array([table[s][0] for s in fr["symbols"]], dtype=np.int32)
        masses = np.array([table[s][1] for s in fr["symbols"]])
        symbols = fr["symbols"][0] if len(table) == 1 else fr["symbols"]
    else:
        raise ControlError("input: the crystal3d generator and lpmd/zlp/xyz files run on the GPU path")
    for pr in ([] if restore else ctl.prepares):
        if pr.get("module") != "temperature":
            raise ControlError(f"prepare {pr.get('module')}: not supported on the GPU path")
        vel = I.maxwell_boltzmann(masses, float(pr.get("t", "0")), seed=int(pr.get("seed", "1")))

    def plugin(uid: str, role: str):
        if uid not in ctl.uses:
            raise ControlError(f"{role} {uid!r}: no use block for it (or its plugin is not on the GPU path)")
        name, args = ctl.uses[uid]
        return gbmd.Plugin(name, args)

    if ctl.cellmanager is None:
        raise ControlError("MissingComponent: cellmanager")
    if not ctl.potentials:
        raise ControlError("MissingComponent: potential")
    if ctl.integrator is None:
        raise ControlError("MissingComponent: integrator")
    sim = gbmd.Simulation(n, cell, device=device)
    sim.set_atoms(pos, vel, Z=Z, mass=masses)
    if flags is not None:
        sim.set_flags(flags)
    sim.set_cell_manager(plugin(ctl.cellmanager, "cellmanager"))
    for uid, a, b in ctl.potentials:
        s1 = -1 if a == "all" else ATOMIC_NUMBER[a]
        s2 = -1 if b == "all" else ATOMIC_NUMBER[b]
        sim.add_potential(plugin(uid, "potential"), s1, s2)
    integ = plugin(ctl.integrator, "integrator")
    sim.set_integrator(integ)
    prec = precision or ctl.options.get("precision", "fp64")
    sim.set_precision(prec)
    sim.update_forces()
    sim.thermo_log()  # the records of the set-up evaluation are not steps

    monitors = []
    for m in ctl.monitors:
        props = m.get("properties", "step").split(",")
        dest = m.get("output", "-")
        stream = out if dest in ("-", "") else open(workdir / dest, "w")
        monitors.append((props, int(m.get("start", 0)), int(m.get("end", -1)), max(1, int(m.get("each", 1))), stream))
    outputs = []
    for o in ctl.outputs:
        kw = {k: v for k, v in o.items() if k not in ("module", "file", "start", "end", "each")}
        try:
            w = F.open_writer(o.get("module", ""), workdir / o.get("file", "noname"), **kw)
        except (ValueError, TypeError) as e:
            raise ControlError(f"output {o.get('module')}: {e}") from None
        w.write_header()  # Application::OpenOutputStreams (lpmd/application.cc:537-556)
        outputs.append((w, int(o.get("start", 0)), int(o.get("end", -1)), max(1, int(o.get("each", 1))), None))
    rows = []

    def emit_frame(w, _):
        p, v, a = sim.atoms()
        w.write_frame(symbols, cell, p, v, a)

    dt = float(_kv(ctl.uses[ctl.integrator][1]).get("dt", "1.0"))
    schedule = modifier_schedule(ctl, dt, first_step=step0)
    by_step: dict[int, list] = {}
    for st_, mode, target, dtt in schedule:
        by_step.setdefault(st_, []).append((mode, target, dtt))
    # Simulation::Dump every `dumping-each` steps into `dumping-file`, and into `lastconfig` at
    # the end (lpmd/lpmd.cc:84-104; lastconfig defaults to lastconfig.dump, controlparser.cc:56)
    dump_each = int(ctl.options.get("dumping-each", "0") or 0)
    dump_file = ctl.options.get("dumping-file", "dump.dump")
    last_file = ctl.options.get("lastconfig", "lastconfig.dump")
    dump_steps = {t for t in range(step0 + 1, ctl.steps + 1) if _active(t, 0, ctl.steps, dump_each)} if dump_each > 0 else set()

    def dump(name: str, step: int):
        p_, v_, a_ = sim.atoms()
        F.write_dump(workdir / name, step, cell, Z if np.ndim(Z) else np.full(n, Z), p_, v_, a_, flags)

    done = step0
    while done < ctl.steps:
        # run to the next output frame, modifier or full thermo log, then report the chunk
        k = min(ctl.steps - done, 1000)
        for f, st, en, ev, lv in outputs:
            for s in range(done + 1, done + k + 1):
                if _active(s, st, en, ev):
                    k = s - done
                    break
        nxt = [t for t in by_step if done < t <= done + k] + [t for t in dump_steps if done < t <= done + k]
        if nxt:
            k = min(nxt) - done
        sim.do_steps(k)
        done += k
        # modifiers, then monitor and output (lpmd/lpmd.cc:93-101): a rescaling step's thermo
        # record already shows the new velocities
        for mode, target, dtt in by_step.get(done, []):
            if mode == 0:
                sim.set_temperature(target)
            else:
                sim.berendsen(target, dtt)
        log = sim.thermo_log()
        for rec in log:
            rec = rec.copy()
            rec[0] += step0  # the device counts the steps of this run
            step = int(round(rec[0]))
            tags = None
            for props, st, en, ev, stream in monitors:
                if _active(step, st, en, ev):
                    tags = tags or _tags(rec, n, cell, masses)
                    vals = []
                    for p in props:
                        if p not in tags:
                            raise ControlError(f"monitor: property {p!r} is not available on the GPU path")
                        vals.append(tags[p])
                    stream.write("  ".join(_fmt(v) for v in vals) + "  \n")
                    rows.append([float(v) for v in vals])
        for f, st, en, ev, lv in outputs:
            if _active(done, st, en, ev):
                emit_frame(f, lv)
        if done in dump_steps:
            dump(dump_file, done)
    dump(last_file, done)
    for *_, stream in monitors:
        if stream is not out:
            stream.close()
    for w, *_ in outputs:
        w.close()
    p, v, a = sim.atoms()
    th = sim.thermo()
    sim.close()
    return {"natoms": n, "steps": ctl.steps, "pos": p, "vel": v, "acc": a, "thermo": th, "rows": rows,
            "skipped": list(ctl.skipped)}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m lpmd2_gb300.control", description=__doc__.splitlines()[0])
    ap.add_argument("control")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default=None)
    ap.add_argument("--strict", action="store_true", help="reject statements outside the timestep path")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    path = Path(a.control)
    ctl = parse(path.read_text(), strict=a.strict)
    for s in ctl.skipped:
        print(f"# skipped (not on the GPU timestep path): {s}", file=sys.stderr)
    run(ctl, device=a.device, precision=a.precision, workdir=path.parent)
    return 0


if __name__ == "__main__":
    sys.exit(main())
