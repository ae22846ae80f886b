"""LPMD configuration files written from device snapshots, and read back.

Writers produce the bytes of the reference's own output plugins for orthogonal cells:

  xyz   XYZFormat::WriteCell (plugins/xyz.cc:218-242): "N", an empty title line, then
        "SYM x y z [vx vy vz [ax ay az]]" in fixed notation with `precout` digits (default 8).
  lpmd  LPMDFormat::WriteHeader / WriteCell (plugins/lpmd.cc:522-640): header
        "LPMD 2.0 L" + "HDR SYM X Y Z [VX VY VZ] [AX AY AZ] ", then per frame "N", the nine
        cell-vector components and "SYM fx fy fz [v] [a]" with fractional positions, all in
        iostream fixed notation (6 digits).
  zlp   the same frame text, deflated: one zlib stream per file (compression level 6 by
        default), each frame compressed in `blocksize`-byte pieces with a sync flush after each,
        and prefixed by a 9-byte record: the byte 8 (sizeof(unsigned long)) and the compressed
        size as the reference stores it on LP64 little-endian hosts (htonl of the 32-bit size
        in an 8-byte word: 4 big-endian bytes, then 4 zero bytes).  The header says "LPMD 2.0 Z".

  dump  Simulation::Dump / Restore (liblpmd/simulation/simulationbuilder.cc:195-293), the text
        checkpoint behind `lastconfig`, `dumping-each` and `restore-file`: the step, the cell
        vectors, "Z x y z vx vy vz ax ay az " per atom in iostream's default notation (6
        significant digits), then a colour line ("false ") and a tag line per atom.

Values are C-formatted ("%.6f" / "%.8f" / "%g"), which rounds exactly as iostream's fixed and
default notations do.  Readers accept what the writers (and the reference) write: xyz frames, and lpmd/zlp
version 2.0 files (LPMDFormat::ReadHeader / ReadCell, plugins/lpmd.cc:125-430) with their
HDR column list.  The reference's legacy 1.0 and binary-header "Z4L2P" variants are not read.
"""
from __future__ import annotations

import zlib
from pathlib import Path

import numpy as np


def _rows(symbols, n: int, cols: list[np.ndarray], prec: int, tail: str = "") -> str:
    """One line per atom: "SYM c0 c1 ..." with every column in %.{prec}f."""
    data = np.hstack([np.asarray(c, dtype=np.float64).reshape(n, 3) for c in cols])
    fmt = " ".join([f"%.{prec}f"] * data.shape[1])
    if isinstance(symbols, str):
        line = symbols + " " + fmt + tail + "\n"
        return "".join(line % tuple(r) for r in data)
    return "".join(s + " " + (fmt % tuple(r)) + tail + "\n" for s, r in zip(symbols, data))


def _symbols(symbols, n: int):
    """A single symbol for all atoms stays a string (fast path); otherwise a list of n."""
    if isinstance(symbols, str):
        return symbols
    s = [str(x) for x in symbols]
    if len(s) != n:
        raise ValueError(f"{len(s)} symbols for {n} atoms")
    return s


def _level_cols(level: int, pos, vel, acc) -> list:
    cols = [pos]
    if level >= 1:
        if vel is None:
            raise ValueError("level >= 1 needs velocities")
        cols.append(vel)
    if level >= 2:
        if acc is None:
            raise ValueError("level 2 needs accelerations")
        cols.append(acc)
    return cols


class XYZWriter:
    """XYZFormat output (plugins/xyz.cc).  `inside` is not applied: device positions are always
    inside the cell after a step (FittedInside)."""

    def __init__(self, path, level: int = 0, precout: int = 8):
        if level not in (0, 1, 2):
            raise ValueError("xyz level must be 0, 1 or 2")
        self.level, self.prec = int(level), int(precout)
        self.f = open(path, "w")

    def write_header(self):
        pass  # XYZFormat::WriteHeader writes nothing

    def write_frame(self, symbols, L, pos, vel=None, acc=None):
        n = len(pos)
        sym = _symbols(symbols, n)
        self.f.write(f"{n}\n\n")
        self.f.write(_rows(sym, n, _level_cols(self.level, pos, vel, acc), self.prec))

    def close(self):
        self.f.close()


def _file_type(path: str, type_: str) -> str:
    """LPMDFormat's constructor: the file name decides ("...lpmd" / "....zlp"), else `type`."""
    if path[-4:] == "lpmd":
        return "lpmd"
    if path[-4:] == ".zlp":
        return "zlp"
    if type_ not in ("lpmd", "zlp"):
        raise ValueError(f"lpmd: unknown type {type_!r}")
    return type_


class LPMDWriter:
    """LPMDFormat output (plugins/lpmd.cc) for orthogonal cells; `extra` may hold TYPE."""

    def __init__(self, path, level: int = 0, type: str = "lpmd", blocksize: int = 1024, compression: int = 6,
                 extra: str = ""):
        if level not in (0, 1, 2):
            raise ValueError("lpmd level must be 0, 1 or 2")
        self.level = int(level)
        self.type = _file_type(str(path), type)
        self.blocksize = int(blocksize)
        if self.blocksize <= 0:
            raise ValueError("blocksize must be positive")
        self.extra = [e for e in str(extra).split(",") if e]
        for e in self.extra:
            if e not in ("TYPE", "type"):
                raise ValueError(f"lpmd: extra column {e!r} is not written (atom colours are not kept)")
        self.z = zlib.compressobj(int(compression)) if self.type == "zlp" else None
        self.f = open(path, "wb")

    def header_bytes(self) -> bytes:
        hdr = ["SYM", "X", "Y", "Z"]
        if self.level >= 1:
            hdr += ["VX", "VY", "VZ"]
        if self.level >= 2:
            hdr += ["AX", "AY", "AZ"]
        hdr += self.extra
        flag = "Z" if self.type == "zlp" else "L"
        return f"LPMD 2.0 {flag}\nHDR {''.join(h + ' ' for h in hdr)}\n".encode()

    def write_header(self):
        self.f.write(self.header_bytes())

    def frame_text(self, symbols, L, pos, vel=None, acc=None) -> str:
        n = len(pos)
        L = np.asarray(L, dtype=np.float64).reshape(3)
        box = np.diag(L).reshape(9)
        frac = np.asarray(pos, dtype=np.float64) / L  # OrthogonalCell::Fractional
        tail = "          ATOMTYPE" * len(self.extra)
        return (f"{n}\n" + " ".join("%.6f" % x for x in box) + "\n" +
                _rows(_symbols(symbols, n), n, _level_cols(self.level, frac, vel, acc), 6, tail))

    def write_frame(self, symbols, L, pos, vel=None, acc=None):
        text = self.frame_text(symbols, L, pos, vel, acc).encode()
        if self.type == "lpmd":
            self.f.write(text)
            return
        parts = []
        for k in range(0, len(text), self.blocksize):
            parts.append(self.z.compress(text[k:k + self.blocksize]))
            parts.append(self.z.flush(zlib.Z_SYNC_FLUSH))
        cbuf = b"".join(parts)
        if len(cbuf) >= 1 << 32:
            raise ValueError("zlp frame larger than 4 GiB")
        self.f.write(bytes([8]) + len(cbuf).to_bytes(4, "big") + bytes(4) + cbuf)

    def close(self):
        self.f.close()


def open_writer(module: str, path, **kw):
    """The writer of an `output module=... file=...` statement."""
    if module == "xyz":
        return XYZWriter(path, level=int(kw.get("level", 0)), precout=int(kw.get("precout", 8)))
    if module == "lpmd":
        return LPMDWriter(path, level=int(kw.get("level", 0)), type=str(kw.get("type", "lpmd")),
                          blocksize=int(kw.get("blocksize", 1024)), compression=int(kw.get("compression", 6)),
                          extra=str(kw.get("extra", "")))
    raise ValueError(f"output module {module!r}: only xyz and lpmd are written")


# ----------------------------------------------------------------------------------------------
# Readers
# ----------------------------------------------------------------------------------------------


def _frame_from_lines(lines: list[str], hdr: list[str]) -> dict:
    n = int(lines[0].split()[0])
    w = [float(x) for x in lines[1].split()]
    if len(w) != 9:
        raise ValueError("lpmd: expected nine cell-vector components")
    cell = np.array(w).reshape(3, 3)
    L = np.sqrt((cell ** 2).sum(axis=1))
    cols = hdr[1:]
    sym, data = [], np.zeros((n, 9))
    idx = {c: k for k, c in enumerate(["X", "Y", "Z", "VX", "VY", "VZ", "AX", "AY", "AZ"])}
    for i in range(n):
        words = lines[2 + i].split()
        if not words:
            raise ValueError("lpmd: empty atom line")
        for k, c in enumerate(cols):
            if c == "SYM":
                sym.append(words[k])
            elif c in idx:
                data[i, idx[c]] = float(words[k])
    return dict(natoms=n, cell=cell, L=L, symbols=sym, pos=data[:, 0:3] * L, vel=data[:, 3:6], acc=data[:, 6:9],
                nlines=2 + n)


def read_lpmd(path) -> list[dict]:
    """Every frame of an lpmd or zlp 2.0 file: symbols, Cartesian positions (fractional x cell
    lengths, OrthogonalCell::Cartesian), velocities, accelerations (zero where not written)."""
    raw = Path(path).read_bytes()
    nl = raw.index(b"\n")
    first = raw[:nl].decode().split()
    if len(first) < 2 or first[0] != "LPMD":
        raise ValueError("Wrong header (not an LPMD/ZLP file)")
    if first[1] != "2.0":
        raise ValueError(f"Format version {first[1]} is not supported")
    ztype = len(first) > 2 and first[2] == "Z"
    nl2 = raw.index(b"\n", nl + 1)
    hdr = raw[nl + 1:nl2].decode().split()
    if not hdr or hdr[0] != "HDR":
        raise ValueError("doesn't seem to be in LPMD 2.0 format (wrong HDR)")
    body = raw[nl2 + 1:]
    frames = []
    if not ztype:
        lines = body.decode().split("\n")
        k = 0
        while k < len(lines) and lines[k].strip():
            fr = _frame_from_lines(lines[k:], hdr)
            k += fr.pop("nlines")
            frames.append(fr)
        return frames
    d = zlib.decompressobj()
    k = 0
    while k < len(body):
        width = body[k]
        size = int.from_bytes(body[k + 1:k + 5], "big")
        k += 1 + width
        text = d.decompress(body[k:k + size]).decode()
        k += size
        fr = _frame_from_lines(text.split("\n"), hdr)
        fr.pop("nlines")
        frames.append(fr)
    return frames


def read_xyz(path) -> list[dict]:
    """Every frame of an xyz file (XYZFormat::ReadCell): symbols, positions, and velocities /
    accelerations when the lines carry 7 / 10 words."""
    lines = Path(path).read_text().split("\n")
    frames, k = [], 0
    while k < len(lines) and lines[k].strip():
        n = int(lines[k].split()[0])
        sym, data = [], np.zeros((n, 9))
        width = 0
        for i in range(n):
            w = lines[k + 2 + i].split()
            if len(w) not in (4, 7, 10):
                raise ValueError(f"xyz: an unidentified line was found, line {k + 3 + i}")
            sym.append(w[0])
            data[i, :len(w) - 1] = [float(x) for x in w[1:]]
            width = len(w)
        frames.append(dict(natoms=n, symbols=sym, pos=data[:, 0:3], vel=data[:, 3:6], acc=data[:, 6:9],
                           level=(width - 4) // 3))
        k += 2 + n
    return frames


# ----------------------------------------------------------------------------------------------
# Simulation::Dump / Restore text (lossy: 6 significant digits)
# ----------------------------------------------------------------------------------------------


def _g(x: float) -> str:
    """iostream's default notation (precision 6) of a double: C's %g."""
    return "%g" % x


def write_dump(path, step: int, L, Z, pos, vel, acc, flags=None) -> None:
    """Simulation::Dump (liblpmd/simulation/simulationbuilder.cc:195-238) of an orthogonal cell.
    flags (GBMD_FLAG_*: 1 fixedvel, 2 fixedpos) become the atoms' tags with value "true"."""
    L = np.asarray(L, dtype=np.float64).reshape(3)
    Z = np.asarray(Z).reshape(-1)
    n = len(Z)
    pos, vel, acc = (np.asarray(a, dtype=np.float64).reshape(n, 3) for a in (pos, vel, acc))
    out = [f"{int(step)}\n"]
    for i in range(3):
        out.append("".join(_g(L[i] if q == i else 0.0) + " " for q in range(3)) + "\n")
    out.append(f"{n}\n")
    fmt = "%d " + "%g " * 9 + "\n"
    data = np.hstack([pos, vel, acc])
    out.extend(fmt % ((int(z),) + tuple(r)) for z, r in zip(Z, data))
    out.append("false \n" * n)
    for i in range(n):
        f = 0 if flags is None else int(flags[i])
        tags = sorted(t for bit, t in ((1, "fixedvel"), (2, "fixedpos")) if f & bit)  # tag keys in key order
        out.append(f"{len(tags)} " + "".join(f"{t} true " for t in tags) + "\n")
    Path(path).write_text("".join(out))


def read_dump(path) -> dict:
    """Simulation::Restore (liblpmd/simulation/simulationbuilder.cc:240-293): step, cell vectors,
    atoms (Z, positions, velocities, accelerations) and the fixedvel / fixedpos tags as flags."""
    w = Path(path).read_text().split()
    k = 0
    step = int(w[k]); k += 1
    cell = np.array([float(x) for x in w[k:k + 9]]).reshape(3, 3); k += 9
    n = int(w[k]); k += 1
    Z = np.zeros(n, dtype=np.int32)
    data = np.zeros((n, 9))
    for i in range(n):
        Z[i] = int(w[k])
        data[i] = [float(x) for x in w[k + 1:k + 10]]
        k += 10
    for i in range(n):
        have = w[k] == "true"
        k += 4 if have else 1
    flags = np.zeros(n, dtype=np.uint8)
    for i in range(n):
        m = int(w[k]); k += 1
        for _ in range(m):
            key, val = w[k], w[k + 1]
            k += 2
            if key == "fixedvel":
                flags[i] |= 1
            elif key == "fixedpos" and val == "true":
                flags[i] |= 2
    return dict(step=step, cell=cell, L=np.sqrt((cell ** 2).sum(axis=1)), Z=Z, pos=data[:, 0:3], vel=data[:, 3:6],
                acc=data[:, 6:9], flags=flags)
