"""Generates tests/golden/formats/: configuration files written by the reference's own output
plugins (plugins/lpmd.cc LPMDFormat, plugins/xyz.cc XYZFormat), compiled into oracle/_ref/ by
``make -C oracle ref`` and driven by ref_driver.cpp::ref_write_frames.

inputs.npz holds the exact frames (two species, three frames, values that sit exactly on a
rounding tie of the printed digit count, negative zeros and tiny negatives); each other file is
the reference's output for one (module, arguments) case in CASES, and frame0.dump is the
reference's Simulation::Dump of the first frame with some atoms tagged fixedvel / fixedpos.

Usage:  python tests/golden/make_format_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "formats"

# file name -> (module, extra arguments); `file <name>` is added
CASES = {
    "l0.lpmd": ("lpmd", "level 0"),
    "l1.lpmd": ("lpmd", "level 1"),
    "l2_type.lpmd": ("lpmd", "level 2 extra TYPE"),
    "l1.zlp": ("lpmd", "level 1 blocksize 256"),
    "l2_c9.zlp": ("lpmd", "level 2 compression 9"),
    "l0.xyz": ("xyz", "level 0"),
    "l2.xyz": ("xyz", "level 2"),
    "l1_p4.xyz": ("xyz", "level 1 precout 4"),
}


def frames(seed: int = 3):
    rng = np.random.default_rng(seed)
    n, nf = 24, 3
    L = np.array([10.5, 11.25, 12.0])
    Z = np.where(np.arange(n) % 3 == 0, 29, 18).astype(np.int32)
    pos = rng.uniform(0, 1, (nf, n, 3)) * L
    vel = rng.normal(0, 0.01, (nf, n, 3))
    acc = rng.normal(0, 1e-3, (nf, n, 3))
    # exact ties at 6 digits (5/128 = 0.0390625, 15/128), at 8 digits (1/512), at 4 (1/32)
    vel[0, 0] = [0.0390625, -0.1171875, 1.0390625]
    acc[0, 1] = [-0.0390625, 0.001953125, 0.03125]
    pos[0, 2] = [0.001953125, 1.0390625, 0.03125]
    vel[1, 3] = [-0.0, -1e-9, 5e-7]
    pos[1, 4] = [0.0, -0.0, 3.0]
    return L, Z, pos, vel, acc


def main() -> None:
    if not oracle.reference_available():
        oracle.build()
    OUT.mkdir(exist_ok=True)
    L, Z, pos, vel, acc = frames()
    flags = np.zeros(len(Z), dtype=np.uint8)
    flags[5], flags[7], flags[11] = 1, 2, 3
    # %g edge cases: large / small magnitudes, exact ties of the 6th digit, negative zero
    acc = acc.copy()
    acc[0, 1] = [1.5e-12, -2.5e7, 123456.5]
    acc[0, 2] = [-0.0, 1.0000005, 9.9999995e-5]
    np.savez_compressed(OUT / "inputs.npz", L=L, Z=Z, pos=pos, vel=vel, acc=acc, flags=flags)
    oracle.write_reference_dump(OUT / "frame0.dump", L, Z, pos[0], vel[0], acc[0], flags)
    print(f"frame0.dump: {(OUT / 'frame0.dump').stat().st_size} bytes")
    for name, (module, args) in CASES.items():
        path = OUT / name
        oracle.write_reference_frames(path, module, f"file {path} {args}", L, Z, pos, vel, acc)
        print(f"{name}: {path.stat().st_size} bytes")


if __name__ == "__main__":
    main()
