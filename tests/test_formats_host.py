"""Configuration writers and readers (lpmd2_gb300/formats.py) against files written by the
reference's own output plugins (tests/golden/formats/, made by make_format_golden.py from
plugins/lpmd.cc and plugins/xyz.cc): byte-identical output for every level, the TYPE extra
column, the compressed zlp variant (block size and compression level), xyz precision, exact
rounding ties, negative zeros; readers recover the frames to the printed precision."""
import zlib
from pathlib import Path

import numpy as np
import pytest

from lpmd2_gb300 import formats as F

GOLD = Path(__file__).resolve().parent / "golden" / "formats"
SYM = {18: "Ar", 29: "Cu"}
CASES = {
    "l0.lpmd": ("lpmd", dict(level=0)),
    "l1.lpmd": ("lpmd", dict(level=1)),
    "l2_type.lpmd": ("lpmd", dict(level=2, extra="TYPE")),
    "l1.zlp": ("lpmd", dict(level=1, blocksize=256)),
    "l2_c9.zlp": ("lpmd", dict(level=2, compression=9)),
    "l0.xyz": ("xyz", dict(level=0)),
    "l2.xyz": ("xyz", dict(level=2)),
    "l1_p4.xyz": ("xyz", dict(level=1, precout=4)),
}


@pytest.fixture(scope="module")
def frames():
    g = np.load(GOLD / "inputs.npz")
    return dict(L=g["L"], sym=[SYM[int(z)] for z in g["Z"]], pos=g["pos"], vel=g["vel"], acc=g["acc"])


def write(tmp_path, name, frames):
    module, kw = CASES[name]
    path = tmp_path / name
    w = F.open_writer(module, path, **kw)
    w.write_header()
    for f in range(len(frames["pos"])):
        w.write_frame(frames["sym"], frames["L"], frames["pos"][f], frames["vel"][f], frames["acc"][f])
    w.close()
    return path.read_bytes()


@pytest.mark.parametrize("name", list(CASES))
def test_writer_bytes_match_reference(name, frames, tmp_path):
    assert write(tmp_path, name, frames) == (GOLD / name).read_bytes()


@pytest.mark.parametrize("name", ["l1.zlp", "l2_c9.zlp"])
def test_zlp_records_decompress_to_the_lpmd_text(name, frames, tmp_path):
    raw = (GOLD / name).read_bytes()
    head, _, rest = raw.partition(b"\n")
    assert head == b"LPMD 2.0 Z"
    hdr, _, body = rest.partition(b"\n")
    d = zlib.decompressobj()
    texts, k = [], 0
    while k < len(body):
        assert body[k] == 8 and body[k + 5:k + 9] == bytes(4)
        size = int.from_bytes(body[k + 1:k + 5], "big")
        texts.append(d.decompress(body[k + 9:k + 9 + size]))
        k += 9 + size
    level = CASES[name][1]["level"]
    plain = F.LPMDWriter(tmp_path / "x.lpmd", level=level)
    want = [plain.frame_text(frames["sym"], frames["L"], frames["pos"][f], frames["vel"][f], frames["acc"][f]).encode()
            for f in range(3)]
    plain.close()
    assert texts == want


@pytest.mark.parametrize("name", ["l0.lpmd", "l1.lpmd", "l2_type.lpmd", "l1.zlp", "l2_c9.zlp"])
def test_read_lpmd(name, frames):
    got = F.read_lpmd(GOLD / name)
    level = CASES[name][1]["level"]
    assert len(got) == 3
    for f, fr in enumerate(got):
        assert fr["symbols"] == frames["sym"]
        np.testing.assert_allclose(fr["L"], frames["L"], rtol=0, atol=0)
        # fractional positions with 6 digits, times the cell length
        assert np.abs(fr["pos"] - frames["pos"][f]).max() <= 0.5e-6 * frames["L"].max() * (1 + 1e-9)
        if level >= 1:
            assert np.abs(fr["vel"] - frames["vel"][f]).max() <= 0.5e-6 * (1 + 1e-9)
        if level >= 2:
            assert np.abs(fr["acc"] - frames["acc"][f]).max() <= 0.5e-6 * (1 + 1e-9)


@pytest.mark.parametrize("name", ["l0.xyz", "l2.xyz", "l1_p4.xyz"])
def test_read_xyz(name, frames):
    got = F.read_xyz(GOLD / name)
    kw = CASES[name][1]
    half = 0.5 * 10.0 ** -kw.get("precout", 8) * (1 + 1e-9)
    assert len(got) == 3
    for f, fr in enumerate(got):
        assert fr["symbols"] == frames["sym"] and fr["level"] == kw["level"]
        assert np.abs(fr["pos"] - frames["pos"][f]).max() <= half * 16  # values up to 12: ulp of the parse
        if kw["level"] >= 1:
            assert np.abs(fr["vel"] - frames["vel"][f]).max() <= half * 1.0001


def test_writer_rejects_what_it_cannot_write(tmp_path):
    with pytest.raises(ValueError):
        F.LPMDWriter(tmp_path / "a.lpmd", level=3)
    with pytest.raises(ValueError):
        F.LPMDWriter(tmp_path / "a.lpmd", extra="RGB")
    with pytest.raises(ValueError):
        F.open_writer("dcd", tmp_path / "a.dcd")
    w = F.LPMDWriter(tmp_path / "a.lpmd", level=1)
    with pytest.raises(ValueError):
        w.write_frame("Ar", [1, 1, 1], np.zeros((2, 3)))
    w.close()
    # the file name decides the type, as LPMDFormat's constructor does
    assert F.LPMDWriter(tmp_path / "b.zlp").type == "zlp"
    assert F.LPMDWriter(tmp_path / "c.out", type="zlp").type == "zlp"
    assert F.LPMDWriter(tmp_path / "d.lpmd", type="zlp").type == "lpmd"


@pytest.mark.parametrize("module,name", [("lpmd", "one.lpmd"), ("lpmd", "one.zlp"), ("xyz", "one.xyz")])
def test_one_symbol_for_all_atoms_writes_what_a_symbol_list_writes(module, name, frames, tmp_path):
    def run(sym, path):
        w = F.open_writer(module, path, level=2)
        w.write_header()
        for f in range(3):
            w.write_frame(sym, frames["L"], frames["pos"][f], frames["vel"][f], frames["acc"][f])
        w.close()
        return path.read_bytes()

    n = len(frames["sym"])
    a = run("Kr", tmp_path / ("a_" + name))
    b = run(["Kr"] * n, tmp_path / ("b_" + name))
    assert a == b
    got = F.read_lpmd(tmp_path / ("a_" + name)) if module == "lpmd" else F.read_xyz(tmp_path / ("a_" + name))
    assert [fr["natoms"] for fr in got] == [n] * 3 and got[0]["symbols"] == ["Kr"] * n


def test_dump_bytes_match_reference_and_read_back(tmp_path):
    # Simulation::Dump of the reference (tests/golden/formats/frame0.dump): the first frame with
    # atoms 5 / 7 / 11 tagged fixedvel / fixedpos / both, and %g edge values in the accelerations
    g = np.load(GOLD / "inputs.npz")
    F.write_dump(tmp_path / "d.dump", 0, g["L"], g["Z"], g["pos"][0], g["vel"][0], g["acc"][0], g["flags"])
    assert (tmp_path / "d.dump").read_bytes() == (GOLD / "frame0.dump").read_bytes()
    d = F.read_dump(GOLD / "frame0.dump")
    assert d["step"] == 0 and list(d["Z"]) == list(g["Z"])
    np.testing.assert_array_equal(d["L"], g["L"])
    np.testing.assert_array_equal(d["flags"], g["flags"])
    for key in ("pos", "vel", "acc"):
        np.testing.assert_allclose(d[key], g[key][0], rtol=5e-6, atol=1e-300)
