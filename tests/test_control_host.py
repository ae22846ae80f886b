"""Control-file runner, host side: the lpmd control language as the runner reads it."""
import numpy as np
import pytest

from lpmd2_gb300 import control as C
from lpmd2_gb300 import inputs as I

TEXT = """
# argon near the triple point
cell cubic 17.1191
input crystal3d type=fcc symbol=Ar nx=3 ny=3 nz=3
output xyz frames.xyz each=10
steps 2000
monitor step,total-energy,temperature start=0 end=-1 each=100
prepare temperature t=10.0
use lennardjones
    sigma 3.41
    epsilon 0.0103408
    cutoff 8.5
enduse
use beeman as integ
    dt 1.0
enduse
use velocityverlet as vv
    dt 1.0
enduse
use minimumimage
    cutoff 8.0
enduse
use gdr
    rcut 10.0
enduse
cellmanager minimumimage
potential lennardjones Ar Ar
integrator vv
property gdr each=100
"""


def test_parse_statements_and_blocks():
    ctl = C.parse(TEXT)
    assert np.array_equal(ctl.cell, [17.1191] * 3)
    assert ctl.input == {"module": "crystal3d", "type": "fcc", "symbol": "Ar", "nx": "3", "ny": "3", "nz": "3"}
    assert ctl.steps == 2000
    assert ctl.uses["lennardjones"] == ("lennardjones", "sigma 3.41 epsilon 0.0103408 cutoff 8.5")
    assert ctl.uses["vv"] == ("velocityverlet", "dt 1.0")
    assert ctl.uses["integ"] == ("beeman", "dt 1.0")  # declared; the integrator statement picks vv
    assert ctl.cellmanager == "minimumimage" and ctl.integrator == "vv"
    assert ctl.potentials == [("lennardjones", "Ar", "Ar")]
    assert ctl.monitors == [{"properties": "step,total-energy,temperature", "start": "0", "end": "-1", "each": "100"}]
    assert ctl.outputs == [{"module": "xyz", "file": "frames.xyz", "each": "10"}]
    assert ctl.prepares == [{"module": "temperature", "t": "10.0"}]
    assert ctl.skipped == ["use gdr", "property gdr each=100"]


def test_strict_rejects_modules_off_the_path():
    with pytest.raises(C.ControlError, match="outside the GPU timestep path"):
        C.parse(TEXT, strict=True)


@pytest.mark.parametrize("bad, msg", [
    ("frobnicate 3", "unknown statement"),
    ("use lennardjones\n sigma 1", "missing enduse"),
    ("cell crystal 10 10 10 90 90 60", "only orthogonal"),
    ("cell vector 1 0 0 0 1 0 0 0 1", "only cubic"),
])
def test_errors(bad, msg):
    with pytest.raises(C.ControlError, match=msg):
        C.parse(bad)


def test_crystal3d_sites():
    p, L = I.fcc_crystal3d(4, 3, 2, 5.26)
    assert np.array_equal(C.crystal3d("fcc", 4, 3, 2, L), p)
    L = np.array([10.0, 12.0, 14.0])
    assert len(C.crystal3d("bcc", 3, 3, 3, L)) == 54
    assert len(C.crystal3d("sc", 3, 3, 3, L)) == 27
    hcp = C.crystal3d("hcp", 2, 2, 2, L)
    assert len(hcp) == 16 and np.all(hcp >= 0) and np.all(hcp < L)
    with pytest.raises(C.ControlError):
        C.crystal3d("diamond", 1, 1, 1, L)


def test_stepper_activity():
    assert [s for s in range(0, 31) if C._active(s, 0, -1, 10)] == [0, 10, 20, 30]
    assert [s for s in range(0, 31) if C._active(s, 5, 25, 10)] == [5, 15, 25]


def test_missing_components_are_reported():
    ctl = C.parse("cell cubic 20\ninput crystal3d type=fcc symbol=Ar nx=2 ny=2 nz=2\nsteps 1\n")
    with pytest.raises(C.ControlError, match="MissingComponent: cellmanager"):
        C.run(ctl)


MODS = """
steps 60
use velocityverlet
    dt 2.0
enduse
integrator velocityverlet
use tempscaling as ramp
    from 100
    to 200
enduse
use temperature as fix
    t 77
enduse
use berendsen
    from 300
    to 300
    tau 8
    start 12
enduse
use gdr
enduse
apply ramp each=20
apply fix start=5 end=5
apply berendsen each=40
apply gdr each=10
"""


def test_modifier_schedule_follows_the_steppers():
    ctl = C.parse(MODS)
    assert set(ctl.modifiers) == {"ramp", "fix", "berendsen"}
    assert any(s.startswith("apply gdr") for s in ctl.skipped)
    sched = C.modifier_schedule(ctl, 2.0)
    # tempscaling: ValueAtStep with end -1 replaced by the step count (lpmd/application.cc:443-444)
    ramp = [(k, t) for k, mode, t, _ in sched if mode == 0 and t != 77.0]
    assert ramp == [(20, 100 + 20 / 60 * 100), (40, 100 + 40 / 60 * 100), (60, 200.0)]
    assert [(k, t) for k, mode, t, _ in sched if t == 77.0] == [(5, 77.0)]
    # berendsen: switched on at step 12 (no rescaling), every step until 12 + tau/dt = 16, off at
    # 17 with its own period restored; next active step 52 -> on, 53..56 rescale, off at 57
    ber = [(k, dtt) for k, mode, _, dtt in sched if mode == 1]
    assert [k for k, _ in ber] == [13, 14, 15, 16, 53, 54, 55, 56]
    assert all(d == 2.0 / 8.0 for _, d in ber)
    # same-step modifiers run in the order of their apply statements
    assert [k for k, *_ in sched] == sorted(k for k, *_ in sched)


def test_apply_of_an_unused_module_is_skipped_and_strict_rejects_it():
    with pytest.raises(C.ControlError):
        C.parse("steps 1\napply nothing each=2\n", strict=True)
    ctl = C.parse("steps 1\napply nothing each=2\n")
    assert ctl.applies == [] and ctl.skipped
