"""The drop-in boundary's input contract on the CPU: ``inputs.txt`` read as the reference's
list-directed reads do (3D/QMS_3D.f90:120-165), its STOP message for an unsupported trajectory,
the inputs on which the reference is undefined rejected up front, and the material-ID lookup of
``geom.bin`` (F:229-254)."""
import numpy as np
import pytest

from alpineqms_gb300.inputs import InputError, material_index, parse_inputs_text, read_geom

VALID = """32,32,24
1e-3,1.0d-3,2e-3
1e-5
10
2
z,16
no
0,0,1e-2
-0.05,0,0
0,-0.05,0
0,0,0.1
1
0,-1e6,1
1
0,0,0
1
0,0,0
2
1
1,1,1
3.5e7,3.5e7,3.5e7
4
200,200,200
2e6,2e6,2e6
geom.bin
"""


def test_valid_file():
    inp = parse_inputs_text(VALID)
    assert (inp.xs, inp.ys, inp.zs) == (32, 32, 24)
    assert (inp.dx, inp.dy, inp.dz) == (1e-3, 1e-3, 2e-3)          # Fortran 'd' exponent
    assert (inp.dt, inp.nt, inp.tt) == (1e-5, 10, 2)
    assert (inp.slice_axis, inp.slice_index) == ("z", 16) and inp.slice_shape() == (32, 32)
    assert not inp.save_all_fields and inp.excitation is None
    assert inp.B == (0.0, 0.0, 1e-2) and inp.G_flat[8] == 0.1
    assert inp.traj[0].accel == -1e6 and inp.traj[0].n_accel == 1
    assert inp.props_table().shape == (2, 7) and inp.props_table()[1, 0] == 4
    assert inp.n_dims == 4 * 33 * 33 * 25 - 33 * 25 - 33 * 25 - 33 * 33
    assert inp.geom_name == "geom.bin"


def test_records_continue_over_lines_and_extra_values_are_skipped():
    text = VALID.replace("32,32,24\n", "32\n32, 24, 99\n", 1)    # a short record continues; the rest is skipped
    assert (parse_inputs_text(text).xs, parse_inputs_text(text).zs) == (32, 24)


def test_excitation_line():
    inp = parse_inputs_text(VALID + "excitation,sin,1000\n")
    assert inp.excitation == ("sin", 1000.0, 0.0)
    inp = parse_inputs_text(VALID + "excitation cos 50 0.5\n")
    assert inp.excitation == ("cos", 50.0, 0.5)
    with pytest.raises(InputError):
        parse_inputs_text(VALID + "excitation,square,50\n")


@pytest.mark.parametrize("old,new,msg", [
    ("1\n0,-1e6,1\n", "4\n0,-1e6,1\n", "ERROR: TYPE OF TRAJECTORY IN X DIRECTION IS NOT SUPPORTED"),
    ("1\n0,0,0\n1\n0,0,0\n2\n", "1\n0,0,0\n0\n0,0,0\n2\n",
     "ERROR: TYPE OF TRAJECTORY IN Z DIRECTION IS NOT SUPPORTED"),
    ("1\n0,-1e6,1\n", "3\n0\n", "at least one value"),
    ("z,16", "w,16", "slice axis"),
    ("z,16", "z,25", "slice index"),
    ("\n2\nz,16", "\n0\nz,16", "tt"),
    ("32,32,24\n", "3,32,24\n", "at least 4 cells"),
    ("32,32,24\n", "32,x,24\n", "bad integer"),
    ("1e-5\n", "-1e-5\n", "positive"),
])
def test_rejected_inputs(old, new, msg):
    assert old in VALID
    with pytest.raises(InputError, match=msg):
        parse_inputs_text(VALID.replace(old, new, 1))


def test_trajectory_types_beyond_one():
    """Type 2 (harmonic: amplitude, f, phase) and type 3 (a velocity table: its length, then a
    record of that many values over any number of lines) extend the reference's type 1."""
    text = VALID.replace("1\n0,-1e6,1\n1\n0,0,0\n", "2\n0.5,2000,0.25\n3\n4\n0.0,1.0\n2.0, 3.0\n", 1)
    inp = parse_inputs_text(text)
    tx, ty, tz = inp.traj
    assert (tx.kind, tx.amp, tx.freq, tx.phase) == (2, 0.5, 2000.0, 0.25)
    assert (ty.kind, ty.table) == (3, (0.0, 1.0, 2.0, 3.0))
    assert tz.kind == 1
    assert inp.props_table().shape == (2, 7) and inp.geom_name == "geom.bin"
    from alpineqms_gb300.workloads import inputs_text
    back = parse_inputs_text(inputs_text(inp))               # the writer's grammar reads back
    assert back.traj == inp.traj


def test_truncated_file_and_terminator():
    with pytest.raises(InputError, match="ended"):
        parse_inputs_text(VALID.split("geom.bin")[0].rsplit("\n", 4)[0])
    with pytest.raises(InputError, match="terminator"):
        parse_inputs_text(VALID.replace("1e-5\n", "/\n", 1))


def test_material_lookup():
    inp = parse_inputs_text(VALID)                                 # IDs 1 and 4
    slots = material_index(np.array([0.0, 1.0, 4.9, 2.0, 3.0, 4.0]), inp)
    assert slots.tolist() == [0, 1, 2, 0, 0, 2]                    # absent IDs are vacuum; IDs truncate
    with pytest.raises(InputError):
        material_index(np.array([5.0]), inp)                       # above the largest table ID
    with pytest.raises(InputError):
        material_index(np.array([-1.0]), inp)
    dup = parse_inputs_text(VALID.replace("\n4\n200", "\n1\n200", 1))
    assert material_index(np.array([1.0]), dup).tolist() == [2]    # the last row of a shared ID wins


def test_short_geometry_file(tmp_path):
    inp = parse_inputs_text(VALID)
    p = tmp_path / "geom.bin"
    np.zeros(10, "<f8").tofile(str(p))
    with pytest.raises(InputError, match="holds 10 values"):
        read_geom(str(p), inp)
    with pytest.raises(InputError, match="not found"):
        read_geom(str(tmp_path / "missing.bin"), inp)
