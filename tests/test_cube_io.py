"""Cube / LOCPOT ingest and the constraint-file parsers (CPU).

The readers must return what the reference readers return (repeat.py:669-804,
1806-1891): checked by round trips through the cube writer, by a hand-made
LOCPOT whose values follow from its definition, and by the file-format rules."""
import gzip
import os

import numpy as np
import pytest

from conftest import load_golden
from pyrepeat_gb300 import cube as cio, synth


def test_cube_round_trip_exact(tmp_path):
    cube, _ = load_golden("tricmini")
    p = os.path.join(tmp_path, "t.cube")
    synth.write_cube(p, cube)
    r = cio.read_gauss_cube(p)
    assert r["n_atoms"] == cube.n_atoms
    assert np.array_equal(r["n_grid"], cube.n_grid)
    assert np.array_equal(r["axis_vector"], cube.axis_vector)
    assert np.array_equal(r["atom_index"], cube.atom_index)
    assert np.array_equal(r["atom_pos"], cube.atom_pos)
    assert np.array_equal(r["V_flat"], cube.V)           # %.16e round trips exactly
    nx, ny, nz = cube.n_grid
    # the reference's layout: V_pot[i + j*nx, k]
    i, j, k = 3, 5, 7
    assert r["V_pot"].shape == (nx * ny, nz)
    assert r["V_pot"][i + j * nx, k] == cube.V[i + j * nx + k * nx * ny]


def test_cube_value_count_checked(tmp_path):
    cube, _ = load_golden("water24")
    p = os.path.join(tmp_path, "w.cube")
    synth.write_cube(p, cube)
    with open(p, "a") as f:
        f.write("1.0\n")          # one value too many
    with pytest.raises(ValueError):
        cio.read_gauss_cube(p)


def test_parser_threads_agree():
    rng = np.random.default_rng(0)
    v = rng.normal(size=300001) * 10.0 ** rng.integers(-8, 8, size=300001)
    text = "\n".join(" ".join("%.17e" % x for x in v[s:s + 6]) for s in range(0, v.size, 6)).encode()
    a = cio.parse_values(text, v.size, threads=1)
    b = cio.parse_values(text, v.size, threads=7)
    assert np.array_equal(a, v) and np.array_equal(b, v)
    c = cio.parse_values(b"1.5D-03 2.0d+01", 2)        # Fortran exponents
    assert np.array_equal(c, [1.5e-3, 20.0])
    with pytest.raises(ValueError):
        cio.parse_values(b"1.0 abc 2.0", 3)


def _locpot_text(vals):
    lines = ["test system", "   1.0", "     2.0 0.0 0.0", "     0.0 3.0 0.0", "     0.0 0.0 4.0", "   H   O",
             "     1     1", "Direct", "  0.0 0.0 0.0", "  0.5 0.25 0.125", "", "    2    3    4"]
    lines += [" ".join("%.10e" % x for x in vals[s:s + 5]) for s in range(0, len(vals), 5)]
    lines += ["augmentation occupancies 1 2", "0.1 0.2"]
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("gz", [False, True])
def test_locpot(tmp_path, gz):
    vals = np.arange(24, dtype=np.float64) * 0.5
    name = os.path.join(tmp_path, "LOCPOT" + (".gz" if gz else ""))
    text = _locpot_text(vals)
    if gz:
        with gzip.open(name, "wt") as f:
            f.write(text)
        name = name[:-3]      # found through the .gz suffix, as the reference does
    else:
        with open(name, "w") as f:
            f.write(text)
    r = cio.read_data(name)
    s = 1.889725985
    assert np.array_equal(r["n_grid"], [2, 3, 4])
    assert list(r["atom_index"]) == [1, 8]
    assert np.allclose(r["atom_pos"][1], [0.5 * 2 * s, 0.25 * 3 * s, 0.125 * 4 * s], rtol=1e-15)
    assert np.allclose(r["axis_vector"], np.diag([2 * s / 2, 3 * s / 3, 4 * s / 4]), rtol=1e-15)
    assert np.allclose(r["V_flat"], -vals / 27.212, rtol=1e-15)     # x fastest, eV -> Hartree
    assert r["V_pot"][1 + 2 * 2, 3] == r["V_flat"][1 + 2 * 2 + 3 * 6]


def test_symmetry_and_resp_files(tmp_path):
    p = os.path.join(tmp_path, "s.txt")
    with open(p, "w") as f:
        f.write("# comment\n1-3, 7   # group one\n\n9,10,9\n12\n")
    assert cio.read_symmetry(p) == [[0, 1, 2, 6], [8, 9], [11]]
    assert cio.parse_atom_ranges("5-3") == []
    q = os.path.join(tmp_path, "r.txt")
    with open(q, "w") as f:
        f.write("C 0.1 0.0\nH 0.0 0.0\nbad line\n")
    assert cio.read_resp(q) == {"C": (0.1, 0.0), "H": (0.0, 0.0)}
