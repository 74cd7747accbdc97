"""Gaussian cube and VASP LOCPOT readers (the data that feeds the fit).

Same results as the reference readers (``read_gauss_cube``, repeat.py:770-804;
``read_vasp_potential``, repeat.py:669-768; the file-name detection of
``ChargeCalculator._read_data``, repeat.py:1782-1804): the header is parsed
line by line in Python and the value block by the parallel C parser
``_cube_io.so`` (strtod over per-thread spans), which replaces the reference's
per-value Python loop.

Every reader returns the reference's dictionary (``n_atoms``, ``n_grid``,
``atom_index``, ``atom_pos``, ``axis_vector``, ``V_pot`` with shape
``(nx*ny, nz)``) plus ``V_flat`` (the values in the flat order
``i + j*nx + k*nx*ny`` the device kernels use, equal to ``V_pot.ravel('F')``)
and ``origin`` (read but, as in the reference, not applied to grid positions).
"""
from __future__ import annotations

import bz2
import ctypes
import glob
import gzip
import os
import re

import numpy as np

from .constants import ATOM_SYMBOLS

ANG_TO_BOHR = 1.889725985   # repeat.py:682
EV_TO_HARTREE = -1.0 / 27.212  # LOCPOT potential energy of an electron (eV) -> ESP (Hartree)

_IO = None


def _io_lib():
    global _IO
    if _IO is None:
        from .build import CUBE_IO_PATH, build_host_helpers
        if not os.path.exists(CUBE_IO_PATH):
            build_host_helpers()
        lib = ctypes.CDLL(CUBE_IO_PATH)
        lib.rp_parse_doubles.restype = ctypes.c_longlong
        lib.rp_parse_doubles.argtypes = [ctypes.c_char_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong,
                                         ctypes.c_int, ctypes.c_int]
        _IO = lib
    return _IO


def parse_values(block: bytes, count: int, threads: int | None = None, exact: bool = True) -> np.ndarray:
    """The first `count` whitespace-separated numbers of `block`; with exact=True the block
    must hold exactly `count` (ValueError otherwise)."""
    out = np.empty(count, dtype=np.float64)
    n = _io_lib().rp_parse_doubles(block, len(block), out.ctypes.data, count, threads or (os.cpu_count() or 1),
                                   0 if exact else 1)
    if n < 0:
        raise ValueError("value block holds a token that is not a number")
    if n < count or (exact and n != count):
        raise ValueError(f"value block holds {n} values, the header announces {count}")
    return out


def _open_text(path: str):
    """Plain, .gz or .bz2 file (the reference's compressed_open, repeat.py:655-667)."""
    names = glob.glob(path) + glob.glob(path + ".gz") + glob.glob(path + ".bz2")
    if not names:
        raise FileNotFoundError(f"File {path} not found")
    name = names[0]
    if name.endswith(".bz2"):
        return bz2.open(name, "rb")
    if name.endswith(".gz"):
        return gzip.open(name, "rb")
    return open(name, "rb")


def read_gauss_cube(path: str, threads: int | None = None) -> dict:
    """Gaussian cube: 2 comment lines, atom count + origin, three grid lines
    (count, step vector), one line per atom (Z, charge, x, y, z), then the values
    with x outermost and z innermost.  Units are taken as Bohr, as the reference does."""
    with open(path, "rb") as f:
        f.readline()
        f.readline()
        parts = f.readline().split()
        n_atoms = int(parts[0])
        origin = np.array([float(x) for x in parts[1:4]]) if len(parts) >= 4 else np.zeros(3)
        n_grid = np.zeros(3, dtype=int)
        axis_vector = np.zeros((3, 3))
        for i in range(3):
            parts = f.readline().split()
            n_grid[i] = int(parts[0])
            axis_vector[i] = [float(x) for x in parts[1:4]]
        atom_index = np.zeros(n_atoms, dtype=int)
        atom_pos = np.zeros((n_atoms, 3))
        for i in range(n_atoms):
            parts = f.readline().split()
            atom_index[i] = int(parts[0])
            atom_pos[i] = [float(x) for x in parts[2:5]]
        block = f.read()
    nx, ny, nz = (int(v) for v in n_grid)
    vals = parse_values(block, nx * ny * nz, threads)
    # file order (i, j, k) with k fastest  ->  V_pot[i + j*nx, k]
    V3 = vals.reshape(nx, ny, nz)
    V_flat = np.ascontiguousarray(V3.transpose(2, 1, 0)).reshape(-1)  # i fastest, then j, then k
    V_pot = V_flat.reshape((nx * ny, nz), order="F")
    return {"n_atoms": n_atoms, "n_grid": n_grid, "atom_index": atom_index, "atom_pos": atom_pos,
            "axis_vector": axis_vector, "V_pot": V_pot, "V_flat": V_flat, "origin": origin}


def read_vasp_potential(path: str, threads: int | None = None) -> dict:
    """VASP LOCPOT (optionally .gz/.bz2): lattice in Angstrom times a scale, element
    names and counts, fractional positions after the 'Direct' line, the grid counts,
    then the potential (eV) with x fastest.  Converted like the reference: Bohr,
    Hartree (times -1/27.212), fractional -> Cartesian, step vectors lattice/n."""
    with _open_text(path) as f:
        f.readline()                                   # system name
        scale = float(f.readline()) * ANG_TO_BOHR
        lattice = np.array([[scale * float(x) for x in f.readline().split()] for _ in range(3)])
        header = ""
        for _ in range(20):
            line = f.readline().decode()
            if "Direct" in line:
                break
            header += line
        # the reference joins the element and count lines without a separator
        # (repeat.py:690-698); VASP indents both, so the tokens stay apart
        tokens = "".join(header.splitlines()).split()
        types = [t for t in tokens if t.isalpha()]
        counts = [int(t) for t in tokens if t.isnumeric()]
        n_atoms = sum(counts)
        atoms = np.zeros((n_atoms, 3))
        for a in range(n_atoms):
            frac = np.array([float(x) for x in f.readline().split()[:3]])
            atoms[a] = frac @ lattice
        f.readline()                                   # blank line
        n_grid = np.array([int(x) for x in f.readline().split()[:3]], dtype=int)
        block = f.read()
    nx, ny, nz = (int(v) for v in n_grid)
    npts = nx * ny * nz
    # the potential may be followed by more data (augmentation occupancies, a second
    # spin block): stop at the first word and keep the first nx*ny*nz values
    m = re.search(rb"[A-DF-Za-df-z]", block)
    if m:
        block = block[:block.rfind(b"\n", 0, m.start()) + 1]
    vals = parse_values(block, npts, threads, exact=False)
    V_flat = EV_TO_HARTREE * vals                      # x fastest, then y, then z: the kernels' order
    atom_index = []
    for t, c in zip(types, counts):
        atom_index.extend([ATOM_SYMBOLS.index(t) if t in ATOM_SYMBOLS else 0] * c)
    axis_vector = np.array([lattice[i] / n_grid[i] for i in range(3)])
    return {"n_atoms": len(atom_index), "n_grid": n_grid, "atom_index": np.array(atom_index, dtype=int),
            "atom_pos": atoms, "axis_vector": axis_vector, "V_pot": V_flat.reshape((nx * ny, nz), order="F"),
            "V_flat": V_flat, "origin": np.zeros(3)}


def read_data(path: str, threads: int | None = None) -> dict:
    """Cube or LOCPOT by file name, as ChargeCalculator._read_data does (repeat.py:1782-1804):
    names containing 'locpot' are read as VASP first, anything else as a Gaussian cube."""
    base = os.path.basename(path).lower()
    if "locpot" in base:
        try:
            return read_vasp_potential(path, threads)
        except Exception as e:  # same fallback as the reference
            print(f"Warning: Failed to read as VASP file: {e}")
            print("Trying to read as cube file...")
    return read_gauss_cube(path, threads)


def parse_atom_ranges(text: str) -> list[int]:
    """'1-5,9,10,15-18' -> 0-based indices, duplicates dropped in order
    (ChargeCalculator._parse_atom_ranges, repeat.py:1806-1830)."""
    out, seen = [], set()
    for part in text.split(","):
        part = part.strip()
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-", 1)
            idx = range(int(a.strip()), int(b.strip()) + 1)
        else:
            idx = [int(part)]
        for i in idx:
            if i - 1 not in seen:
                seen.add(i - 1)
                out.append(i - 1)
    return out


def read_symmetry(path: str) -> list[list[int]]:
    """One group of equivalent atoms per line (1-based ranges, '#' comments); the first
    atom is the base (ChargeCalculator._read_symmetry, repeat.py:1832-1878)."""
    groups = []
    with open(path) as f:
        for line in f:
            if "#" in line:
                line = line.split("#")[0]
            line = line.strip()
            if not line:
                continue
            g = parse_atom_ranges(line)
            if g:
                groups.append(g)
    return groups


def read_resp(path: str) -> dict:
    """'element strength target' per line (ChargeCalculator._read_resp_params,
    repeat.py:1880-1891) -> {element: (strength, target)}."""
    out = {}
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3:
                out[parts[0]] = (float(parts[1]), float(parts[2]))
    return out
