"""Seeded synthetic cubes for the periodic REPEAT fit.

The reference ships no example cube, so every workload here is generated from
a seed: a cell, atoms placed by rejection sampling at a minimum periodic
separation and wrapped into the cell, seeded neutral charges, and an ESP equal
to the Ewald potential of those charges on every grid point plus Gaussian
noise.  The Ewald conventions are the ones of ``repeat.py`` (k-set by integer
index, ``kcoef = 4 pi / V exp(-k^2 / 4 alpha) / k^2`` with no factor 2,
``alpha = (pi / Rc)^2``, real-space images by ``nmax = floor(Rc/|a_i|) + 1``;
``repeat.py:1077-1143``), so a fit of the generated cube recovers the planted
charges up to the noise.

Grid values are stored in the reference's flat order
``flat = i + j*nx + k*nx*ny`` (``repeat.py:2086`` ravels the ``(nx*ny, nz)``
array in Fortran order).

Workloads (sizes are the ones the benchmark names):

* ``water``   cubic 18.0 Bohr, 72^3 grid, 3 waters, K = 754 (KMAX 7)
* ``mof``     cubic 25.8 Bohr, 128^3 grid, 424 atoms Zn:O:C:H = 32:104:192:96,
              KMAX 12 (K = 3779)
* ``tric``    triclinic 40 x 42 x 45 Bohr, 85/95/100 deg, 200 x 210 x 225 grid,
              2000 atoms C/H/N/O = 800/800/200/200, 150 symmetry groups,
              RESP 0.1 -> 0 on C, N, O
* ``batch``   one cube of the batched distribution (20-300 atoms, 12-30 Bohr,
              40^3-96^3 grid)
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field

import numpy as np

from .constants import ATOM_SYMBOLS, symbol_to_z

BOHR_TO_ANG = 0.529177


@dataclass
class Cube:
    """One ESP cube plus the fit settings that go with it."""
    atom_index: np.ndarray            # (N,) int, atomic numbers
    atom_pos: np.ndarray              # (N, 3) float64, Bohr
    n_grid: np.ndarray                # (3,) int
    axis_vector: np.ndarray           # (3, 3) float64, grid step vectors (rows)
    V: np.ndarray                     # (nx*ny*nz,) float64, flat order i + j*nx + k*nx*ny
    origin: np.ndarray = field(default_factory=lambda: np.zeros(3))
    charges_true: np.ndarray | None = None
    symm_groups: list | None = None   # list of lists of 0-based atom indices (first = base)
    resp: dict | None = None          # element symbol -> (strength, target)
    kmax: int = 7
    cutoff: float = 20.0
    vdw_factor: float = 1.0
    vdw_max: float = 1000.0
    total_charge: float = 0.0
    name: str = ""
    V_dev: object = None              # optional device copy of V (torch tensor)

    def host_V(self) -> np.ndarray:
        if self.V is None and self.V_dev is not None:
            self.V = self.V_dev.cpu().numpy()
        return self.V

    @property
    def n_atoms(self) -> int:
        return int(len(self.atom_index))

    @property
    def box_vectors(self) -> np.ndarray:
        return np.array([self.n_grid[i] * self.axis_vector[i] for i in range(3)], dtype=np.float64)

    @property
    def n_points(self) -> int:
        return int(np.prod(self.n_grid))

    def nbytes_device(self) -> int:
        """HBM bytes a fit of this cube keeps resident (grid values, kept
        indices, tables, normal equations)."""
        n = self.n_atoms
        return int(self.n_points * (8 + 4 + 1) + n * n * 8 * 3 + n * 64 * 1024)


# ----------------------------------------------------------------------------- cells

def lower_triangular_cell(a: float, b: float, c: float,
                          alpha_deg: float = 90.0, beta_deg: float = 90.0,
                          gamma_deg: float = 90.0) -> np.ndarray:
    """Cell rows a, b, c with a along x and b in the xy plane."""
    al, be, ga = (math.radians(x) for x in (alpha_deg, beta_deg, gamma_deg))
    va = np.array([a, 0.0, 0.0])
    vb = np.array([b * math.cos(ga), b * math.sin(ga), 0.0])
    cx = c * math.cos(be)
    cy = c * (math.cos(al) - math.cos(be) * math.cos(ga)) / math.sin(ga)
    cz = math.sqrt(max(c * c - cx * cx - cy * cy, 0.0))
    return np.array([va, vb, [cx, cy, cz]], dtype=np.float64)


def _min_image_dist2(frac_a: np.ndarray, frac_b: np.ndarray, cell: np.ndarray) -> np.ndarray:
    """Squared periodic distance between one fractional point and many, taking
    the smallest of the 27 neighbouring images (exact for the cells used here)."""
    d = frac_b - frac_a
    d -= np.round(d)
    best = None
    for s in _NEIGH27:
        cart = (d + s) @ cell
        r2 = np.einsum("ij,ij->i", cart, cart)
        best = r2 if best is None else np.minimum(best, r2)
    return best


_NEIGH27 = np.array([(i, j, k) for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)],
                    dtype=np.float64)


def place_atoms(rng: np.random.Generator, cell: np.ndarray, n: int, min_sep: float,
                max_tries: int = 2000000) -> np.ndarray:
    """Rejection-sample n points in the cell at periodic separation >= min_sep."""
    fracs = np.empty((n, 3))
    m = 0
    tries = 0
    min2 = min_sep * min_sep
    while m < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"could not place {n} atoms at separation {min_sep}")
        f = rng.random(3)
        if m and np.min(_min_image_dist2(f, fracs[:m], cell)) < min2:
            continue
        fracs[m] = f
        m += 1
    return fracs @ cell


# ----------------------------------------------------------------------------- Ewald potential on a grid

def ewald_alpha(cutoff: float) -> float:
    """alpha = (pi / Rc)^2 (``repeat.py:1083``)."""
    return (math.pi / cutoff) ** 2


def kspace_indices(kmax: int) -> np.ndarray:
    """Integer k indices in the reference order: kx in [0, KMAX], ky, kz in
    [-KMAX, KMAX], 0 < kx^2+ky^2+kz^2 < KMAX^2 (``repeat.py:1127-1141``)."""
    out = []
    ksqmax = kmax * kmax
    for kx in range(kmax + 1):
        for ky in range(-kmax, kmax + 1):
            for kz in range(-kmax, kmax + 1):
                s = kx * kx + ky * ky + kz * kz
                if s == 0 or s >= ksqmax:
                    continue
                out.append((kx, ky, kz))
    return np.asarray(out, dtype=np.int64).reshape(-1, 3)


def reciprocal_vectors(box: np.ndarray) -> tuple[np.ndarray, float]:
    a, b, c = box
    vol = float(np.dot(a, np.cross(b, c)))
    rec = np.array([2 * math.pi * np.cross(b, c) / vol,
                    2 * math.pi * np.cross(c, a) / vol,
                    2 * math.pi * np.cross(a, b) / vol])
    return rec, vol


def kspace(box: np.ndarray, cutoff: float, kmax: int):
    """k vectors and coefficients exactly as ``repeat.py:1127-1143`` forms them."""
    rec, vol = reciprocal_vectors(box)
    alpha = ewald_alpha(cutoff)
    beta = 1.0 / (4.0 * alpha)
    idx = kspace_indices(kmax)
    kv = np.array([kx * rec[0] + ky * rec[1] + kz * rec[2] for kx, ky, kz in idx]).reshape(-1, 3)
    ksq = np.einsum("ij,ij->i", kv, kv)
    kc = (4.0 * math.pi / vol) * np.exp(-beta * ksq) / ksq
    return idx, kv, kc


def realspace_shifts(box: np.ndarray, cutoff: float) -> np.ndarray:
    """All shifts ix*a + iy*b + iz*c, |i| <= floor(Rc/|a_i|)+1 (``repeat.py:1101-1104, 815-822``)."""
    nmax = [int(math.floor(cutoff / float(np.linalg.norm(box[i])))) + 1 for i in range(3)]
    out = []
    for ix in range(-nmax[0], nmax[0] + 1):
        for iy in range(-nmax[1], nmax[1] + 1):
            for iz in range(-nmax[2], nmax[2] + 1):
                out.append(ix * box[0] + iy * box[1] + iz * box[2])
    return np.asarray(out, dtype=np.float64)


def reciprocal_potential_grid(n_grid, box, atom_pos, q, cutoff, kmax) -> np.ndarray:
    """Reciprocal part of the Ewald potential of charges q on every grid point.

    On the cube lattice k.g = 2 pi (n1 i/nx + n2 j/ny + n3 l/nz) exactly, so
    sum_k w_k Re(conj(S_k) e^{i k.g}) with S_k = sum_a q_a e^{i k.a} is an
    inverse DFT of the weighted structure factors.
    """
    nx, ny, nz = (int(v) for v in n_grid)
    idx, kv, kc = kspace(box, cutoff, kmax)
    phase = atom_pos @ kv.T                      # (N, K)
    S = (q[:, None] * np.exp(1j * phase)).sum(axis=0)
    F = np.zeros((nx, ny, nz), dtype=np.complex128)
    np.add.at(F, (idx[:, 0] % nx, idx[:, 1] % ny, idx[:, 2] % nz), kc * np.conj(S))
    V = np.fft.ifftn(F).real * (nx * ny * nz)
    return np.ascontiguousarray(V.ravel(order="F"))


_SYNTH_LIB = None


def _synth_lib():
    global _SYNTH_LIB
    if _SYNTH_LIB is None:
        path = os.path.join(os.path.dirname(__file__), "_synth_host.so")
        if not os.path.exists(path):
            from .build import build_host_helpers
            build_host_helpers()
        lib = ctypes.CDLL(path)
        lib.synth_realspace_grid.restype = ctypes.c_int
        lib.synth_realspace_grid.argtypes = [
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,   # nx ny nz axis[9]
            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,              # N atoms[3N] q[N]
            ctypes.c_int, ctypes.c_void_p,                               # S shifts[3S]
            ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p]  # Rc sqrt_alpha threads out
        _SYNTH_LIB = lib
    return _SYNTH_LIB


def realspace_potential_grid(n_grid, axis, box, atom_pos, q, cutoff, threads=None) -> np.ndarray:
    """Real-space part sum_a q_a sum_s [r <= Rc] erfc(sqrt(alpha) r)/r on every
    grid point, skipping the r ~ 0 self image (``repeat.py:944-966``)."""
    nx, ny, nz = (int(v) for v in n_grid)
    shifts = np.ascontiguousarray(realspace_shifts(box, cutoff))
    out = np.zeros(nx * ny * nz, dtype=np.float64)
    ax = np.ascontiguousarray(axis, dtype=np.float64)
    pos = np.ascontiguousarray(atom_pos, dtype=np.float64)
    qq = np.ascontiguousarray(q, dtype=np.float64)
    threads = threads or (os.cpu_count() or 1)
    rc = _synth_lib().synth_realspace_grid(
        nx, ny, nz, ax.ctypes.data, len(qq), pos.ctypes.data, qq.ctypes.data,
        len(shifts), shifts.ctypes.data, float(cutoff), math.sqrt(ewald_alpha(cutoff)),
        int(threads), out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"synth_realspace_grid failed ({rc})")
    return out


def ewald_potential_grid(n_grid, axis, atom_pos, q, cutoff, kmax, threads=None) -> np.ndarray:
    box = np.array([n_grid[i] * axis[i] for i in range(3)])
    return (reciprocal_potential_grid(n_grid, box, atom_pos, q, cutoff, kmax)
            + realspace_potential_grid(n_grid, axis, box, atom_pos, q, cutoff, threads))


# ----------------------------------------------------------------------------- workloads

def _finish(cube: Cube, rng: np.random.Generator, noise: float, threads=None, ctx=None, esp: bool = True) -> Cube:
    """ESP = Ewald potential of the planted charges + N(0, noise).  With a
    pyrepeat_gb300.fit.Context the potential is evaluated on its GPU (rp_potential)
    and the cube keeps V only on the device (V_dev); otherwise on the host.  With
    esp=False the grid holds the noise alone: the same geometry and fit work (a timing
    stand-in where the host cannot afford the Ewald sum over every grid point)."""
    if not esp:
        cube.V = rng.normal(0.0, noise, size=cube.n_points)
        return cube
    if ctx is not None:
        import torch
        ew = ctx.ewald(cube.n_grid, cube.axis_vector, cube.cutoff, cube.kmax)
        try:
            V = ctx.potential(ew, cube.atom_pos, cube.charges_true, npts=cube.n_points)
        finally:
            ew.close()
        gen = torch.Generator(device=V.device)
        gen.manual_seed(int(rng.integers(0, 2**62)))
        V += noise * torch.randn(V.shape, dtype=V.dtype, device=V.device, generator=gen)
        cube.V_dev = V
        cube.V = None
        return cube
    V = ewald_potential_grid(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.charges_true,
                             cube.cutoff, cube.kmax, threads)
    cube.V = V + rng.normal(0.0, noise, size=V.shape)
    return cube


def make_water(seed: int = 1, n_grid: int = 72, noise: float = 1e-4, threads=None, ctx=None) -> Cube:
    """3 waters in a cubic 18.0 Bohr cell (O separated by >= 5 Bohr; H at 1.81
    Bohr and 104.5 deg, random orientation; q_O ~ N(-0.8, 0.05), H = -q_O/2)."""
    rng = np.random.default_rng(seed)
    L = 18.0
    cell = lower_triangular_cell(L, L, L)
    O = place_atoms(rng, cell, 3, 5.0)
    pos, Z, q = [], [], []
    half = math.radians(104.5) / 2
    for o in O:
        # random orthonormal frame
        u = rng.normal(size=3); u /= np.linalg.norm(u)
        v = rng.normal(size=3); v -= u * np.dot(u, v); v /= np.linalg.norm(v)
        h1 = o + 1.81 * (math.cos(half) * u + math.sin(half) * v)
        h2 = o + 1.81 * (math.cos(half) * u - math.sin(half) * v)
        qo = rng.normal(-0.8, 0.05)
        for p, z, qq in ((o, 8, qo), (h1, 1, -qo / 2), (h2, 1, -qo / 2)):
            pos.append(p); Z.append(z); q.append(qq)
    pos = np.array(pos)
    frac = pos @ np.linalg.inv(cell)
    pos = (frac - np.floor(frac)) @ cell
    axis = cell / n_grid
    cube = Cube(np.array(Z), pos, np.array([n_grid] * 3), axis, None,
                charges_true=np.array(q), kmax=7, name=f"water-{n_grid}")
    return _finish(cube, rng, noise, threads, ctx)


def _random_neutral(rng, n, sigma):
    q = rng.normal(0.0, sigma, size=n)
    return q - q.mean()


def make_mof(seed: int = 2, n_grid: int = 128, kmax: int = 12, noise: float = 1e-4,
             L: float = 25.8, counts=(32, 104, 192, 96), threads=None, ctx=None, esp: bool = True) -> Cube:
    """MOF-like cubic cell: Zn:O:C:H = 4:13:24:12 (x8 = 424 atoms) at >= 2.2 Bohr."""
    rng = np.random.default_rng(seed)
    cell = lower_triangular_cell(L, L, L)
    Z = np.array([30] * counts[0] + [8] * counts[1] + [6] * counts[2] + [1] * counts[3])
    Z = Z[rng.permutation(len(Z))]
    pos = place_atoms(rng, cell, len(Z), 2.2)
    q = _random_neutral(rng, len(Z), 0.5)
    axis = cell / n_grid
    cube = Cube(Z, pos, np.array([n_grid] * 3), axis, None, charges_true=q, kmax=kmax,
                name=f"mof-{len(Z)}-{n_grid}-k{kmax}")
    return _finish(cube, rng, noise, threads, ctx, esp)


def random_symmetry_groups(rng, n_atoms, n_groups, lo=2, hi=6):
    """Disjoint groups of lo..hi atoms (first = base), 0-based."""
    perm = rng.permutation(n_atoms)
    groups, pos = [], 0
    for _ in range(n_groups):
        g = int(rng.integers(lo, hi + 1))
        if pos + g > n_atoms:
            break
        groups.append(sorted(int(x) for x in perm[pos:pos + g]))
        pos += g
    return groups


def make_tric(seed: int = 3, n_grid=(200, 210, 225), n_atoms: int = 2000, noise: float = 1e-4,
              n_groups: int = 150, threads=None, lengths=(40.0, 42.0, 45.0),
              angles=(85.0, 95.0, 100.0), kmax: int = 7, ctx=None, esp: bool = True) -> Cube:
    """Triclinic cell 40 x 42 x 45 Bohr, 85/95/100 deg; C/H/N/O 40/40/10/10%;
    150 symmetry groups of 2-6 atoms; RESP 0.1 -> 0 on C, N, O."""
    rng = np.random.default_rng(seed)
    cell = lower_triangular_cell(*lengths, *angles)
    nC = int(round(0.4 * n_atoms)); nH = nC; nN = int(round(0.1 * n_atoms)); nO = n_atoms - nC - nH - nN
    Z = np.array([6] * nC + [1] * nH + [7] * nN + [8] * nO)
    Z = Z[rng.permutation(len(Z))]
    pos = place_atoms(rng, cell, len(Z), 2.0)
    q = _random_neutral(rng, len(Z), 0.4)
    groups = random_symmetry_groups(rng, len(Z), n_groups)
    # planted charges obey the symmetry constraint
    for g in groups:
        q[g] = q[g].mean()
    q -= q.mean()
    for g in groups:
        q[g] = q[g].mean()
    ng = np.array(n_grid)
    axis = cell / ng[:, None]
    cube = Cube(Z, pos, ng, axis, None, charges_true=q, symm_groups=groups,
                resp={"C": (0.1, 0.0), "N": (0.1, 0.0), "O": (0.1, 0.0)}, kmax=kmax,
                name=f"tric-{len(Z)}-{'x'.join(map(str, n_grid))}")
    return _finish(cube, rng, noise, threads, ctx, esp)


BATCH_ELEMENTS = (1, 6, 7, 8, 16, 30)


def make_batch_item(seed: int, large: bool = False, noise: float = 1e-4, threads=None,
                    with_symmetry: bool | None = None, ctx=None) -> Cube:
    """One cube of the batched distribution: 20-300 atoms (800-1500 and 160^3
    when large), cubic or orthorhombic 12-30 Bohr, spacing 0.2-0.3 Bohr
    clamped to 40..96 points per axis; q ~ N(0, 0.5) neutral; half carry
    symmetry groups, the other half RESP restraints."""
    rng = np.random.default_rng(seed)
    if large:
        n = int(rng.integers(800, 1501))
        # at most one atom per 90 Bohr^3 here too, so the vdW spheres leave ESP points
        L = max(float(rng.uniform(26.0, 30.0)), (n * 90.0) ** (1 / 3))
        lengths = np.array([L, L, L])
        ng = np.array([160, 160, 160])
    else:
        n = int(rng.integers(20, 301))
        if rng.random() < 0.5:
            L = rng.uniform(12.0, 30.0); lengths = np.array([L, L, L])
        else:
            lengths = rng.uniform(12.0, 30.0, size=3)
        # at most one atom per 90 Bohr^3, so the vdW spheres leave ESP points
        vol_min = n * 90.0
        if np.prod(lengths) < vol_min:
            lengths *= (vol_min / np.prod(lengths)) ** (1 / 3)
        h = rng.uniform(0.2, 0.3)
        ng = np.clip(np.round(lengths / h).astype(int), 40, 96)
    cell = lower_triangular_cell(*lengths)
    Z = rng.choice(np.array(BATCH_ELEMENTS), size=n, p=[0.4, 0.3, 0.1, 0.15, 0.03, 0.02])
    pos = place_atoms(rng, cell, n, 2.0)
    q = _random_neutral(rng, n, 0.5)
    if with_symmetry is None:
        with_symmetry = bool(seed % 2 == 0)
    groups, resp = None, None
    if with_symmetry:
        groups = random_symmetry_groups(rng, n, max(1, n // 20))
        for g in groups:
            q[g] = q[g].mean()
    else:
        resp = {"C": (0.1, 0.0), "N": (0.1, 0.0), "O": (0.1, 0.0), "S": (0.1, 0.0)}
    axis = cell / ng[:, None]
    cube = Cube(Z, pos, ng, axis, None, charges_true=q, symm_groups=groups, resp=resp, kmax=7,
                name=f"batch-{seed}")
    return _finish(cube, rng, noise, threads, ctx)


# ----------------------------------------------------------------------------- files

def write_cube(path: str, cube: Cube, fmt: str = "%.16e") -> None:
    """Gaussian cube text: values written x outer, z inner, 6 per line."""
    nx, ny, nz = (int(v) for v in cube.n_grid)
    with open(path, "w") as f:
        f.write(f"synthetic ESP cube {cube.name}\n")
        f.write("generated by pyrepeat_gb300.synth\n")
        o = cube.origin
        f.write(f"{cube.n_atoms:5d} {o[0]:.12f} {o[1]:.12f} {o[2]:.12f}\n")
        for i in range(3):
            a = cube.axis_vector[i]
            f.write(f"{int(cube.n_grid[i]):5d} {a[0]:.17g} {a[1]:.17g} {a[2]:.17g}\n")
        for z, p in zip(cube.atom_index, cube.atom_pos):
            f.write(f"{int(z):5d} {0.0:.6f} {p[0]:.17g} {p[1]:.17g} {p[2]:.17g}\n")
        V3 = cube.V.reshape((nx, ny, nz), order="F")
        flat = V3.reshape(-1)   # C order over (i, j, k): k fastest
        for s in range(0, flat.size, 6):
            f.write(" ".join(fmt % v for v in flat[s:s + 6]) + "\n")


def write_symmetry_file(path: str, groups) -> None:
    with open(path, "w") as f:
        f.write("# symmetry groups, 1-based, first atom is the base\n")
        for g in groups:
            f.write(",".join(str(i + 1) for i in g) + "\n")


def write_resp_file(path: str, resp: dict) -> None:
    with open(path, "w") as f:
        for el, (s, t) in resp.items():
            f.write(f"{el} {s} {t}\n")


__all__ = ["Cube", "make_water", "make_mof", "make_tric", "make_batch_item", "write_cube",
           "write_symmetry_file", "write_resp_file", "kspace", "kspace_indices",
           "realspace_shifts", "ewald_alpha", "lower_triangular_cell", "ATOM_SYMBOLS",
           "symbol_to_z", "BOHR_TO_ANG"]
