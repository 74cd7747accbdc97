"""Python driver of the C oracle — TEST INFRASTRUCTURE ONLY.

Used by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py``, to check results; the product never imports it.  It strings the C
restatement together in the order of ``repeat.py``'s ``ChargeCalculator``:
filter (repeat.py:1922-2113) -> pruned shifts (1708-1731) -> streamed normal
equations (2184-2276) -> symmetry/RESP/bordered solve (2278-2313); and QEq
charges (2539-2634) as NumPy: the pairwise Coulomb matrix and the reference's own
difference-form system.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "repeat_cpu_omp")
_lib = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_L = ctypes.c_int64


def build(force: bool = False) -> str:
    src = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "oracle.h")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(s) > os.path.getmtime(LIB) for s in src):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "all"], check=True)
    return LIB


def build_reference(reference_dir: str | None = None) -> str | None:
    """Compile repeat_cpu_omp.cpp from the reference tree into _ref/ (only where
    the reference sources exist).  The tree is `reference_dir`, else the
    PYREPEAT_REFERENCE environment variable, else the Makefile's REFERENCE."""
    reference_dir = reference_dir or os.environ.get("PYREPEAT_REFERENCE")
    if reference_dir is None:
        p = subprocess.run(["make", "-s", "-C", HERE, "--no-print-directory", "print-reference"],
                           stdout=subprocess.PIPE, text=True)
        reference_dir = p.stdout.strip()
    if not reference_dir or not os.path.exists(os.path.join(reference_dir, "repeat_cpu_omp.cpp")):
        return REF_BIN if os.path.exists(REF_BIN) else None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={reference_dir}"], check=True)
    return REF_BIN


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_kspace.restype = _I
        L.orc_kspace.argtypes = [_P, _D, _I, _P, _P, _I]
        L.orc_realspace_shifts.restype = _I
        L.orc_realspace_shifts.argtypes = [_P, _D, _P, _I]
        L.orc_prune_shifts.restype = _I
        L.orc_prune_shifts.argtypes = [_P, _I, _P, _L, _P, _I, _D, _P, ctypes.POINTER(_I)]
        for f in (L.orc_filter, L.orc_filter_sqrt):
            f.restype = _L
            f.argtypes = [_I, _I, _I, _P, _I, _P, _P, _D, _D, _P, _I]
        L.orc_compact.restype = None
        L.orc_compact.argtypes = [_I, _I, _I, _P, _P, _P, _P, _P, _P, _L]
        L.orc_phi.restype = None
        L.orc_phi.argtypes = [_L, _P, _I, _P, _I, _P, _P, _I, _P, _I, _D, _D, _P, _I]
        L.orc_normal_equations.restype = _I
        L.orc_normal_equations.argtypes = [_L, _P, _P, _I, _P, _I, _P, _P, _I, _P, _I, _D, _P, _P, _P,
                                           ctypes.POINTER(_D), _I]
        L.orc_solve.restype = _I
        L.orc_solve.argtypes = [_I, _P, _P, _I, _P, _P, _P, _P, _D, _P]
        L.orc_lu_solve.restype = _I
        L.orc_lu_solve.argtypes = [_I, _P, _P, _P]
        _lib = L
    return _lib


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def threads_default() -> int:
    return max(1, os.cpu_count() or 1)


def kspace(box, cutoff, kmax):
    box = _c(box)
    K = -lib().orc_kspace(box.ctypes.data, cutoff, kmax, None, None, 0)
    kv = np.zeros((K, 3)); kc = np.zeros(K)
    lib().orc_kspace(box.ctypes.data, cutoff, kmax, kv.ctypes.data, kc.ctypes.data, K)
    return kv, kc


def shifts(box, cutoff):
    box = _c(box)
    S = -lib().orc_realspace_shifts(box.ctypes.data, cutoff, None, 0)
    out = np.zeros((S, 3))
    lib().orc_realspace_shifts(box.ctypes.data, cutoff, out.ctypes.data, S)
    return out


def prune_shifts(sh, grid, atoms, cutoff):
    sh = _c(sh); grid = _c(grid); atoms = _c(atoms)
    out = np.zeros_like(sh)
    z = _I(-1)
    n = lib().orc_prune_shifts(sh.ctypes.data, len(sh), grid.ctypes.data, len(grid), atoms.ctypes.data,
                               len(atoms), cutoff, out.ctypes.data, ctypes.byref(z))
    return out[:n].copy(), z.value


def filter_mask(n_grid, axis, atoms, Z, vdw_factor=1.0, vdw_max=1000.0, sqrt_rule=False, threads=None):
    nx, ny, nz = (int(v) for v in n_grid)
    axis = _c(axis); atoms = _c(atoms); Z = _c(Z, np.int32)
    mask = np.zeros(nx * ny * nz, dtype=np.uint8)
    f = lib().orc_filter_sqrt if sqrt_rule else lib().orc_filter
    kept = f(nx, ny, nz, axis.ctypes.data, len(Z), atoms.ctypes.data, Z.ctypes.data, vdw_factor, vdw_max,
             mask.ctypes.data, threads or threads_default())
    return mask, int(kept)


def compact(n_grid, axis, mask, V):
    nx, ny, nz = (int(v) for v in n_grid)
    M = int(mask.sum())
    kept = np.zeros(M, dtype=np.int64); grid = np.zeros((M, 3)); Vc = np.zeros(M)
    axis = _c(axis); mask = _c(mask, np.uint8); V = _c(V)
    lib().orc_compact(nx, ny, nz, axis.ctypes.data, mask.ctypes.data, V.ctypes.data, kept.ctypes.data,
                      grid.ctypes.data, Vc.ctypes.data, M)
    return kept, grid, Vc


def phi(grid, atoms, kv, kc, sh, zero_idx, cutoff, threads=None):
    grid = _c(grid); atoms = _c(atoms); kv = _c(kv); kc = _c(kc); sh = _c(sh)
    out = np.zeros((len(grid), len(atoms)))
    lib().orc_phi(len(grid), grid.ctypes.data, len(atoms), atoms.ctypes.data, len(kc), kv.ctypes.data,
                  kc.ctypes.data, len(sh), sh.ctypes.data, zero_idx, cutoff, math.sqrt((math.pi / cutoff) ** 2),
                  out.ctypes.data, threads or threads_default())
    return out


def normal_equations(grid, Vc, atoms, kv, kc, sh, zero_idx, cutoff, threads=None):
    grid = _c(grid); Vc = _c(Vc); atoms = _c(atoms); kv = _c(kv); kc = _c(kc); sh = _c(sh)
    N = len(atoms)
    A = np.zeros((N, N)); b = np.zeros(N); sp = np.zeros(N); sv = _D(0)
    rc = lib().orc_normal_equations(len(grid), grid.ctypes.data, Vc.ctypes.data, N, atoms.ctypes.data,
                                    len(kc), kv.ctypes.data, kc.ctypes.data, len(sh), sh.ctypes.data,
                                    zero_idx, cutoff, A.ctypes.data, b.ctypes.data, sp.ctypes.data,
                                    ctypes.byref(sv), threads or threads_default())
    if rc != 0:
        raise MemoryError("oracle normal equations failed")
    return A, b, sp, sv.value


def groups_to_csr(groups):
    ptr = [0]; idx = []
    for g in groups or []:
        idx.extend(int(x) for x in g); ptr.append(len(idx))
    return np.asarray(ptr, dtype=np.int32), np.asarray(idx if idx else [0], dtype=np.int32)


def resp_arrays(Z, resp):
    from_sym = {}
    if resp:
        from_sym = resp
    import sys
    sys.path.insert(0, os.path.dirname(HERE))
    from pyrepeat_gb300.constants import z_to_symbol
    s = np.zeros(len(Z)); t = np.zeros(len(Z))
    for i, z in enumerate(Z):
        sym = z_to_symbol(int(z))
        if sym in from_sym:
            s[i], t[i] = from_sym[sym]
    return s, t


def solve(A, b, Z, groups=None, resp=None, qtot=0.0):
    A = np.array(A, dtype=np.float64, copy=True); b = np.array(b, dtype=np.float64, copy=True)
    N = len(b)
    ptr, idx = groups_to_csr(groups)
    rs, rt = resp_arrays(Z, resp)
    q = np.zeros(N)
    sing = lib().orc_solve(N, A.ctypes.data, b.ctypes.data, len(ptr) - 1, ptr.ctypes.data, idx.ctypes.data,
                           rs.ctypes.data, rt.ctypes.data, qtot, q.ctypes.data)
    return q, bool(sing)


def qeq_matrix(atoms, box, cutoff, kmax, j_self):
    """Coulomb matrix of compute_qeq_charges (repeat.py:2575-2595): J_ii = j_self; for the
    periodic fit (kmax > 0) J_ij = sum over the full shift list of erfc(sqrt(alpha) r)/r for
    r > 1e-10 (no cutoff) + sum_k kcoef cos(k.(r_i - r_j)) (_ewald_pairwise,
    repeat.py:2615-2634); for kmax 0, 1/r_ij for r > 1e-10.  Pairs i < j, mirrored."""
    from scipy.special import erfc
    atoms = _c(atoms)
    N = len(atoms)
    J = np.zeros((N, N))
    np.fill_diagonal(J, _c(j_self))
    if kmax > 0:
        kv, kc = kspace(box, cutoff, kmax)
        sh = shifts(box, cutoff)
        sa = math.sqrt((math.pi / cutoff) ** 2)
    for i in range(N - 1):
        d = atoms[i] - atoms[i + 1:]
        if kmax > 0:
            r = np.linalg.norm(d[:, None, :] + sh[None, :, :], axis=2)
            ok = r > 1e-10
            real = np.where(ok, erfc(sa * r) / np.where(ok, r, 1.0), 0.0).sum(axis=1)
            v = real + (kc[None, :] * np.cos(d @ kv.T)).sum(axis=1)
        else:
            r = np.linalg.norm(d, axis=1)
            v = np.where(r > 1e-10, 1.0 / np.where(r > 1e-10, r, 1.0), 0.0)
        J[i, i + 1:] = v
        J[i + 1:, i] = v
    return J


def qeq_charges(J, chi, qtot=0.0):
    """repeat.py:2597-2613: sum q = qtot and rows J[i-1] - J[i] against chi[i] - chi[i-1],
    solved by LU (least squares where LU reports a singular matrix)."""
    N = len(chi)
    A = np.zeros((N, N))
    b = np.zeros(N)
    A[0, :] = 1.0
    b[0] = qtot
    for i in range(1, N):
        A[i, :] = J[i - 1, :] - J[i, :]
        b[i] = chi[i] - chi[i - 1]
    try:
        return np.linalg.solve(A, b)
    except np.linalg.LinAlgError:
        return np.linalg.lstsq(A, b, rcond=None)[0]


class OracleFit:
    """Everything the reference computes for one cube, in FP64."""

    def __init__(self, cube, threads=None, sample=None, seed=0):
        """``sample``: fit a seeded random subset of that many kept points
        (a bounded CPU baseline); None fits all kept points."""
        self.threads = threads or threads_default()
        c = cube
        self.mask, self.M_total = filter_mask(c.n_grid, c.axis_vector, c.atom_pos, c.atom_index,
                                              c.vdw_factor, c.vdw_max, threads=self.threads)
        self.kept, self.grid, self.Vc = compact(c.n_grid, c.axis_vector, self.mask, c.V)
        if sample is not None and sample < len(self.kept):
            rng = np.random.default_rng(seed)
            sel = np.sort(rng.choice(len(self.kept), size=sample, replace=False))
            self.grid = self.grid[sel]; self.Vc = self.Vc[sel] - self.Vc[sel].mean()
        box = c.box_vectors
        if c.kmax == 0:
            # the non-periodic basis of --fit-type 0 (repeat.py:991-994): 1/|g - r_a| for the
            # atom itself (0 at r <= 1e-10), i.e. the real-space term with alpha 0, one zero
            # shift and no cutoff, and no k-vectors
            self.kv, self.kc = np.zeros((0, 3)), np.zeros(0)
            self.shifts, self.zero_idx = np.zeros((1, 3)), 0
            self.cutoff = math.inf
        else:
            self.kv, self.kc = kspace(box, c.cutoff, c.kmax)
            full = shifts(box, c.cutoff)
            self.shifts, self.zero_idx = prune_shifts(full, self.grid, c.atom_pos, c.cutoff)
            self.cutoff = c.cutoff
        self.cube = c

    def normal_equations(self):
        c = self.cube
        return normal_equations(self.grid, self.Vc, c.atom_pos, self.kv, self.kc, self.shifts,
                                self.zero_idx, self.cutoff, self.threads)

    def fit(self):
        c = self.cube
        A, b, sp, sv = self.normal_equations()
        self.A, self.b, self.sum_phi, self.sum_V = A, b, sp, sv
        q, sing = solve(A, b, c.atom_index, c.symm_groups, c.resp, c.total_charge)
        self.singular = sing
        return q

    def phi(self):
        c = self.cube
        return phi(self.grid, c.atom_pos, self.kv, self.kc, self.shifts, self.zero_idx, self.cutoff, self.threads)


def run_reference_binary(cube_path: str, timeout: int = 3600) -> np.ndarray | None:
    """Charges printed by the compiled repeat_cpu_omp (plain fit: vdw 1.0/1000,
    Rc 20, qtot 0, KMAX 7; repeat_cpu_omp.cpp:514-519)."""
    if not os.path.exists(REF_BIN):
        return None
    p = subprocess.run([REF_BIN, cube_path], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=timeout)
    q = []
    for line in p.stdout.splitlines():
        if line.startswith("Charge ") and " = " in line:
            q.append(float(line.split("=")[-1]))
    return np.array(q)
