"""Device-side fit pipeline: filter -> Ewald setup -> normal equations -> solve.

``Context`` owns one ``rp_ctx`` (scratch HBM, cuBLAS handle) on one device.
``fit_cube`` runs one whole fit with the cube's grid values already on the
device (or copies them there); ``fit_host`` is the end-to-end path from host
memory through the C ABI's ``rp_fit``.
"""
from __future__ import annotations

import ctypes
import itertools
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .constants import z_to_symbol


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pyrepeat_gb300 needs a CUDA device (no CPU fallback)")
    return torch


@dataclass
class FitResult:
    charges: np.ndarray
    n_kept: int
    precision: str
    A: object = None          # torch tensor (N, N) on the device, mean-removed normal matrix
    b: object = None          # torch tensor (N,)
    info: dict = field(default_factory=dict)


def constraint_arrays(Z, symm_groups=None, resp=None):
    """CSR symmetry groups (0-based, base first) and per-atom RESP arrays."""
    N = len(Z)
    groups = [g for g in (symm_groups or []) if len(g) >= 1]
    ptr = np.zeros(len(groups) + 1, dtype=np.int32)
    if groups:
        np.cumsum(np.fromiter(map(len, groups), dtype=np.int32, count=len(groups)), out=ptr[1:])
        idx = np.fromiter(itertools.chain.from_iterable(groups), dtype=np.int32, count=int(ptr[-1]))
    else:
        idx = np.zeros(1, dtype=np.int32)
    rs = rt = None
    if resp:
        # per element (Z) values, then gathered per atom
        zs = np.asarray(Z, dtype=np.int64)
        uz = np.unique(zs)
        ts = np.zeros(int(uz.max()) + 1 if len(uz) else 1)
        tt = np.zeros_like(ts)
        for z in uz:
            st = resp.get(z_to_symbol(int(z)))
            if st:
                ts[z], tt[z] = float(st[0]), float(st[1])
        rs, rt = ts[zs], tt[zs]
    return len(groups), ptr, idx, rs, rt


def _ptr(a):
    return None if a is None else a.ctypes.data


class Context:
    """One rp_ctx on one CUDA device."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.torch = _torch()
        self.lib = _lib.load()
        self.device = device
        self.dev = self.torch.device(f"cuda:{device}")
        self.torch.cuda.set_device(self.device)
        p = ctypes.c_void_p()
        rc = self.lib.rp_ctx_create(device, hbm_budget, ctypes.byref(p))
        if rc != 0:
            raise _lib.RepeatError(rc, "rp_ctx_create failed")
        self.ptr = p

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.rp_ctx_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _stream(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def check(self, rc, what=""):
        _lib.check(self.ptr, rc, what)

    # ------------------------------------------------------------------ stages
    def filter(self, n_grid, axis, atoms, Z, V_dev, vdw_factor=1.0, vdw_max=1000.0, want_mask=False):
        t = self.torch
        n = int(np.prod(n_grid))
        kept = t.empty(n, dtype=t.int32, device=self.dev)
        Vc = t.empty(n, dtype=t.float64, device=self.dev)
        mask = t.empty(n, dtype=t.uint8, device=self.dev) if want_mask else None
        M = ctypes.c_int64(0)
        g = _lib.make_grid(n_grid, axis)
        atoms = np.ascontiguousarray(atoms, dtype=np.float64)
        Zi = np.ascontiguousarray(Z, dtype=np.int32)
        rc = self.lib.rp_filter(self.ptr, ctypes.byref(g), atoms.ctypes.data, Zi.ctypes.data, len(Zi),
                                V_dev.data_ptr(), float(vdw_factor), float(vdw_max), kept.data_ptr(),
                                Vc.data_ptr(), n, ctypes.byref(M), mask.data_ptr() if want_mask else None,
                                self._stream())
        self.check(rc, "rp_filter")
        m = int(M.value)
        return kept[:m], Vc[:m], m, mask

    def ewald(self, n_grid, axis, cutoff=20.0, kmax=7):
        return Ewald(self, n_grid, axis, cutoff, kmax)

    def gram(self, ew, atoms, kept, Vc, precision=_lib.PREC_MIXED, want_sum_phi=False):
        t = self.torch
        atoms = np.ascontiguousarray(atoms, dtype=np.float64)
        N = len(atoms)
        A = t.empty((N, N), dtype=t.float64, device=self.dev)
        b = t.empty(N, dtype=t.float64, device=self.dev)
        sp = t.empty(N, dtype=t.float64, device=self.dev) if want_sum_phi else None
        rc = self.lib.rp_gram(self.ptr, ew.ptr, atoms.ctypes.data, N, kept.data_ptr(), Vc.data_ptr(),
                              int(kept.numel()), int(precision), A.data_ptr(), b.data_ptr(),
                              sp.data_ptr() if sp is not None else None, self._stream())
        self.check(rc, "rp_gram")
        return A, b, sp

    def solve(self, A, b, Z, symm_groups=None, resp=None, qtot=0.0):
        t = self.torch
        N = int(b.numel())
        ng, ptr, idx, rs, rt = constraint_arrays(Z, symm_groups, resp)
        q = t.empty(N, dtype=t.float64, device=self.dev)
        info = np.zeros(_lib.SOLVE_INFO_WORDS)
        rc = self.lib.rp_solve(self.ptr, A.data_ptr(), b.data_ptr(), N, ng, ptr.ctypes.data, idx.ctypes.data,
                               _ptr(rs), _ptr(rt), float(qtot), q.data_ptr(), info.ctypes.data, self._stream())
        self.check(rc, "rp_solve")
        return q, _lib.solve_info(info)

    def set_kappa_limit(self, kappa_max: float):
        """Mixed-precision fits whose kappa / (n+1) exceeds this are refitted in FP64 (0 = never;
        default 2e5)."""
        self.check(self.lib.rp_set_kappa_limit(self.ptr, float(kappa_max)), "rp_set_kappa_limit")

    def set_timing(self, on: bool = True):
        self.check(self.lib.rp_set_timing(self.ptr, 1 if on else 0), "rp_set_timing")

    def stage_times(self) -> dict:
        """{stage: (total ms, launches)} since the last call (CUDA events on each stage's stream)."""
        names = ctypes.create_string_buffer(8192)
        ms = np.zeros(2 * 64)
        cnt = ctypes.c_int(64)
        self.check(self.lib.rp_stage_times(self.ptr, names, 8192, ms.ctypes.data, ctypes.byref(cnt)),
                   "rp_stage_times")
        labels = names.value.decode().split("\n")[:cnt.value]
        return {lab: (float(ms[2 * i]), int(ms[2 * i + 1])) for i, lab in enumerate(labels)}

    def potential(self, ew, atoms, q, idx=None, npts=None):
        """Ewald potential of charges q at grid points (all points when idx is None)."""
        t = self.torch
        atoms = np.ascontiguousarray(atoms, dtype=np.float64)
        q = np.ascontiguousarray(q, dtype=np.float64)
        if idx is None:
            if npts is None:
                raise ValueError("npts needed when idx is None")
        else:
            npts = int(idx.numel())
        out = t.zeros(int(npts), dtype=t.float64, device=self.dev)
        rc = self.lib.rp_potential(self.ptr, ew.ptr, atoms.ctypes.data, q.ctypes.data, len(q),
                                   idx.data_ptr() if idx is not None else None, int(npts), out.data_ptr(),
                                   self._stream())
        self.check(rc, "rp_potential")
        return out

    def qeq(self, n_grid, axis, atoms, chi, j_self, qtot=0.0, cutoff=20.0, kmax=7, want_J=False):
        """QEq charges through rp_qeq: the Coulomb matrix of the atoms under the Ewald
        object of (grid, cutoff, kmax; kmax 0 = the 1/r matrix) and the equalisation
        solve.  Returns (charges, J or None, info)."""
        atoms = np.ascontiguousarray(atoms, dtype=np.float64)
        N = len(atoms)
        chi = np.ascontiguousarray(chi, dtype=np.float64)
        j_self = np.ascontiguousarray(j_self, dtype=np.float64)
        if chi.shape != (N,) or j_self.shape != (N,):
            raise ValueError("chi and j_self need one value per atom")
        q = np.zeros(N)
        J = np.zeros((N, N)) if want_J else None
        info = np.zeros(_lib.SOLVE_INFO_WORDS)
        ew = self.ewald(n_grid, axis, cutoff, kmax)
        try:
            rc = self.lib.rp_qeq(self.ptr, ew.ptr, atoms.ctypes.data, N, chi.ctypes.data, j_self.ctypes.data,
                                 float(qtot), q.ctypes.data, J.ctypes.data if J is not None else None,
                                 info.ctypes.data, self._stream())
            self.check(rc, "rp_qeq")
        finally:
            ew.close()
        return q, J, _lib.solve_info(info)

    # ------------------------------------------------------------------ whole fits
    def fit_cube(self, cube, precision=_lib.PREC_MIXED, V_dev=None, keep_normal=False):
        """Fit one synth.Cube-like object (atom_index, atom_pos, n_grid, axis_vector, V,
        symm_groups, resp, kmax, cutoff, vdw_factor, vdw_max, total_charge)."""
        t = self.torch
        if V_dev is None:
            V_dev = getattr(cube, "V_dev", None)
        if V_dev is None:
            V_dev = t.from_numpy(np.ascontiguousarray(cube.V, dtype=np.float64)).to(self.dev)
        kept, Vc, M, _ = self.filter(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index, V_dev,
                                     cube.vdw_factor, cube.vdw_max)
        if M == 0:
            raise _lib.RepeatError(-1, "no grid point survives the vdW filter")
        ew = self.ewald(cube.n_grid, cube.axis_vector, cube.cutoff, cube.kmax)
        try:
            A, b, _ = self.gram(ew, cube.atom_pos, kept, Vc, precision)
        finally:
            ew.close()
        q, info = self.solve(A, b, cube.atom_index, cube.symm_groups, cube.resp, cube.total_charge)
        res = FitResult(q.cpu().numpy(), M, "fp64" if precision == _lib.PREC_FP64 else "mixed", info=info)
        if keep_normal:
            res.A, res.b = A, b
        return res

    def _desc(self, cube, precision, keep, d=None):
        """rp_fit_desc for a cube (filled into `d` when given); arrays it points to are
        appended to `keep`."""
        if d is None:
            d = _lib.RpFitDesc()
        d.grid = _lib.make_grid(cube.n_grid, cube.axis_vector)
        atoms = np.ascontiguousarray(cube.atom_pos, dtype=np.float64)
        Z = np.ascontiguousarray(cube.atom_index, dtype=np.int32)
        ng, ptr, idx, rs, rt = constraint_arrays(Z, cube.symm_groups, cube.resp)
        V = None
        if cube.V is not None and not hasattr(cube.V, "data_ptr"):
            V = np.ascontiguousarray(cube.V, dtype=np.float64)
        keep.extend([atoms, Z, ptr, idx, rs, rt, V])
        d.V = V.ctypes.data if V is not None else None
        d.atoms, d.Z, d.N = atoms.ctypes.data, Z.ctypes.data, len(Z)
        d.vdw_factor, d.vdw_max, d.cutoff, d.qtot = cube.vdw_factor, cube.vdw_max, cube.cutoff, cube.total_charge
        d.kmax, d.n_groups = cube.kmax, ng
        d.group_ptr, d.group_idx, d.resp_s, d.resp_t = ptr.ctypes.data, idx.ctypes.data, _ptr(rs), _ptr(rt)
        d.precision = int(precision)
        return d

    def fit_host(self, cube, precision=_lib.PREC_MIXED):
        """End to end through rp_fit: host V and atoms in, host charges out."""
        keep = []
        d = self._desc(cube, precision, keep)
        q = np.zeros(cube.n_atoms)
        M = ctypes.c_int64(0)
        rc = self.lib.rp_fit(self.ptr, ctypes.byref(d), q.ctypes.data, ctypes.byref(M), self._stream())
        self.check(rc, "rp_fit")
        return FitResult(q, int(M.value), "fp64" if precision == _lib.PREC_FP64 else "mixed")

    def fit_batch(self, cubes, precision=_lib.PREC_MIXED, V_dev=None, out=None):
        """Fit many cubes in one rp_fit_batch call.  V_dev: optional list of device
        tensors holding each cube's grid values (else cube.V is read from the host).
        Returns a list of charge arrays (views into one buffer) and the kept counts."""
        n = len(cubes)
        keep = []
        arr = (_lib.RpFitDesc * n)()
        for i, c in enumerate(cubes):
            self._desc(c, precision[i] if isinstance(precision, (list, tuple)) else precision, keep, arr[i])
        vptr = None
        if V_dev is not None:
            vptr = (ctypes.c_void_p * n)(*[v.data_ptr() if v is not None else None for v in V_dev])
        total = sum(c.n_atoms for c in cubes)
        q = out if out is not None else np.zeros(total)
        M = np.zeros(n, dtype=np.int64)
        info = np.zeros(_lib.FIT_INFO_WORDS * n)
        rc = self.lib.rp_fit_batch(self.ptr, n, ctypes.cast(arr, ctypes.c_void_p), vptr, q.ctypes.data,
                                   M.ctypes.data, info.ctypes.data, self._stream())
        self.check(rc, "rp_fit_batch")
        res, o = [], 0
        for c in cubes:
            res.append(q[o:o + c.n_atoms])
            o += c.n_atoms
        return res, M, info.reshape(n, _lib.FIT_INFO_WORDS)

    def autotune(self, cubes, cache_path: str | None = None, V_dev=None) -> dict:
        """Tile shapes of the mixed path timed per (atoms, kept points, KMAX) bucket of the
        cubes (rp_autotune); with cache_path the table is written there.  Returns
        {bucket key: (phi_atoms, gram_split, best_ms, default_ms, N, M)} for the buckets
        this call measured (read back from the cache when one is given)."""
        n = len(cubes)
        keep = []
        arr = (_lib.RpFitDesc * n)()
        for i, c in enumerate(cubes):
            arr[i] = self._desc(c, _lib.PREC_MIXED, keep)
        vptr = None
        if V_dev is None and any(getattr(c, "V_dev", None) is not None for c in cubes):
            V_dev = [getattr(c, "V_dev", None) for c in cubes]
        if V_dev is not None:
            vptr = (ctypes.c_void_p * n)(*[v.data_ptr() if v is not None else None for v in V_dev])
        path = cache_path.encode() if cache_path else None
        self.check(self.lib.rp_autotune(self.ptr, n, ctypes.cast(arr, ctypes.c_void_p), vptr, path), "rp_autotune")
        table = {}
        if cache_path:
            with open(cache_path) as f:
                for line in f:
                    if line.startswith("#"):
                        continue
                    v = line.split()
                    if len(v) >= 7:
                        table[int(v[0])] = (int(v[1]), int(v[2]), float(v[3]), float(v[4]), int(v[5]), int(v[6]))
        return table

    def load_tiles(self, cache_path: str):
        """Tile shapes from an rp_autotune cache file."""
        self.check(self.lib.rp_load_tiles(self.ptr, cache_path.encode()), "rp_load_tiles")

    def batch_submit(self, cubes, precision=_lib.PREC_MIXED, V_dev=None) -> "PendingBatch":
        """Queue a batch on the context's worker thread (rp_batch_submit) and return at once.
        The returned handle keeps every array the worker reads alive until it is done."""
        n = len(cubes)
        keep = []
        arr = (_lib.RpFitDesc * n)()
        for i, c in enumerate(cubes):
            arr[i] = self._desc(c, precision[i] if isinstance(precision, (list, tuple)) else precision, keep)
        vptr = None
        if V_dev is not None:
            vptr = (ctypes.c_void_p * n)(*[v.data_ptr() if v is not None else None for v in V_dev])
        pb = PendingBatch(self, cubes, keep + [arr, vptr, V_dev])
        t = ctypes.c_longlong()
        rc = self.lib.rp_batch_submit(self.ptr, n, ctypes.cast(arr, ctypes.c_void_p), vptr, pb.q.ctypes.data,
                                      pb.M.ctypes.data, pb.info.ctypes.data, ctypes.byref(t))
        self.check(rc, "rp_batch_submit")
        pb.ticket = t.value
        return pb


class PendingBatch:
    """A batch queued with rp_batch_submit: poll() without blocking, result() waits."""

    def __init__(self, ctx: Context, cubes, keep):
        self.ctx, self.cubes, self._keep = ctx, cubes, keep
        self.q = np.zeros(sum(c.n_atoms for c in cubes))
        self.M = np.zeros(len(cubes), dtype=np.int64)
        self.info = np.zeros(_lib.FIT_INFO_WORDS * len(cubes))
        self.ticket = None
        self.status = None

    def poll(self) -> bool:
        if self.status is None:
            done, st = ctypes.c_int(), ctypes.c_int()
            self.ctx.check(self.ctx.lib.rp_batch_poll(self.ctx.ptr, self.ticket, ctypes.byref(done),
                                                      ctypes.byref(st)), "rp_batch_poll")
            if done.value:
                self.status = st.value
        return self.status is not None

    def result(self):
        """(charges per cube, kept counts, info[n, FIT_INFO_WORDS]); raises the batch's error."""
        if self.status is None:
            st = ctypes.c_int()
            self.ctx.check(self.ctx.lib.rp_batch_wait(self.ctx.ptr, self.ticket, ctypes.byref(st)), "rp_batch_wait")
            self.status = st.value
        self.ctx.check(self.status, "batch")
        res, o = [], 0
        for c in self.cubes:
            res.append(self.q[o:o + c.n_atoms])
            o += c.n_atoms
        return res, self.M, self.info.reshape(-1, _lib.FIT_INFO_WORDS)


class Ewald:
    def __init__(self, ctx: Context, n_grid, axis, cutoff, kmax):
        self.ctx = ctx
        p = ctypes.c_void_p()
        g = _lib.make_grid(n_grid, axis)
        ctx.check(ctx.lib.rp_ewald_setup(ctx.ptr, ctypes.byref(g), float(cutoff), int(kmax), ctypes.byref(p)),
                  "rp_ewald_setup")
        self.ptr = p
        K, S, al = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        ctx.lib.rp_ewald_info(p, ctypes.byref(K), ctypes.byref(S), ctypes.byref(al))
        self.K, self.S, self.alpha = K.value, S.value, al.value

    def close(self):
        if self.ptr:
            self.ctx.lib.rp_ewald_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
