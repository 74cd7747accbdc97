"""``ChargeCalculator``: the reference's fit entry point, on the GB300 path.

Mirrors ``ChargeCalculator`` of repeat.py (constructor at repeat.py:1736-1780,
``fit_charges`` at 2184, ``compute_stats`` at 2326-2441) for the periodic
REPEAT fit: the same constructor arguments and file formats (cube or LOCPOT,
symmetry groups, RESP parameters), ``fit_charges()`` returning the charges and
``compute_stats()`` returning the RMS of the fitted ESP.  Underneath, one
``rp_fit_batch`` call runs the filter, the normal equations and the constrained
solve on the device (no Phi matrix, no host Gram), and ``rp_potential`` gives
Phi q for the statistics without forming Phi.

Arguments that only steer the reference's CPU backends (``n_cores``,
``block_k``, ``use_jit``) are accepted and have no effect.  ``fit_flag=0`` fits the
non-periodic 1/r basis (repeat.py:991-994) with the same machinery (KMAX 0 in the
device library).  A QEq file restrains the fit as the reference's ``_apply_qeq``
does, and ``compute_qeq_charges()`` gives QEq charges (repeat.py:2539-2634) from
``rp_qeq``: the Coulomb matrix on the device and the equalisation solve.  There is
no CPU fallback: without a CUDA device every call raises.
"""
from __future__ import annotations

import numpy as np

from . import _lib, cube as cube_io, qeq as qeq_mod
from .fit import Context
from .synth import Cube

_CTX: dict[int, Context] = {}


def _context(device: int) -> Context:
    if device not in _CTX:
        _CTX[device] = Context(device)
    return _CTX[device]


class ChargeCalculator:
    """Periodic REPEAT fit of one ESP cube on one GPU."""

    def __init__(self, cube_file, fit_flag=1, vdw_factor=1.0, vdw_max=1000.0, R_cutoff=20.0, q_tot=0.0,
                 symm_file=None, resp_file=None, qeq_file=None, n_cores=None, block_k=64, use_jit=True,
                 device: int = 0, fp64: bool = False, kmax: int = 7, verbose: bool = False):
        self.cube_file = cube_file
        self.fit_flag = int(fit_flag)
        if self.fit_flag not in (0, 1):
            raise ValueError("fit_flag must be 0 (non-periodic 1/r basis) or 1 (periodic Ewald)")
        self.vdw_factor = float(vdw_factor)
        self.vdw_max = float(vdw_max)
        self.R_cutoff = float(R_cutoff)
        self.q_tot = float(q_tot)
        self.symm_file, self.resp_file, self.qeq_file = symm_file, resp_file, qeq_file
        self.n_cores, self.block_k, self.use_jit = n_cores, block_k, use_jit
        self.device, self.fp64, self.kmax, self.verbose = int(device), bool(fp64), int(kmax), verbose

        self.cube = cube_io.read_data(cube_file)
        self.n_atoms = int(self.cube["n_atoms"])
        self.box_vectors = np.array([self.cube["n_grid"][i] * self.cube["axis_vector"][i] for i in range(3)],
                                    dtype=np.float64)
        self.volume = float(np.dot(self.box_vectors[0], np.cross(self.box_vectors[1], self.box_vectors[2])))
        groups = cube_io.read_symmetry(symm_file) if symm_file else []
        self.symm_data = {"trees": [{"n_equiv": len(g), "base": g[0], "linked": g[1:]} for g in groups],
                          "n_independent": len(groups)} if symm_file else None
        resp = cube_io.read_resp(resp_file) if resp_file else None
        self.resp_data = ({el: {"strength": s, "target": t} for el, (s, t) in resp.items()} if resp_file
                          else None)
        self.qeq_data = qeq_mod.read_qeq_file(qeq_file) if qeq_file else None
        self._groups = groups or None
        self._resp = resp or None
        # repeat.py:2288-2294: RESP when its table is non-empty, else the QEq restraint when
        # the QEq table is non-empty; both are diagonal restraints of the bordered system
        self._restraint = self._resp or (qeq_mod.restraint_table(self.cube["atom_index"], self.qeq_data)
                                         if self.qeq_data else None) or None
        self._kept = None      # device kept indices (flat order) and centred ESP, for the statistics
        self._Vc = None
        self.charges = None
        self.n_kept = None
        self.info = None

    # ---------------------------------------------------------------- helpers
    @property
    def ctx(self) -> Context:
        return _context(self.device)

    def to_cube(self) -> Cube:
        """The fit description the device library takes."""
        c = self.cube
        return Cube(np.asarray(c["atom_index"], dtype=np.int64), np.asarray(c["atom_pos"], dtype=np.float64),
                    np.asarray(c["n_grid"], dtype=np.int64), np.asarray(c["axis_vector"], dtype=np.float64),
                    np.ascontiguousarray(c["V_flat"], dtype=np.float64), symm_groups=self._groups,
                    resp=self._restraint,
                    kmax=self.kmax if self.fit_flag == 1 else 0, cutoff=self.R_cutoff,
                    vdw_factor=self.vdw_factor, vdw_max=self.vdw_max,
                    total_charge=self.q_tot, name=str(self.cube_file))

    def _filtered(self):
        """Kept flat indices (reference order) and the centred ESP at them, on the device."""
        if self._kept is None:
            t = self.ctx.torch
            c = self.cube
            V = t.from_numpy(np.ascontiguousarray(c["V_flat"], dtype=np.float64)).to(self.ctx.dev)
            kept, Vc, M, _ = self.ctx.filter(c["n_grid"], c["axis_vector"], c["atom_pos"], c["atom_index"], V,
                                             self.vdw_factor, self.vdw_max)
            self._kept, self._Vc = kept, Vc
            self.n_kept = M
        return self._kept, self._Vc

    @property
    def grid_pos(self) -> np.ndarray:
        """Kept grid positions (M, 3), i*a0 + j*a1 + k*a2 without the origin (repeat.py:2090-2110)."""
        kept, _ = self._filtered()
        f = kept.cpu().numpy().astype(np.int64)
        nx, ny, _nz = (int(v) for v in self.cube["n_grid"])
        k = f // (nx * ny)
        r = f - k * nx * ny
        j = r // nx
        i = r - j * nx
        a = np.asarray(self.cube["axis_vector"], dtype=np.float64)
        g = np.empty((len(f), 3))
        g[:] = a[0]
        g *= i[:, None]
        g += a[1] * j[:, None]
        g += a[2] * k[:, None]
        return g

    @property
    def V_pot(self) -> np.ndarray:
        """Centred ESP at the kept points (repeat.py:2113)."""
        _, Vc = self._filtered()
        return Vc.cpu().numpy()

    # ---------------------------------------------------------------- the fit
    def fit_charges(self) -> np.ndarray:
        """Fitted charges (N,) under the total-charge, symmetry and RESP constraints."""
        prec = _lib.PREC_FP64 if self.fp64 else _lib.PREC_MIXED
        q, M, info = self.ctx.fit_batch([self.to_cube()], prec)
        self.charges = np.asarray(q[0], dtype=np.float64)
        self.n_kept = int(M[0])
        self.info = _lib.fit_info(info[0])
        return self.charges

    def compute_stats(self, charges, need_v_coul=True) -> dict:
        """RMS of the fitted ESP against the centred QM ESP over the kept points, both
        shifted by their means (repeat.py:2326-2441); 'rrms' adds the relative RMS
        sqrt(sum d^2 / sum Vc^2).  V_coul = Phi q comes from rp_potential."""
        kept, Vc = self._filtered()
        c = self.cube
        ew = self.ctx.ewald(c["n_grid"], c["axis_vector"], self.R_cutoff, self.kmax if self.fit_flag == 1 else 0)
        try:
            vcoul = self.ctx.potential(ew, c["atom_pos"], np.asarray(charges, dtype=np.float64), kept)
        finally:
            ew.close()
        avrg_coul = float(vcoul.mean())
        avrg_qm = float(Vc.mean())
        d = (vcoul - avrg_coul) - (Vc - avrg_qm)
        ss = float((d * d).sum())
        n = int(Vc.numel())
        out = {"rms_error": float(np.sqrt(ss / n)), "avrg_qm": avrg_qm, "avrg_coul": avrg_coul,
               "rrms": float(np.sqrt(ss / max(float((Vc * Vc).sum()), 1e-300)))}
        if need_v_coul:
            out["V_coul"] = vcoul.cpu().numpy()
        return out

    def compute_qeq_charges(self, param_set=None) -> np.ndarray:
        """QEq charges (repeat.py:2539-2634): per-atom chi and J_ii from the QEq file, then
        ``param_set`` (default: the reference's table; a caller's set selects EQeq and its
        hydrogen rule), else 0.15 / 0.50 with a warning; then rp_qeq builds the Coulomb
        matrix under this calculator's Ewald parameters (1/r for fit_flag 0) and solves
        the equalisation system under the total charge."""
        c = self.cube
        chi, jself, method, missing = qeq_mod.charge_parameters(c["atom_index"], self.qeq_data, param_set)
        for sym in missing:
            print(f"Warning: No parameters for {sym}, using defaults")
        if self.verbose:
            print(f"Computing {method} Coulomb matrix...")
        q, _J, info = self.ctx.qeq(c["n_grid"], c["axis_vector"], c["atom_pos"], chi, jself, self.q_tot,
                                   self.R_cutoff, self.kmax if self.fit_flag == 1 else 0)
        self.qeq_info = info
        return q
