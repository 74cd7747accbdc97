"""Generate the golden fixtures from the reference itself (run in the container
that holds the reference tree; other machines only read the results).

For every case the seeded generator (pyrepeat_gb300.synth) builds a cube, the
cube is written as a Gaussian cube file, and:

* ``repeat.py`` (FP64, NumPy path, via ref_harness) reads it and fits charges;
  its kept-point mask, kept count and charges are recorded;
* for plain fits (vdw 1.0/1000, Rc 20, Q 0, KMAX 7) the compiled
  ``repeat_cpu_omp`` binary fits the same file and its charges are recorded.

Stored per case (tests/golden/<name>.npz): atoms, Z, grid, V exactly as read
back from the cube text, groups, RESP table, the reference's kept mask (packed
bits) and charges.  Large cubes store V only when small enough; otherwise the
test regenerates it from the stored atoms/charges/seed with the same generator.

Usage:  python tests/golden/make_golden.py [case ...]
        python tests/golden/make_golden.py --nonperiodic    (fit-type 0 charges of the small cases)
        python tests/golden/make_golden.py --qeq            (QEq charges and QEq-restrained fits)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from pyrepeat_gb300 import synth  # noqa: E402

MAX_STORED_V = 200_000


def cases():
    return {
        "water24": lambda: synth.make_water(1, n_grid=24),
        "water72": lambda: synth.make_water(1, n_grid=72),
        "mof128k12": lambda: synth.make_mof(2),
        "mofmini": lambda: synth.make_mof(5, n_grid=40, kmax=9, L=14.0, counts=(4, 13, 24, 12)),
        "tricmini": lambda: synth.make_tric(7, n_grid=(30, 32, 34), n_atoms=40, n_groups=6,
                                            lengths=(16.0, 17.0, 18.0)),
        "batch1": lambda: synth.make_batch_item(1),
        "batch2": lambda: synth.make_batch_item(2),
    }


def mask_digest(mask: np.ndarray) -> str:
    return hashlib.sha256(np.packbits(mask.astype(np.uint8)).tobytes()).hexdigest()


def reference_fit(R, cube_path, cube, kmax, fit_flag=1):
    """Run repeat.py's ChargeCalculator on a cube file; KMAX other than 7 is
    applied by re-running the reference's own k-space rule (repeat.py:1127-1143)
    with the larger KMAX after construction."""
    symm = resp = None
    tmp = os.path.dirname(cube_path)
    if cube.symm_groups:
        symm = os.path.join(tmp, "symm.txt")
        synth.write_symmetry_file(symm, cube.symm_groups)
    if cube.resp:
        resp = os.path.join(tmp, "resp.txt")
        synth.write_resp_file(resp, cube.resp)
    with kmax_patch(R, kmax):
        calc = R.ChargeCalculator(cube_path, fit_flag=fit_flag, vdw_factor=cube.vdw_factor, vdw_max=cube.vdw_max,
                                  R_cutoff=cube.cutoff, q_tot=cube.total_charge, symm_file=symm,
                                  resp_file=resp, use_jit=False)
        q = calc.fit_charges()
    nx, ny, nz = (int(v) for v in cube.n_grid)
    idx = np.rint(calc.grid_pos @ np.linalg.inv(cube.axis_vector)).astype(np.int64)
    flat = idx[:, 0] + idx[:, 1] * nx + idx[:, 2] * nx * ny
    mask = np.zeros(nx * ny * nz, dtype=np.uint8)
    mask[flat] = 1
    V_read = calc.cube["V_pot"].ravel(order="F").copy()
    return q, mask, V_read, len(calc.ewald.kvecs)


class kmax_patch:
    """Within the block, repeat.py's EwaldCalculator builds its k-set with this KMAX
    (the reference's own rule, repeat.py:1127-1143, with the constant replaced)."""

    def __init__(self, R, kmax):
        self.R, self.kmax, self.orig = R, kmax, None

    def __enter__(self):
        R, kmax = self.R, self.kmax
        if kmax == 7:
            return self
        self.orig = R.EwaldCalculator._setup_kspace

        def setup_kmax(self, _K=kmax):
            KMAX, KSQMAX = _K, _K * _K
            beta = 1.0 / (4.0 * self.alpha)
            kv, kc = [], []
            for kx in range(KMAX + 1):
                for ky in range(-KMAX, KMAX + 1):
                    for kz in range(-KMAX, KMAX + 1):
                        ksq = kx * kx + ky * ky + kz * kz
                        if ksq >= KSQMAX or ksq == 0:
                            continue
                        k = kx * self.recip_vectors[0] + ky * self.recip_vectors[1] + kz * self.recip_vectors[2]
                        k2 = np.dot(k, k)
                        kv.append(k)
                        kc.append((4.0 * np.pi / self.volume) * np.exp(-beta * k2) / k2)
            self.kvecs = np.asarray(kv, dtype=np.float64)
            self.kcoefs = np.asarray(kc, dtype=np.float64)
        R.EwaldCalculator._setup_kspace = setup_kmax
        return self

    def __exit__(self, *exc):
        if self.orig is not None:
            self.R.EwaldCalculator._setup_kspace = self.orig


NONPERIODIC_CASES = ("water24", "tricmini", "mofmini")


def main_nonperiodic():
    """--fit-type 0 (the non-periodic 1/r basis) of the small cases: repeat.py's charges
    on the same cube files, stored as tests/golden/nonperiodic.npz (q_ref0_<case>)."""
    from ref_harness import load_reference
    R = load_reference()
    allc = cases()
    out = {}
    for name in NONPERIODIC_CASES:
        cube = allc[name]()
        d = tempfile.mkdtemp()
        path = os.path.join(d, f"{name}.cube")
        synth.write_cube(path, cube)
        q, _mask, _V, _K = reference_fit(R, path, cube, 7, fit_flag=0)
        out[f"q_ref0_{name}"] = q
        print(name, "fit-type 0 charges", np.round(q[:4], 6), flush=True)
    np.savez_compressed(os.path.join(HERE, "nonperiodic.npz"), **out)


QEQ_CASES = ("water24", "tricmini", "mofmini")
QEQ_FILE_TEXT = "O 0.31 0.30\nC 0.21 0.22\n"   # two elements; the others fall back to the default table
QEQ_QTOT = 0.5
PB_Z = 82                                       # lead: no entry in the default QEq table


def main_qeq():
    """QEq of the small cases through repeat.py, stored as tests/golden/qeq.npz:
    q_qeq<f>_<case>  compute_qeq_charges() with the QEq file, fit type f (1 periodic, 0 1/r);
    q_eqeq_<case>    compute_qeq_charges(param_set=DEFAULT_QEQ_PARAMS): EQeq (hydrogen rule);
    q_qeqr<f>_<case> fit_charges() restrained by the QEq file (symmetry groups kept, no RESP);
    q_qeq1_pb        water24 with its last atom made lead (no parameters: 0.15 / 0.50), no file.
    Every run uses total charge QEQ_QTOT and the case's KMAX."""
    from ref_harness import load_reference
    R = load_reference()
    allc = cases()
    out = {"qtot": QEQ_QTOT, "qeq_file": QEQ_FILE_TEXT}
    for name in QEQ_CASES + ("pb",):
        cube = allc["water24" if name == "pb" else name]()
        if name == "pb":
            cube.atom_index = cube.atom_index.copy()
            cube.atom_index[-1] = PB_Z
            out["atom_index_pb"] = cube.atom_index.astype(np.int32)
        d = tempfile.mkdtemp()
        path = os.path.join(d, f"{name}.cube")
        synth.write_cube(path, cube)
        qf = None
        if name != "pb":
            qf = os.path.join(d, "qeq.txt")
            with open(qf, "w") as f:
                f.write(QEQ_FILE_TEXT)
        symm = None
        if cube.symm_groups:
            symm = os.path.join(d, "symm.txt")
            synth.write_symmetry_file(symm, cube.symm_groups)
        for fit_flag in ((1,) if name == "pb" else (1, 0)):
            with kmax_patch(R, cube.kmax):
                calc = R.ChargeCalculator(path, fit_flag=fit_flag, vdw_factor=cube.vdw_factor,
                                          vdw_max=cube.vdw_max, R_cutoff=cube.cutoff, q_tot=QEQ_QTOT,
                                          symm_file=symm, qeq_file=qf, use_jit=False)
                out[f"q_qeq{fit_flag}_{name}"] = calc.compute_qeq_charges()
                if name == "pb":
                    continue
                if fit_flag == 1:
                    out[f"q_eqeq_{name}"] = calc.compute_qeq_charges(param_set=R.DEFAULT_QEQ_PARAMS)
                out[f"q_qeqr{fit_flag}_{name}"] = calc.fit_charges()
            print(name, fit_flag, np.round(out[f"q_qeq{fit_flag}_{name}"][:4], 6), flush=True)
    np.savez_compressed(os.path.join(HERE, "qeq.npz"), **out)


def main(names):
    from ref_harness import load_reference
    import oracle as O
    R = load_reference()
    O.build_reference()
    allc = cases()
    summary = {}
    for name in names or list(allc):
        t0 = time.time()
        cube = allc[name]()
        d = tempfile.mkdtemp()
        path = os.path.join(d, f"{name}.cube")
        synth.write_cube(path, cube)
        q, mask, V_read, K = reference_fit(R, path, cube, cube.kmax)
        plain = (cube.kmax == 7 and not cube.symm_groups and not cube.resp and cube.vdw_factor == 1.0
                 and cube.vdw_max == 1000.0 and cube.cutoff == 20.0 and cube.total_charge == 0.0)
        q_bin = O.run_reference_binary(path) if plain else None
        store_V = V_read.size <= MAX_STORED_V
        groups = cube.symm_groups or []
        gptr, gidx = O.groups_to_csr(groups)
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            atom_index=cube.atom_index.astype(np.int32), atom_pos=cube.atom_pos, n_grid=cube.n_grid,
            axis_vector=cube.axis_vector, charges_true=cube.charges_true,
            V=V_read if store_V else np.zeros(0), mask_bits=np.packbits(mask),
            q_ref=q, q_bin=q_bin if q_bin is not None else np.zeros(0),
            group_ptr=gptr, group_idx=gidx,
            resp=json.dumps(cube.resp or {}), kmax=cube.kmax, cutoff=cube.cutoff,
            vdw_factor=cube.vdw_factor, vdw_max=cube.vdw_max, total_charge=cube.total_charge)
        summary[name] = {"kept": int(mask.sum()), "mask_sha256": mask_digest(mask), "K": K,
                         "N": cube.n_atoms, "grid": [int(v) for v in cube.n_grid], "V_stored": store_V,
                         "q_bin_vs_ref": (float(np.abs(q_bin - q).max()) if q_bin is not None else None),
                         "seconds": round(time.time() - t0, 1)}
        print(name, summary[name], flush=True)
    meta = os.path.join(HERE, "golden.json")
    old = json.load(open(meta)) if os.path.exists(meta) else {}
    old.update(summary)
    with open(meta, "w") as f:
        json.dump(old, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if sys.argv[1:] == ["--nonperiodic"]:
        main_nonperiodic()
    elif sys.argv[1:] == ["--qeq"]:
        main_qeq()
    else:
        main(sys.argv[1:])
