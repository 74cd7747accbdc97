"""QEq: the charges of compute_qeq_charges (repeat.py:2539-2634) through rp_qeq, and the
QEq restraint of the fit (repeat.py:2288-2294, 2522-2535).

CPU: the parameter rules (file, default table, EQeq hydrogen, missing elements, the
reference's all-or-nothing file parser, RESP taking precedence) and the restraint's
(s, t) form.  GPU: rp_qeq's charges against repeat.py's (golden fixtures) and its
Coulomb matrix against the oracle's, periodic and 1/r; the restrained fit through
ChargeCalculator; the command line with --charge qeq and --output."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, load_golden, load_qeq
from pyrepeat_gb300 import qeq as Q, synth

SMALL = ["water24", "tricmini", "mofmini"]


def test_qeq_file_parser(tmp_path):
    f = tmp_path / "q.txt"
    f.write_text("O 0.31 0.30\n# comment\nC 0.21 0.22 extra\n\nN 1\n")
    assert Q.read_qeq_file(str(f)) == {"O": {"electroneg": 0.31, "hardness": 0.30},
                                       "C": {"electroneg": 0.21, "hardness": 0.22}}
    f.write_text("O 0.31 0.30\nC x 0.22\n")              # one unreadable value: no table at all
    assert Q.read_qeq_file(str(f)) == {}
    assert Q.read_qeq_file(str(tmp_path / "missing.txt")) == {}


def test_charge_parameters_rules():
    Z = [8, 1, 82, 6]                                   # O, H, Pb (no parameters), C
    qd = {"C": {"electroneg": 0.21, "hardness": 0.22}}
    chi, js, method, missing = Q.charge_parameters(Z, qd)
    assert method == "QEq" and missing == ["Pb"]
    assert chi.tolist() == [0.320234, 0.166401, 0.15, 0.21]
    assert js.tolist() == [2 * 0.314869, 2 * 0.255225, 0.50, 2 * 0.22]
    chi, js, method, _ = Q.charge_parameters(Z, qd, Q.DEFAULT_QEQ_PARAMS)
    assert method == "EQeq"
    assert chi[1] == 0.5 * (13.598 + -2.0) * Q.EV_TO_HARTREE and js[1] == (13.598 - -2.0) * Q.EV_TO_HARTREE


def test_restraint_table_form():
    qd = {"O": {"electroneg": 0.31, "hardness": 0.30}, "Zz": {"electroneg": 1.0, "hardness": 1.0}}
    t = Q.restraint_table([8, 1, 1, 82], qd)
    assert set(t) == {"O", "H"}                          # Pb: neither in the file nor in the table
    s, tt = t["O"]
    assert s == 0.30 and abs(s * tt - 0.31) <= 1e-16
    assert t["H"][0] == 0.255225
    assert Q.restraint_table([8], {"O": {"electroneg": 0.0, "hardness": 0.0}}) == {}
    with pytest.raises(ValueError):
        Q.restraint_table([8], {"O": {"electroneg": 0.3, "hardness": 0.0}})


def test_resp_takes_precedence(tmp_path):
    """repeat.py:2288-2294: a non-empty RESP table wins over the QEq file."""
    from pyrepeat_gb300.calculator import ChargeCalculator
    cube, _ = load_golden("water24")
    cf = tmp_path / "w.cube"
    synth.write_cube(str(cf), cube)
    qf = tmp_path / "q.txt"
    qf.write_text("O 0.31 0.30\n")
    rf = tmp_path / "r.txt"
    synth.write_resp_file(str(rf), {"H": (0.01, 0.4)})
    a = ChargeCalculator(str(cf), qeq_file=str(qf))
    assert a._restraint == Q.restraint_table(cube.atom_index, Q.read_qeq_file(str(qf)))
    b = ChargeCalculator(str(cf), qeq_file=str(qf), resp_file=str(rf))
    assert b._restraint == b._resp and "O" not in b._restraint


@pytest.mark.gpu
@pytest.mark.parametrize("name", SMALL + ["pb"])
def test_qeq_charges_match_reference(name, gpu_ctx, oracle_mod):
    z, qd, _, qtot = load_qeq()
    cube, _ = load_golden("water24" if name == "pb" else name)
    Z = z["atom_index_pb"] if name == "pb" else cube.atom_index
    qd = None if name == "pb" else qd
    for f in ((1,) if name == "pb" else (1, 0)):
        kmax = cube.kmax if f else 0
        chi, js, _, _ = Q.charge_parameters(Z, qd)
        q, J, info = gpu_ctx.qeq(cube.n_grid, cube.axis_vector, cube.atom_pos, chi, js, qtot, cube.cutoff, kmax,
                                 want_J=True)
        assert np.array_equal(J, J.T) and np.array_equal(np.diag(J), js)
        Jo = oracle_mod.qeq_matrix(cube.atom_pos, cube.box_vectors, cube.cutoff, kmax, js)
        assert np.abs(J - Jo).max() <= 1e-12 * np.abs(Jo).max()
        assert np.abs(q - z[f"q_qeq{f}_{name}"]).max() <= 1e-9
        assert abs(q.sum() - qtot) <= 1e-12
        assert info["residual"] <= 1e-10
    if name != "pb":
        chi, js, _, _ = Q.charge_parameters(Z, qd, Q.DEFAULT_QEQ_PARAMS)
        q, _, _ = gpu_ctx.qeq(cube.n_grid, cube.axis_vector, cube.atom_pos, chi, js, qtot, cube.cutoff, cube.kmax)
        assert np.abs(q - z[f"q_eqeq_{name}"]).max() <= 1e-9


@pytest.mark.gpu
def test_qeq_large_system_matches_oracle(gpu_ctx, oracle_mod):
    """An 800-atom cell (atoms on a jittered 5 Bohr lattice: J stays positive definite and
    the system well conditioned, cond ~250; at 3.3 Bohr random elements make it
    indefinite, charges reach hundreds of e and any two FP64 solvers differ at cond x eps):
    rp_qeq's matrix and charges against the oracle's (the wide LU with FP64 refinement)."""
    rng = np.random.default_rng(11)
    L = 50.0
    n = 800
    site = np.stack(np.meshgrid(*[np.arange(10)] * 3, indexing="ij"), -1).reshape(-1, 3)
    site = site[rng.choice(len(site), size=n, replace=False)]
    atoms = (site + 0.5 + rng.uniform(-0.15, 0.15, size=(n, 3))) * (L / 10)
    Z = rng.choice([1, 6, 8, 30], size=n)
    chi, js, _, _ = Q.charge_parameters(Z)
    ngrid = np.array([100, 100, 100])
    axis = np.eye(3) * (L / 100)
    q, J, info = gpu_ctx.qeq(ngrid, axis, atoms, chi, js, 0.0, 20.0, 7, want_J=True)
    Jo = oracle_mod.qeq_matrix(atoms, np.eye(3) * L, 20.0, 7, js)
    assert np.abs(J - Jo).max() <= 1e-12 * np.abs(Jo).max()
    qo = oracle_mod.qeq_charges(Jo, chi, 0.0)
    assert np.abs(q - qo).max() <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", SMALL)
def test_qeq_restrained_fit_matches_reference(name, tmp_path):
    """ChargeCalculator with a QEq file (no RESP): mixed and FP64 fits against repeat.py."""
    from pyrepeat_gb300.calculator import ChargeCalculator
    z, _, text, qtot = load_qeq()
    cube, _ = load_golden(name)
    cf = os.path.join(tmp_path, "c.cube")
    synth.write_cube(cf, cube)
    qf = os.path.join(tmp_path, "q.txt")
    with open(qf, "w") as f:
        f.write(text)
    sf = None
    if cube.symm_groups:
        sf = os.path.join(tmp_path, "s.txt")
        synth.write_symmetry_file(sf, cube.symm_groups)
    for f in (1, 0):
        ref = z[f"q_qeqr{f}_{name}"]
        for fp64, tol in ((True, 1e-8), (False, 1e-5)):
            calc = ChargeCalculator(cf, fit_flag=f, q_tot=qtot, symm_file=sf, qeq_file=qf, kmax=cube.kmax,
                                    fp64=fp64)
            q = calc.fit_charges()
            assert np.abs(q - ref).max() <= tol, (f, fp64)


@pytest.mark.gpu
def test_cli_qeq_charges(tmp_path):
    """--charge qeq through the whole program: printed charges and the --output file."""
    z, _, text, qtot = load_qeq()
    cube, _ = load_golden("tricmini")
    cf = os.path.join(tmp_path, "t.cube")
    qf = os.path.join(tmp_path, "q.txt")
    of = os.path.join(tmp_path, "qeq.txt")
    synth.write_cube(cf, cube)
    with open(qf, "w") as f:
        f.write(text)
    cmd = [sys.executable, "-m", "pyrepeat_gb300", cf, "--gpu", "0", "--charge", "qeq", "--qeq-file", qf,
           "--total-charge", str(qtot), "--output", of]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "QEq Charges:" in r.stdout
    rows = re.findall(r"^\s*(\d+)\s+([A-Z][a-z]?)\s+(-?\d+\.\d+)\s*$", r.stdout, re.M)
    q = np.array([float(x[2]) for x in rows])
    ref = z["q_qeq1_tricmini"]
    assert len(q) == cube.n_atoms and np.abs(q - ref).max() <= 5e-7
    out = open(of).read().split("\n")
    assert len([ln for ln in out if ln.strip()]) == cube.n_atoms
    f0 = out[0].split()
    assert f0[0] == "1" and np.allclose([float(v) for v in f0[2:5]], cube.atom_pos[0], atol=1e-6)
    assert abs(float(f0[5]) - ref[0]) <= 5e-7
