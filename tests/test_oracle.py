"""The CPU oracle pinned against the reference's own outputs (golden fixtures
made by running repeat.py and the compiled repeat_cpu_omp on the same cubes)."""
import hashlib

import numpy as np
import pytest

from conftest import load_golden

SMALL = ["water24", "mofmini", "tricmini"]


@pytest.mark.parametrize("name", SMALL)
def test_oracle_mask_matches_reference(name, oracle_mod):
    cube, g = load_golden(name)
    mask, kept = oracle_mod.filter_mask(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index,
                                        cube.vdw_factor, cube.vdw_max)
    assert kept == g["kept"]
    assert np.array_equal(mask, g["mask"])
    assert hashlib.sha256(np.packbits(mask).tobytes()).hexdigest() == g["mask_sha256"]


@pytest.mark.parametrize("name", SMALL)
def test_sqrt_rule_agrees_with_squared_rule(name, oracle_mod):
    """The reference's CPU cdist filter compares sqrt distances, its GPU filter
    squared ones; they may differ only at rounding ties (expected: none)."""
    cube, g = load_golden(name)
    m2, _ = oracle_mod.filter_mask(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index)
    m1, _ = oracle_mod.filter_mask(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index, sqrt_rule=True)
    assert int((m1 != m2).sum()) == 0


# FP64 vs FP64: the dense MOF-like cube is ill-conditioned, so two FP64
# implementations (different summation order) agree only to ~1e-9 there
@pytest.mark.parametrize("name,tol", [("water24", 1e-10), ("mofmini", 1e-7), ("tricmini", 1e-10)])
def test_oracle_charges_match_reference(name, tol, oracle_mod):
    cube, g = load_golden(name)
    q = oracle_mod.OracleFit(cube).fit()
    assert np.abs(q - g["q_ref"]).max() < tol
    assert abs(q.sum() - cube.total_charge) < 1e-10


@pytest.mark.parametrize("name,tol", [("water24", 1e-10), ("mofmini", 1e-7), ("tricmini", 1e-10)])
def test_oracle_nonperiodic_charges_match_reference(name, tol, oracle_mod):
    """--fit-type 0 (the 1/r basis, KMAX 0 here): the oracle against repeat.py's charges."""
    from conftest import load_nonperiodic
    cube, q_ref0 = load_nonperiodic(name)
    q = oracle_mod.OracleFit(cube).fit()
    assert np.abs(q - q_ref0).max() <= tol * max(1.0, np.abs(q_ref0).max())


@pytest.mark.parametrize("name", SMALL + ["pb"])
def test_oracle_qeq_charges_match_reference(name, oracle_mod):
    """QEq charges (repeat.py:2539-2634): the oracle's Coulomb matrix and difference-form
    solve against repeat.py's compute_qeq_charges, periodic and 1/r, QEq and EQeq."""
    from conftest import load_qeq
    from pyrepeat_gb300 import qeq as Q
    z, qd, _, qtot = load_qeq()
    cube, _ = load_golden("water24" if name == "pb" else name)
    Z = z["atom_index_pb"] if name == "pb" else cube.atom_index
    qd = None if name == "pb" else qd
    for f in ((1,) if name == "pb" else (1, 0)):
        chi, js, _, missing = Q.charge_parameters(Z, qd)
        assert missing == (["Pb"] if name == "pb" else [])
        J = oracle_mod.qeq_matrix(cube.atom_pos, cube.box_vectors, cube.cutoff, cube.kmax if f else 0, js)
        q = oracle_mod.qeq_charges(J, chi, qtot)
        assert np.abs(q - z[f"q_qeq{f}_{name}"]).max() <= 1e-10
        assert abs(q.sum() - qtot) <= 1e-12
    if name != "pb":
        chi, js, method, _ = Q.charge_parameters(Z, qd, Q.DEFAULT_QEQ_PARAMS)
        assert method == "EQeq"
        J = oracle_mod.qeq_matrix(cube.atom_pos, cube.box_vectors, cube.cutoff, cube.kmax, js)
        assert np.abs(oracle_mod.qeq_charges(J, chi, qtot) - z[f"q_eqeq_{name}"]).max() <= 1e-10


@pytest.mark.parametrize("name", SMALL)
def test_oracle_qeq_restrained_fit_matches_reference(name, oracle_mod):
    """--qeq-file without RESP (repeat.py:2288-2294, 2522-2535) restrains the fit; as the
    diagonal restraint (s, t) = (hardness, chi / hardness) the oracle matches repeat.py."""
    import copy
    from conftest import load_qeq
    from pyrepeat_gb300 import qeq as Q
    z, qd, _, qtot = load_qeq()
    cube, _ = load_golden(name)
    for f in (1, 0):
        c = copy.copy(cube)
        c.resp = Q.restraint_table(cube.atom_index, qd)
        c.total_charge = qtot
        c.kmax = cube.kmax if f else 0
        q = oracle_mod.OracleFit(c).fit()
        assert np.abs(q - z[f"q_qeqr{f}_{name}"]).max() <= 1e-10


def test_reference_binary_agrees_on_plain_fit(oracle_mod):
    """repeat_cpu_omp prints 6 decimals; it fits the same plain problem."""
    cube, g = load_golden("water24")
    assert g["q_bin"] is not None
    assert np.abs(g["q_bin"] - g["q_ref"]).max() < 1e-6


def test_oracle_kspace_counts(oracle_mod):
    box = np.diag([18.0, 18.0, 18.0])
    for kmax, K in ((7, 754), (12, 3779), (13, 4804)):
        kv, kc = oracle_mod.kspace(box, 20.0, kmax)
        assert len(kc) == K
        assert np.all(kc > 0)


def test_planted_charges_recovered_without_noise(oracle_mod):
    """Known answer: V = Phi q exactly (no noise) -> the fit returns q."""
    from pyrepeat_gb300 import synth
    c = synth.make_water(3, n_grid=20, noise=0.0)
    q = oracle_mod.OracleFit(c).fit()
    assert np.abs(q - c.charges_true).max() < 1e-8


def test_constant_shift_of_V_leaves_charges(oracle_mod):
    cube, g = load_golden("water24")
    q0 = oracle_mod.OracleFit(cube).fit()
    cube.V = cube.V + 0.37
    q1 = oracle_mod.OracleFit(cube).fit()
    assert np.abs(q1 - q0).max() < 1e-9


def test_symmetry_groups_share_charge(oracle_mod):
    cube, g = load_golden("tricmini")
    q = oracle_mod.OracleFit(cube).fit()
    for grp in cube.symm_groups:
        assert np.ptp(q[grp]) == 0.0
