"""GPU parity of the filter and the plain FP64 fit against the oracle and the
reference's golden outputs (called through the C ABI)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["water24", "mofmini", "tricmini", "water72"])
def test_filter_mask_bit_exact(name, gpu_ctx, oracle_mod):
    import torch
    cube, g = load_golden(name)
    V = torch.from_numpy(cube.V).to(gpu_ctx.dev)
    kept, Vc, M, mask = gpu_ctx.filter(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index, V,
                                       cube.vdw_factor, cube.vdw_max, want_mask=True)
    m = mask.cpu().numpy()
    om, okept = oracle_mod.filter_mask(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index,
                                       cube.vdw_factor, cube.vdw_max)
    assert M == okept
    assert np.array_equal(m, om)
    if np.array_equal(g["atom_pos"], cube.atom_pos):
        assert np.array_equal(m, g["mask"])
    # kept indices ordered, V centred over kept points (repeat.py:2113)
    k = kept.cpu().numpy()
    assert np.all(np.diff(k) > 0)
    assert np.array_equal(k, np.flatnonzero(om))
    vk = cube.V[k]
    assert np.allclose(Vc.cpu().numpy(), vk - vk.mean(), rtol=0, atol=1e-13)


@pytest.mark.parametrize("name,tol", [("water24", 1e-8), ("mofmini", 1e-6), ("tricmini", 1e-8), ("water72", 1e-7)])
def test_fp64_fit_matches_reference(name, tol, gpu_ctx):
    from pyrepeat_gb300 import _lib
    cube, g = load_golden(name)
    r = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64)
    assert r.n_kept == g["kept"]
    assert np.abs(r.charges - g["q_ref"]).max() < tol
    assert abs(r.charges.sum() - cube.total_charge) < 1e-10


@pytest.mark.parametrize("name,tol", [("water24", 1e-8), ("mofmini", 1e-6), ("tricmini", 1e-8)])
def test_nonperiodic_fp64_fit_matches_reference(name, tol, gpu_ctx):
    """--fit-type 0 in plain FP64 against repeat.py's charges."""
    from conftest import load_nonperiodic
    from pyrepeat_gb300 import _lib
    cube, q0 = load_nonperiodic(name)
    r = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64)
    assert np.abs(r.charges - q0).max() <= tol * max(1.0, np.abs(q0).max())


def test_fp64_normal_equations_match_oracle(gpu_ctx, oracle_mod):
    from pyrepeat_gb300 import _lib
    cube, _ = load_golden("tricmini")
    r = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64, keep_normal=True)
    of = oracle_mod.OracleFit(cube)
    A, b, sp, sv = of.normal_equations()
    Ag = r.A.cpu().numpy()
    bg = r.b.cpu().numpy()
    assert np.abs(Ag - A).max() <= 1e-9 * np.abs(A).max()
    assert np.abs(bg - b).max() <= 1e-9 * np.abs(b).max() + 1e-12


def test_host_entry_point_equals_staged_fit(gpu_ctx):
    from pyrepeat_gb300 import _lib
    cube, g = load_golden("tricmini")
    a = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64)
    b = gpu_ctx.fit_host(cube, precision=_lib.PREC_FP64)
    assert a.n_kept == b.n_kept
    assert np.abs(a.charges - b.charges).max() < 1e-12


def test_repeated_fits_are_bitwise_identical(gpu_ctx):
    from pyrepeat_gb300 import _lib
    cube, _ = load_golden("mofmini")
    a = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64).charges
    b = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64).charges
    assert np.array_equal(a, b)


def test_no_survivors_is_an_error(gpu_ctx):
    from pyrepeat_gb300 import _lib, synth
    cube, _ = load_golden("water24")
    cube.vdw_factor = 50.0   # every point inside some sphere
    with pytest.raises(_lib.RepeatError):
        gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64)
