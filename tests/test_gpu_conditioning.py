"""Conditioning and precision escalation on the GPU, through the C ABI.

Every solve reports kappa = ||A||_1 ||K^-1||_1 of its bordered system.  A
mixed-precision fit whose kappa / (n+1) exceeds the context's limit (default 2e5)
is refitted in plain FP64 and flagged, so an ill-conditioned cube never comes back
with silently wrong charges.  Parity bars:

* cfg2 (MOF-like, 424 atoms, 128^3, KMAX 12; golden ``mof128k12`` from repeat.py):
  kappa ~ 8e12.  Two FP64 solvers of the same normal equations already differ by
  2-4e-5 e there (rounding of A alone, 1e-16 relative, times kappa/(n+1) ~ 2e10), so
  the bar against repeat.py is 3e-5 e for the FP64 path and for the escalated
  mixed path (measured 2.3e-5 and 1.8e-5).
* cfg3 cell (triclinic 40 x 42 x 45 Bohr, 85/95/100 deg, symmetry + RESP): the
  mixed path against the FP64 path, 1e-5 e with 500 atoms.  At the full 2000 atoms /
  9.45 M points kappa ~ 2e12 escalates the mixed fit, and two FP64 fits of such a
  system agree only to a small multiple of kappa * eps64 * |q| (their sums run in
  different orders and, in the escalated fit, by other FP64 algorithms: the separable
  reciprocal sum, the exact two-word Gram): measured 1.7e-5 to 2.6e-4 e on charges of
  RMS 6.3 e and max 122 e.  The bar is 1e-3 e; unescalated the mixed fit is 9.9e-2
  away.
* well-conditioned cubes are not escalated (the mixed path's speed is kept).
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

COND_BAR = 3e-5   # cfg2 against repeat.py: the FP64 solver spread on this system


@pytest.fixture(scope="module")
def mof128(gpu_ctx):
    return load_golden("mof128k12")


def _batch(ctx, cube, prec):
    from pyrepeat_gb300 import _lib
    q, M, info = ctx.fit_batch([cube], prec, V_dev=[cube.V_dev] if cube.V is None else None)
    return np.asarray(q[0]).copy(), int(M[0]), _lib.fit_info(info[0])


def test_fp64_fit_cfg2_matches_reference(gpu_ctx, mof128):
    from pyrepeat_gb300 import _lib
    cube, g = mof128
    q, M, info = _batch(gpu_ctx, cube, _lib.PREC_FP64)
    assert M == g["kept"]
    assert info["precision"] == "fp64" and not info["escalated"]
    assert info["kappa"] > 1e12
    assert np.abs(q - g["q_ref"]).max() <= COND_BAR


def test_mixed_fit_cfg2_escalates_to_fp64(gpu_ctx, mof128):
    from pyrepeat_gb300 import _lib
    cube, g = mof128
    q, _, info = _batch(gpu_ctx, cube, _lib.PREC_MIXED)
    assert info["escalated"] and info["precision"] == "fp64"
    assert np.abs(q - g["q_ref"]).max() <= COND_BAR


def test_mixed_fit_without_escalation_reports_kappa(gpu_ctx, mof128):
    """With escalation off the mixed charges come back as they are, and kappa says why
    they cannot be trusted: kappa/(n+1) far above the default limit."""
    from pyrepeat_gb300 import _lib
    cube, _ = mof128
    gpu_ctx.set_kappa_limit(0.0)
    try:
        _, _, info = _batch(gpu_ctx, cube, _lib.PREC_MIXED)
    finally:
        gpu_ctx.set_kappa_limit(_lib.DEFAULT_KAPPA_LIMIT)
    assert not info["escalated"] and info["precision"] == "mixed"
    n1 = cube.n_atoms + 1
    assert info["kappa"] / n1 > 100 * _lib.DEFAULT_KAPPA_LIMIT


def test_mofmini_escalates_and_matches_reference(gpu_ctx):
    """The mini MOF cube (53 atoms on 800 kept points, kappa/(n+1) ~ 3e6) lands 6e-5 e
    from FP64 in mixed precision; escalated it matches repeat.py to 1e-7."""
    from pyrepeat_gb300 import _lib
    cube, g = load_golden("mofmini")
    q, _, info = _batch(gpu_ctx, cube, _lib.PREC_MIXED)
    assert info["escalated"]
    assert np.abs(q - g["q_ref"]).max() <= 1e-7


@pytest.mark.parametrize("name", ["water72", "tricmini", "batch1", "batch2"])
def test_well_conditioned_fits_stay_mixed(name, gpu_ctx):
    from pyrepeat_gb300 import _lib
    cube, g = load_golden(name)
    q, _, info = _batch(gpu_ctx, cube, _lib.PREC_MIXED)
    assert not info["escalated"] and info["precision"] == "mixed"
    assert info["kappa"] / (cube.n_atoms + 1) < _lib.DEFAULT_KAPPA_LIMIT
    assert np.abs(q - g["q_ref"]).max() <= 1e-5


def test_kappa_estimate_matches_numpy(gpu_ctx):
    """The solve's Hager estimate of ||K^-1||_1 against NumPy's exact inverse (small
    bordered system with symmetry and RESP folded in)."""
    from pyrepeat_gb300 import _lib
    cube, _ = load_golden("tricmini")
    r = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64, keep_normal=True)
    A = r.A.cpu().numpy()
    N = cube.n_atoms
    base = np.arange(N)
    for grp in cube.symm_groups:
        base[grp[1:]] = grp[0]
    keep = [i for i in range(N) if base[i] == i]
    G = np.zeros((N, len(keep)))
    for i in range(N):
        G[i, keep.index(base[i])] = 1.0
    Ar = G.T @ A @ G
    from pyrepeat_gb300.constants import z_to_symbol
    for k, a in enumerate(keep):
        s = cube.resp.get(z_to_symbol(int(cube.atom_index[a])))
        if s:
            Ar[k, k] += s[0]
    n = len(keep)
    K = np.zeros((n + 1, n + 1))
    K[:n, :n] = Ar
    K[:n, n] = K[n, :n] = G.sum(axis=0)
    kappa = np.abs(Ar).sum(axis=0).max() * np.abs(np.linalg.inv(K)).sum(axis=0).max()
    assert kappa / 3 <= r.info["kappa"] <= kappa * (1 + 1e-3)


def test_staged_mixed_gram_many_chunks(gpu_ctx):
    """rp_gram's two-pass mixed path over many chunks (each with a fixed-point scale of
    its own, the first chunk's centre) against one chunk and against FP64."""
    from pyrepeat_gb300 import _lib
    L = gpu_ctx.lib
    L.rp_debug_chunk_cap.restype = ctypes.c_int
    L.rp_debug_chunk_cap.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
    cube, g = load_golden("batch1")
    one = gpu_ctx.fit_cube(cube, precision=_lib.PREC_MIXED).charges
    assert L.rp_debug_chunk_cap(gpu_ctx.ptr, 8192) == 0
    try:
        many = gpu_ctx.fit_cube(cube, precision=_lib.PREC_MIXED).charges
    finally:
        L.rp_debug_chunk_cap(gpu_ctx.ptr, 0)
    assert np.abs(many - one).max() <= 1e-6
    assert np.abs(many - g["q_ref"]).max() <= 1e-5


def _tric_cell(gpu_ctx, n_atoms, n_groups, n_grid, seed):
    from pyrepeat_gb300 import synth
    return synth.make_tric(seed, n_grid=n_grid, n_atoms=n_atoms, n_groups=n_groups, ctx=gpu_ctx)


def test_tric_cell_500_atoms_mixed_matches_fp64(gpu_ctx):
    """cfg3's full triclinic cell with 500 atoms, 40 symmetry groups and RESP on a
    100 x 105 x 113 grid: the mixed fit (escalated or not, as its kappa decides) within
    1e-5 e of the FP64 fit."""
    from pyrepeat_gb300 import _lib
    cube = _tric_cell(gpu_ctx, 500, 40, (100, 105, 113), 11)
    q64, M, i64 = _batch(gpu_ctx, cube, _lib.PREC_FP64)
    qm, Mm, im = _batch(gpu_ctx, cube, _lib.PREC_MIXED)
    assert M == Mm > 0
    assert np.abs(qm - q64).max() <= 1e-5
    for grp in cube.symm_groups:
        assert np.ptp(qm[grp]) == 0.0


def test_tric_full_size_mixed_against_fp64(gpu_ctx):
    """cfg3 at full size (2000 atoms, 200 x 210 x 225 grid, 150 groups, RESP): kappa/(n+1)
    ~ 1e9 sends the mixed fit to FP64; it agrees with the plain FP64 fit to the FP64
    spread of this system (the order of the sums; see the module docstring)."""
    from pyrepeat_gb300 import _lib
    cube = _tric_cell(gpu_ctx, 2000, 150, (200, 210, 225), 1000)
    q64, M, i64 = _batch(gpu_ctx, cube, _lib.PREC_FP64)
    qm, _, im = _batch(gpu_ctx, cube, _lib.PREC_MIXED)
    assert im["escalated"]
    assert np.abs(qm - q64).max() <= 1e-3
