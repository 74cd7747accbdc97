"""GPU parity of the mixed-precision fit (separable double-float reciprocal sum,
FP32 real space with FP64 cutoff decisions, exact fixed-point Gram on the
tensor cores) against the reference's golden charges, the oracle's Phi and the
FP64 path, through the C ABI.

Tolerance: max|dq| <= 1e-5 e on well-conditioned fits (the target the fit is
specified to); measured margins are far larger (~1e-7 e or better)."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

WELL_CONDITIONED = ["water24", "tricmini", "water72", "batch1", "batch2"]


@pytest.mark.parametrize("name", WELL_CONDITIONED)
def test_mixed_fit_matches_reference(name, gpu_ctx):
    from pyrepeat_gb300 import _lib
    cube, g = load_golden(name)
    r = gpu_ctx.fit_cube(cube, precision=_lib.PREC_MIXED)
    assert r.n_kept == g["kept"]
    assert np.abs(r.charges - g["q_ref"]).max() <= 1e-5
    assert abs(r.charges.sum() - cube.total_charge) < 1e-10


@pytest.mark.parametrize("name", ["water24", "tricmini"])
def test_nonperiodic_mixed_fit_matches_reference(name, gpu_ctx):
    """--fit-type 0 (the 1/r basis, KMAX 0): staged path and batched single-pass path
    against repeat.py's charges."""
    from conftest import load_nonperiodic
    from pyrepeat_gb300 import _lib
    cube, q0 = load_nonperiodic(name)
    r = gpu_ctx.fit_cube(cube, precision=_lib.PREC_MIXED)
    assert np.abs(r.charges - q0).max() <= 1e-5
    q, _, _ = gpu_ctx.fit_batch([cube], _lib.PREC_MIXED)
    assert np.abs(q[0] - q0).max() <= 1e-5


@pytest.mark.parametrize("name", ["tricmini", "batch1"])
def test_mixed_normal_equations_close_to_fp64(name, gpu_ctx):
    from pyrepeat_gb300 import _lib
    cube, _ = load_golden(name)
    a = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64, keep_normal=True)
    b = gpu_ctx.fit_cube(cube, precision=_lib.PREC_MIXED, keep_normal=True)
    A64, Am = a.A.cpu().numpy(), b.A.cpu().numpy()
    b64, bm = a.b.cpu().numpy(), b.b.cpu().numpy()
    assert np.abs(Am - A64).max() <= 1e-6 * np.abs(A64).max()
    assert np.abs(bm - b64).max() <= 1e-6 * np.abs(b64).max()


def _brick_order(kept, n_grid):
    """The batched fit's point order: bricks of 8 x 4 x 4 grid points, x fastest, bricks
    row by row, points inside a brick in the same order."""
    nx, ny, _nz = (int(v) for v in n_grid)
    f = kept.astype(np.int64)
    k, j, i = f // (nx * ny), (f // nx) % ny, f % nx
    nbx, nby = (nx + 7) // 8, (ny + 3) // 4
    brick = (i // 8) + nbx * ((j // 4) + nby * (k // 4))
    inner = (i % 8) + 8 * ((j % 4) + 4 * (k % 4))
    return np.lexsort((inner, brick))


@pytest.mark.parametrize("name,order", [("water24", "flat"), ("tricmini", "flat"), ("tricmini", "shuffled"),
                                        ("tricmini", "brick"), ("mofmini", "brick")])
def test_mixed_phi_parts_match_oracle(name, order, gpu_ctx, oracle_mod):
    """Each part of the mixed Phi against the oracle's FP64 Phi on the same kept points.
    Both parts carry FP32 rounding (the real-space terms, reciprocal stages B and C),
    so the bound is 1e-6 of max|Phi| (measured 2-4e-7).  The kernel takes the points in
    any order (the batched fit passes them brick by brick); a shuffled order gives every
    128-point tile a bounding box of the whole cell, the widest image culling."""
    import torch
    L = gpu_ctx.lib
    L.rp_debug_mixed_phi.restype = ctypes.c_int
    L.rp_debug_mixed_phi.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]
    cube, _ = load_golden(name)
    V = torch.from_numpy(cube.V).cuda()
    kept, Vc, M, _ = gpu_ctx.filter(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index, V)
    ew = gpu_ctx.ewald(cube.n_grid, cube.axis_vector, cube.cutoff, cube.kmax)
    of = oracle_mod.OracleFit(cube)
    grid = of.grid
    if order != "flat":
        perm = (np.random.default_rng(5).permutation(M) if order == "shuffled"
                else _brick_order(kept.cpu().numpy(), cube.n_grid))
        kept = kept[torch.from_numpy(perm).cuda()].contiguous()
        grid = grid[perm]
    atoms = np.ascontiguousarray(cube.atom_pos, dtype=np.float64)
    real_ref = oracle_mod.phi(grid, atoms, of.kv[:0], of.kc[:0], of.shifts, of.zero_idx, cube.cutoff)
    rec_ref = oracle_mod.phi(grid, atoms, of.kv, of.kc, of.shifts[:0], -1, cube.cutoff)
    N = len(atoms)
    for parts, ref, tol in ((1, real_ref, 1e-6), (2, rec_ref, 1e-6), (3, real_ref + rec_ref, 1e-6)):
        out = torch.zeros((N, M), dtype=torch.float64, device="cuda")
        gpu_ctx.check(L.rp_debug_mixed_phi(gpu_ctx.ptr, ew.ptr, atoms.ctypes.data, N, kept.data_ptr(), M, parts,
                                           out.data_ptr()))
        err = np.abs(out.cpu().numpy().T - ref).max() / np.abs(ref).max()
        assert err <= tol, (parts, err)
    ew.close()


def test_single_pass_clamp_falls_back_to_two_passes(gpu_ctx):
    """The batched fit scales Phi by a-priori bounds and writes its digits in one pass.
    Bounds shrunk 1000-fold make values clamp: each such cube is redone in two passes
    (centre and scale from the data), and its charges agree with the single-pass ones."""
    from pyrepeat_gb300 import _lib
    L = gpu_ctx.lib
    L.rp_debug_bound_scale.restype = ctypes.c_int
    L.rp_debug_bound_scale.argtypes = [ctypes.c_void_p, ctypes.c_double]
    L.rp_debug_last_fallbacks.restype = ctypes.c_int
    L.rp_debug_last_fallbacks.argtypes = [ctypes.c_void_p]
    cubes = [load_golden(n)[0] for n in ("water24", "tricmini")]
    q0, _, _ = gpu_ctx.fit_batch(cubes, _lib.PREC_MIXED)
    assert L.rp_debug_last_fallbacks(gpu_ctx.ptr) == 0
    assert L.rp_debug_bound_scale(gpu_ctx.ptr, 1e-3) == 0
    try:
        q1, _, _ = gpu_ctx.fit_batch(cubes, _lib.PREC_MIXED)
        fell_back = L.rp_debug_last_fallbacks(gpu_ctx.ptr)
    finally:
        L.rp_debug_bound_scale(gpu_ctx.ptr, 1.0)
    assert fell_back == len(cubes)
    for a, b in zip(q0, q1):
        assert np.abs(np.asarray(a) - np.asarray(b)).max() <= 1e-6


def test_mixed_fit_is_deterministic(gpu_ctx):
    from pyrepeat_gb300 import _lib
    cube, _ = load_golden("tricmini")
    q1 = gpu_ctx.fit_cube(cube, precision=_lib.PREC_MIXED).charges
    q2 = gpu_ctx.fit_cube(cube, precision=_lib.PREC_MIXED).charges
    assert np.array_equal(q1, q2)


def test_exact_gram_kernel_is_exact(gpu_ctx):
    """The fixed-point Gram kernel returns the exact integer sum of all slice products."""
    import torch
    L = gpu_ctx.lib
    L.rp_debug_gram_slices.restype = ctypes.c_int
    L.rp_debug_gram_slices.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                                               ctypes.c_int, ctypes.c_void_p]
    rng = np.random.default_rng(0)
    Np, cols = 200, 4096
    X = [np.zeros((256, cols), np.float16) for _ in range(4)]
    X[0][:Np] = rng.integers(-32, 33, size=(Np, cols))
    for q in (1, 2, 3):
        X[q][:Np] = rng.integers(-64, 65, size=(Np, cols))
    xd = [torch.from_numpy(a).cuda() for a in X]
    x64 = [a[:Np].astype(np.float64) for a in X]
    ref = sum((x64[a] @ x64[b].T) * 2.0 ** (7 * (6 - a - b)) for a in range(4) for b in range(4)) * 2.0 ** -54
    I = torch.zeros((Np, Np), dtype=torch.float64, device="cuda")
    for flush in (8, 16):   # 16: the product's flush period, exact at the digits' largest magnitudes
        I.zero_()
        gpu_ctx.check(L.rp_debug_gram_slices(gpu_ctx.ptr, *[x.data_ptr() for x in xd], Np, cols, flush, 16,
                                             I.data_ptr()))
        assert np.abs(I.cpu().numpy() - ref).max() <= 1e-15 * np.abs(ref).max()
    # every digit at its largest magnitude, one sign: the largest exact sums a flush can hold
    Xm = [np.zeros((256, cols), np.float16) for _ in range(4)]
    Xm[0][:Np] = 32
    for q in (1, 2, 3):
        Xm[q][:Np] = 64
    xm = [torch.from_numpy(a).cuda() for a in Xm]
    xm64 = [a[:Np].astype(np.float64) for a in Xm]
    refm = sum((xm64[a] @ xm64[b].T) * 2.0 ** (7 * (6 - a - b)) for a in range(4) for b in range(4)) * 2.0 ** -54
    I.zero_()
    gpu_ctx.check(L.rp_debug_gram_slices(gpu_ctx.ptr, *[x.data_ptr() for x in xm], Np, cols, 16, 16, I.data_ptr()))
    assert np.abs(I.cpu().numpy() - refm).max() <= 1e-15 * np.abs(refm).max()


def test_exact_gram_over_several_launches(gpu_ctx):
    """A Gram of more work units than one launch takes (one 64-point block per unit: 6 tiles x
    1024 point splits = 6144 units, cut into launches of 16 rounds of one unit per SM) gives
    bitwise the totals of 16 blocks per unit in a single launch, and both the exact sum (every
    slice product is an integer below 2^53 in FP64; the 16 scaled products are added in FP64,
    so the reference itself carries a few ulps)."""
    import torch
    L = gpu_ctx.lib
    L.rp_debug_gram_slices.restype = ctypes.c_int
    L.rp_debug_gram_slices.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_longlong, ctypes.c_int,
                                                               ctypes.c_int, ctypes.c_void_p]
    rng = np.random.default_rng(1)
    Np, cols = 200, 65536
    X = [np.zeros((256, cols), np.float16) for _ in range(4)]
    X[0][:Np] = rng.integers(-32, 33, size=(Np, cols))
    for q in (1, 2, 3):
        X[q][:Np] = rng.integers(-64, 65, size=(Np, cols))
    xd = [torch.from_numpy(a).cuda() for a in X]
    out = []
    for split in (16, 1):
        I = torch.zeros((Np, Np), dtype=torch.float64, device="cuda")
        gpu_ctx.check(L.rp_debug_gram_slices(gpu_ctx.ptr, *[x.data_ptr() for x in xd], Np, cols, 16, split,
                                             I.data_ptr()))
        out.append(I.cpu().numpy())
    assert np.array_equal(out[0], out[1])
    x64 = [torch.from_numpy(a[:Np].astype(np.float64)).cuda() for a in X]
    ref = sum((x64[a] @ x64[b].T) * 2.0 ** (7 * (6 - a - b)) for a in range(4) for b in range(4)) * 2.0 ** -54
    ref = ref.cpu().numpy()
    assert np.abs(out[1] - ref).max() <= 2e-15 * np.abs(ref).max()


def test_batch_equals_single_fits(gpu_ctx):
    """A cube's charges are the same fitted alone (rp_fit) and inside a batch
    (rp_fit_batch): bitwise.  The staged entry points (rp_filter -> rp_gram ->
    rp_solve) visit the kept points in flat instead of brick order, which changes
    the first-chunk centre in its last bits and so the 28-bit quantisation of every
    Gram input: well below 1e-6 e."""
    from pyrepeat_gb300 import _lib
    cubes = [load_golden(n)[0] for n in ("water24", "tricmini", "mofmini")]
    alone = [gpu_ctx.fit_host(c, precision=_lib.PREC_MIXED).charges for c in cubes]
    batch, M, info = gpu_ctx.fit_batch(cubes, _lib.PREC_MIXED)
    for a, b in zip(alone, batch):
        assert np.array_equal(a, b)
    for c, b in zip(cubes[:2], batch[:2]):
        staged = gpu_ctx.fit_cube(c, precision=_lib.PREC_MIXED).charges
        assert np.abs(staged - b).max() <= 1e-6


def test_pipelined_batch_equals_single_fits(gpu_ctx):
    """A batch of 64 or more cubes runs as four pipeline groups (filters, normal equations
    and solves of different groups in flight on different streams).  Every cube's charges
    equal its fit alone, bitwise, and the per-group kept counts come back in order."""
    from pyrepeat_gb300 import _lib
    names = ("water24", "tricmini", "mofmini")
    cubes = [load_golden(names[i % 3])[0] for i in range(66)]
    alone = {n: gpu_ctx.fit_host(load_golden(n)[0], precision=_lib.PREC_MIXED).charges for n in names}
    batch, M, info = gpu_ctx.fit_batch(cubes, _lib.PREC_MIXED)
    for i, (q, m) in enumerate(zip(batch, M)):
        name = names[i % 3]
        assert np.array_equal(q, alone[name]), (i, name)
        assert m == load_golden(name)[1]["kept"]


def test_potential_matches_phi_q(gpu_ctx, oracle_mod):
    """rp_potential (the stats pass) equals the oracle's Phi q at kept points."""
    import torch
    cube, _ = load_golden("tricmini")
    V = torch.from_numpy(cube.V).cuda()
    kept, Vc, M, _ = gpu_ctx.filter(cube.n_grid, cube.axis_vector, cube.atom_pos, cube.atom_index, V)
    ew = gpu_ctx.ewald(cube.n_grid, cube.axis_vector, cube.cutoff, cube.kmax)
    pot = gpu_ctx.potential(ew, cube.atom_pos, cube.charges_true, kept).cpu().numpy()
    ew.close()
    of = oracle_mod.OracleFit(cube)
    ref = of.phi() @ cube.charges_true
    assert np.abs(pot - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("N", [300, 900])
def test_bordered_solve_ill_conditioned_takes_fp64(gpu_ctx, N):
    """cond(A) = 1e10, beyond what FP32 factors can refine: the FP64 factorisation takes over
    (cuSOLVER's getrf for 256 or more unknowns, refined on the host path; one CTA below) and
    the charges match an FP64 LU of the same bordered system to cond x eps."""
    import scipy.linalg as sl
    import torch
    rng = np.random.default_rng(7 + N)
    Q, _ = np.linalg.qr(rng.normal(size=(N, N)))
    A = (Q * np.logspace(0, -10, N)) @ Q.T
    A = 0.5 * (A + A.T)
    b = rng.normal(size=N)
    q, info = gpu_ctx.solve(torch.from_numpy(A).cuda(), torch.from_numpy(b).cuda(), np.full(N, 6), qtot=0.5)
    K = np.zeros((N + 1, N + 1))
    K[:N, :N] = A
    K[:N, N] = K[N, :N] = 1.0
    rhs = np.concatenate([b, [0.5]])
    ref = sl.solve(K, rhs)[:N]
    q = q.cpu().numpy()
    assert np.abs(q - ref).max() <= 1e-4 * np.abs(ref).max()
    assert abs(q.sum() - 0.5) <= 1e-8 * np.abs(q).max()
    assert info["pivot_min"] > 0.0


@pytest.mark.parametrize("N", [61, 700, 767, 1000, 1600, 1800, 3500])
def test_bordered_solve_large_systems(gpu_ctx, N):
    """The bordered solve on systems of many panels against an FP64 LU of the same
    bordered system: the one-CTA blocked FP32 LU (N + 1 < 768) and the wide factorisation
    across the GPU (panels of 32 columns, of 16 while the panel has more than 1745 rows and
    of 8 past 3388, cuBLAS trailing updates), both with FP64 refinement (the wide systems'
    on the host path: cuBLAS DGEMV residuals and STRSV solves)."""
    import scipy.linalg as sl
    import torch
    rng = np.random.default_rng(N)
    X = rng.normal(size=(3 * N, N)) + 0.3 * rng.normal(size=(1, N))
    A = X.T @ X / (3 * N)
    b = rng.normal(size=N)
    Z = np.full(N, 6)
    q, _ = gpu_ctx.solve(torch.from_numpy(A).cuda(), torch.from_numpy(b).cuda(), Z, qtot=0.5)
    K = np.zeros((N + 1, N + 1))
    K[:N, :N] = A
    K[:N, N] = K[N, :N] = 1.0
    ref = sl.solve(K, np.concatenate([b, [0.5]]))[:N]
    q = q.cpu().numpy()
    assert np.abs(q - ref).max() <= 1e-9 * max(1.0, np.abs(ref).max())


def test_real_space_erfc_error_bound(gpu_ctx):
    """The real-space kernels' FP32 erfc (the all-range Chebyshev fit evaluated in base 2
    with the approximate reciprocal and exponential instructions) against FP64 erfc over
    the real-space range 0 <= x = sqrt(alpha) r <= pi, and against CUDA's own erfcf:
    within 1.5e-6 relative below x = 1.5 and 2.5e-6 up to pi (where the terms are ~1e-6
    of the largest), and within 2e-6 of erfcf's own error."""
    import torch
    from scipy.special import erfc
    L = gpu_ctx.lib
    L.rp_debug_erfc.restype = ctypes.c_int
    L.rp_debug_erfc.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
    x = torch.linspace(0.0, float(np.pi), 200001, dtype=torch.float32, device="cuda")
    out = torch.empty_like(x)
    assert L.rp_debug_erfc(x.data_ptr(), x.numel(), out.data_ptr()) == 0
    xs = x.cpu().numpy().astype(np.float64)
    ref = erfc(xs)
    rel = np.abs(out.cpu().numpy().astype(np.float64) / ref - 1.0)
    assert rel[xs < 1.5].max() <= 1.5e-6
    assert rel.max() <= 2.5e-6
    cuda_rel = np.abs(torch.special.erfc(x).cpu().numpy().astype(np.float64) / ref - 1.0)
    assert rel.max() <= cuda_rel.max() + 2e-6


def test_pipeline_wait_timeout_is_reported_and_the_context_recovers():
    """The Gram kernel's bounded waits: with a budget of zero every wait of the tensor-core
    pipeline gives up at once (as if it had run out), the kernel unwinds (waits for its
    own copies and MMAs, frees TMEM) and the fit returns RP_E_TIMEOUT; the same context
    then fits the cube normally, with the same charges as a fresh context."""
    from pyrepeat_gb300 import _lib
    from pyrepeat_gb300.fit import Context
    cube, _ = load_golden("water24")
    ref = Context(0)
    try:
        q_ref = np.asarray(ref.fit_batch([cube], _lib.PREC_MIXED)[0][0]).copy()
    finally:
        ref.close()
    ctx = Context(0)
    try:
        L = ctx.lib
        L.rp_debug_wait_budget.restype = ctypes.c_int
        L.rp_debug_wait_budget.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
        assert L.rp_debug_wait_budget(ctx.ptr, 0) == 0
        try:
            with pytest.raises(_lib.RepeatError) as err:
                ctx.fit_batch([cube], _lib.PREC_MIXED)
            assert err.value.code == -5
        finally:
            assert L.rp_debug_wait_budget(ctx.ptr, -1) == 0
        q = np.asarray(ctx.fit_batch([cube], _lib.PREC_MIXED)[0][0])
        assert np.array_equal(q, q_ref)
    finally:
        ctx.close()
