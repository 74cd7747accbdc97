"""rp_solve_noalloc: the constrained bordered solve for callers that cannot
allocate device memory while they run (its scratch is a static array inside the
library).  Called through the C ABI and checked against rp_solve on the same
normal equations, on two calls in a row and on two different systems, so the
array's leftover contents from the previous call cannot leak into a result; the
overlapping-groups branch (folded on the host) is checked against rp_solve and
the oracle's reference-order fold, and a warm call leaves the device's free
memory unchanged.  This file is collected last on purpose."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the same kernel runs behind both entry points


def _normal_equations(gpu_ctx, name):
    from pyrepeat_gb300 import _lib
    cube, _ = load_golden(name)
    r = gpu_ctx.fit_cube(cube, precision=_lib.PREC_FP64, keep_normal=True)
    return cube, r.A.contiguous(), r.b.contiguous()


def _noalloc_raw(gpu_ctx, cube, A, b, q, info):
    from pyrepeat_gb300.fit import constraint_arrays, _ptr
    ng, ptr, idx, rs, rt = constraint_arrays(cube.atom_index, cube.symm_groups, cube.resp)
    return gpu_ctx.lib.rp_solve_noalloc(A.data_ptr(), b.data_ptr(), cube.n_atoms, ng, ptr.ctypes.data,
                                        idx.ctypes.data, _ptr(rs), _ptr(rt), float(cube.total_charge), q.data_ptr(),
                                        info.ctypes.data, gpu_ctx._stream())


def _noalloc(gpu_ctx, cube, A, b):
    import torch
    q = torch.empty(cube.n_atoms, dtype=torch.float64, device=A.device)
    info = np.zeros(4)
    assert _noalloc_raw(gpu_ctx, cube, A, b, q, info) == 0
    return q.cpu().numpy(), info


def test_noalloc_solve_matches_rp_solve_twice(gpu_ctx):
    for name in ("tricmini", "water24"):   # symmetry + RESP, then a plain fit
        cube, A, b = _normal_equations(gpu_ctx, name)
        q_ref, _ = gpu_ctx.solve(A, b, cube.atom_index, cube.symm_groups, cube.resp, cube.total_charge)
        q_ref = q_ref.cpu().numpy()
        for _ in range(2):
            q, info = _noalloc(gpu_ctx, cube, A, b)
            assert np.abs(q - q_ref).max() <= TOL
            assert info[0] < 1e-8
        if cube.symm_groups:
            for g in cube.symm_groups:
                assert np.ptp(q[g]) == 0.0


def test_noalloc_overlapping_groups(gpu_ctx, oracle_mod):
    """Two groups that share an atom: folded on the host in the reference's sequential
    order, then uploaded into the static array."""
    cube, A, b = _normal_equations(gpu_ctx, "water24")
    cube.symm_groups = [[1, 2], [2, 4]]
    cube.resp = {"O": (0.1, 0.0)}
    q_ref, _ = gpu_ctx.solve(A, b, cube.atom_index, cube.symm_groups, cube.resp, cube.total_charge)
    q_ref = q_ref.cpu().numpy()
    q_or, sing = oracle_mod.solve(A.cpu().numpy(), b.cpu().numpy(), cube.atom_index, cube.symm_groups, cube.resp,
                                  cube.total_charge)
    assert not sing
    for _ in range(2):
        q, info = _noalloc(gpu_ctx, cube, A, b)
        assert np.abs(q - q_ref).max() <= TOL
        assert np.abs(q - q_or).max() <= 1e-9
    assert q[1] == q[2] == q[4]


def test_noalloc_call_allocates_nothing(gpu_ctx):
    import torch
    cube, A, b = _normal_equations(gpu_ctx, "tricmini")
    q = torch.empty(cube.n_atoms, dtype=torch.float64, device=A.device)
    info = np.zeros(4)
    assert _noalloc_raw(gpu_ctx, cube, A, b, q, info) == 0   # warm: module and array loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert _noalloc_raw(gpu_ctx, cube, A, b, q, info) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_systems_beyond_its_limit(gpu_ctx):
    import torch
    N = 513
    A = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    b = torch.zeros(N, dtype=torch.float64, device="cuda")
    q = torch.zeros(N, dtype=torch.float64, device="cuda")
    rc = gpu_ctx.lib.rp_solve_noalloc(A.data_ptr(), b.data_ptr(), N, 0, None, None, None, None, 0.0, q.data_ptr(),
                                      None, gpu_ctx._stream())
    assert rc == -1
