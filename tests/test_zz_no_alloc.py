"""rp_solve_noalloc: the constrained bordered solve for callers that cannot
allocate device memory while they run (its scratch is a static array inside the
library).  Called through the C ABI and checked against rp_solve on the same
normal equations, on two calls in a row and on two different systems, so the
array's leftover contents from the previous call cannot leak into a result.
This file is collected last on purpose."""
import ctypes

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


def _noalloc(gpu_ctx, cube, A, b):
    import torch
    from pyrepeat_gb300.fit import constraint_arrays, _ptr
    ng, ptr, idx, rs, rt = constraint_arrays(cube.atom_index, cube.symm_groups, cube.resp)
    q = torch.empty(cube.n_atoms, dtype=torch.float64, device=A.device)
    info = np.zeros(3)
    rc = gpu_ctx.lib.rp_solve_noalloc(A.data_ptr(), b.data_ptr(), cube.n_atoms, ng, ptr.ctypes.data,
                                      idx.ctypes.data, _ptr(rs), _ptr(rt), float(cube.total_charge), q.data_ptr(),
                                      info.ctypes.data, gpu_ctx._stream())
    assert rc == 0
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


def test_noalloc_rejects_systems_beyond_its_limit(gpu_ctx):
    import torch
    N = 513
    A = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    b = torch.zeros(N, dtype=torch.float64, device="cuda")
    q = torch.zeros(N, dtype=torch.float64, device="cuda")
    rc = gpu_ctx.lib.rp_solve_noalloc(A.data_ptr(), b.data_ptr(), N, 0, None, None, None, None, 0.0, q.data_ptr(),
                                      None, gpu_ctx._stream())
    assert rc == -1
