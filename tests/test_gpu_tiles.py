"""Tile shapes of the mixed-precision path and their autotuner, through the C ABI.

Neither the Phi kernel's atoms per CTA nor the Gram's points per CTA changes a
result (each Phi value and each exact digit sum is the same whatever the tiling),
so fits with any table are bitwise equal to fits with the defaults."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

NAMES = ("water24", "tricmini", "batch1")


def _fit(ctx, cubes):
    from pyrepeat_gb300 import _lib
    q, M, _ = ctx.fit_batch(cubes, _lib.PREC_MIXED)
    return [np.asarray(x).copy() for x in q], M


@pytest.mark.parametrize("at,split", [(8, 4), (32, 8), (16, 16)])
def test_every_tile_shape_gives_the_same_charges(at, split, tmp_path):
    from pyrepeat_gb300 import _lib
    from pyrepeat_gb300.fit import Context
    cubes = [load_golden(n)[0] for n in NAMES]
    ctx = Context(0)
    try:
        q0, M = _fit(ctx, cubes)
        path = tmp_path / "tiles.txt"
        with open(path, "w") as f:
            for c, m in zip(cubes, M):
                f.write(f"{_lib.tile_key(c.n_atoms, int(m), c.kmax)} {at} {split}\n")
        ctx.load_tiles(str(path))
        q1, _ = _fit(ctx, cubes)
    finally:
        ctx.close()
    for a, b in zip(q0, q1):
        assert np.array_equal(a, b)


def test_autotune_writes_a_table_that_a_new_context_loads(tmp_path):
    from pyrepeat_gb300.fit import Context
    cubes = [load_golden(n)[0] for n in NAMES]
    path = str(tmp_path / "tiles.txt")
    ctx = Context(0)
    try:
        q0, _ = _fit(ctx, cubes)
        table = ctx.autotune(cubes, path)
        assert len(table) == 3                       # three buckets, each measured once
        for key, (at, split, best, default, N, M) in table.items():
            assert at in (8, 16, 32) and split in (4, 8, 16)
            assert 0 < best <= default * 1.0001
        q1, _ = _fit(ctx, cubes)
    finally:
        ctx.close()
    ctx2 = Context(0)
    try:
        ctx2.load_tiles(path)
        q2, _ = _fit(ctx2, cubes)
    finally:
        ctx2.close()
    for a, b, c in zip(q0, q1, q2):
        assert np.array_equal(a, b) and np.array_equal(a, c)
