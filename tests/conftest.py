"""Shared fixtures: golden cases produced from the reference (tests/golden/) and
the CPU oracle (oracle/, test infrastructure only)."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from pyrepeat_gb300 import synth  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests of the CUDA path")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


# generator calls that produced each golden case (tests/golden/make_golden.py)
FACTORIES = {
    "water24": lambda: synth.make_water(1, n_grid=24),
    "water72": lambda: synth.make_water(1, n_grid=72),
    "mof128k12": lambda: synth.make_mof(2),
    "mofmini": lambda: synth.make_mof(5, n_grid=40, kmax=9, L=14.0, counts=(4, 13, 24, 12)),
    "tricmini": lambda: synth.make_tric(7, n_grid=(30, 32, 34), n_atoms=40, n_groups=6, lengths=(16.0, 17.0, 18.0)),
    "batch1": lambda: synth.make_batch_item(1),
    "batch2": lambda: synth.make_batch_item(2),
}


def golden_meta():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def load_golden(name: str):
    """(cube, golden dict).  V comes from the fixture when stored, otherwise the
    seeded generator rebuilds the cube."""
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"), allow_pickle=False)
    if z["V"].size:
        ptr, idx = z["group_ptr"], z["group_idx"]
        groups = [list(map(int, idx[ptr[g]:ptr[g + 1]])) for g in range(len(ptr) - 1)] or None
        resp = json.loads(str(z["resp"])) or None
        if resp:
            resp = {k: tuple(v) for k, v in resp.items()}
        cube = synth.Cube(z["atom_index"].astype(np.int64), z["atom_pos"], z["n_grid"].astype(np.int64),
                          z["axis_vector"], z["V"], charges_true=z["charges_true"], symm_groups=groups, resp=resp,
                          kmax=int(z["kmax"]), cutoff=float(z["cutoff"]), vdw_factor=float(z["vdw_factor"]),
                          vdw_max=float(z["vdw_max"]), total_charge=float(z["total_charge"]), name=name)
    else:
        cube = FACTORIES[name]()
    g = {"q_ref": z["q_ref"], "q_bin": z["q_bin"] if z["q_bin"].size else None,
         "mask": np.unpackbits(z["mask_bits"])[: cube.n_points].astype(np.uint8),
         "atom_pos": z["atom_pos"]}
    g.update(golden_meta()[name])
    return cube, g


def load_nonperiodic(name: str):
    """(cube with KMAX 0 = the non-periodic basis, repeat.py's --fit-type 0 charges)."""
    cube, _ = load_golden(name)
    cube.kmax = 0
    z = np.load(os.path.join(GOLDEN, "nonperiodic.npz"), allow_pickle=False)
    return cube, z[f"q_ref0_{name}"]


def load_qeq():
    """repeat.py's QEq results on the small cases (tests/golden/qeq.npz), the QEq
    parameter file they used (parsed) and its text, and their total charge."""
    z = dict(np.load(os.path.join(GOLDEN, "qeq.npz"), allow_pickle=False))
    text = str(z["qeq_file"])
    qd = {}
    for line in text.splitlines():
        p = line.split()
        qd[p[0]] = {"electroneg": float(p[1]), "hardness": float(p[2])}
    return z, qd, text, float(z["qtot"])


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from pyrepeat_gb300.fit import Context
    ctx = Context(0)
    yield ctx
    ctx.close()
