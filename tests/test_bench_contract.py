"""bench.py's CPU-side contract: the reference arm's JSON line (the reference CPU path
timed on the host, run here on a tiny sample) and the synthetic QEq cell's layout."""
import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT


def test_reference_arm_line_has_the_contract_keys():
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--n-cubes", "1",
           "--cpu-sample", "300"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env={**os.environ, "CUDA_VISIBLE_DEVICES": ""})
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "fits/s"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1


def test_qeq_cell_is_seeded_and_well_separated():
    sys.path.insert(0, ROOT)
    import bench
    a1, Z1, ng, axis = bench.qeq_cell(300, 5)
    a2, Z2, _, _ = bench.qeq_cell(300, 5)
    assert np.array_equal(a1, a2) and np.array_equal(Z1, Z2)
    L = float(axis[0, 0] * ng[0])
    assert a1.min() > 0 and a1.max() < L
    d = a1[:, None, :] - a1[None, :, :]
    d -= L * np.rint(d / L)                      # minimum image
    r = np.sqrt((d * d).sum(-1)) + np.eye(len(a1)) * 1e9
    assert r.min() > 5.0 * 0.7                   # jittered 5 Bohr lattice
