"""The reference-compatible command line (python -m pyrepeat_gb300).

CPU: flag handling and the refusals (device lists, a missing cube).
GPU: the whole program on a golden cube written as a Gaussian cube file, with
symmetry and RESP files: printed charges against the reference's (1e-5 e), the
--output file (x y z V_coul V_qm per kept point) and the RMS against the oracle."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, load_golden
from pyrepeat_gb300 import __main__ as cli, synth


def test_flags_match_the_reference():
    p = cli.build_parser()
    opts = {a.dest for a in p._actions}
    for dest in ("cube_file", "fit_type", "vdw_factor", "vdw_max", "cutoff", "total_charge", "symm_file",
                 "resp_file", "qeq_file", "cores", "block_k", "no_jit", "gpu", "fp64", "output", "charge",
                 "stats"):
        assert dest in opts
    a = p.parse_args(["x.cube", "--gpu"])
    assert a.gpu == "0" and a.cutoff == 20.0 and a.vdw_max == 1000.0 and a.kmax == 7


def test_root_command_is_the_same_program():
    r = subprocess.run([sys.executable, "repeat_gb300.py", "--help"], cwd=ROOT, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0 and "--fit-type" in r.stdout and "--qeq-file" in r.stdout


def test_device_lists_refused():
    assert cli.parse_device(None) == 0 and cli.parse_device("3") == 3
    for spec in ("0,1", "all", "x"):
        with pytest.raises(SystemExit):
            cli.parse_device(spec)


def test_missing_cube_exits_with_message(capsys):
    assert cli.main([os.path.join(ROOT, "no_such.cube")]) == 1
    assert cli.main([os.path.join(ROOT, "no_such.cube"), "--fit-type", "0"]) == 1
    assert cli.main([os.path.join(ROOT, "no_such.cube"), "--charge", "qeq"]) == 1
    out = capsys.readouterr().out
    assert out.count("not found") == 3


@pytest.mark.gpu
def test_cli_end_to_end(tmp_path, oracle_mod):
    cube, g = load_golden("tricmini")
    cf = os.path.join(tmp_path, "t.cube")
    sf = os.path.join(tmp_path, "s.txt")
    rf = os.path.join(tmp_path, "r.txt")
    of = os.path.join(tmp_path, "esp.txt")
    synth.write_cube(cf, cube)
    synth.write_symmetry_file(sf, cube.symm_groups)
    synth.write_resp_file(rf, cube.resp)
    cmd = [sys.executable, "-m", "pyrepeat_gb300", cf, "--gpu", "0", "--total-charge", str(cube.total_charge),
           "--symm-file", sf, "--resp-file", rf, "--kmax", str(cube.kmax), "--output", of]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = re.findall(r"^\s*(\d+)\s+([A-Z][a-z]?)\s+(-?\d+\.\d+)\s*$", r.stdout, re.M)
    q = np.array([float(x[2]) for x in rows])
    assert len(q) == cube.n_atoms
    assert np.abs(q - g["q_ref"]).max() <= 1e-5 + 5e-7          # printed with 6 decimals
    rms = float(re.search(r"RMS error: (\S+)", r.stdout).group(1))
    out = np.loadtxt(of)
    assert out.shape == (g["kept"], 5)
    of_ = oracle_mod.OracleFit(cube)
    assert np.allclose(out[:, :3], of_.grid, atol=5e-7)
    assert np.allclose(out[:, 4], of_.Vc, atol=1e-7)
    vcoul = of_.phi() @ g["q_ref"]
    d = (vcoul - vcoul.mean()) - (of_.Vc - of_.Vc.mean())
    assert abs(rms - np.sqrt((d * d).mean())) <= 1e-3 * rms + 1e-9


@pytest.mark.gpu
def test_cli_nonperiodic_end_to_end(tmp_path):
    """--fit-type 0 through the whole program: printed charges against repeat.py's."""
    from conftest import load_nonperiodic
    cube, q0 = load_nonperiodic("tricmini")
    cf = os.path.join(tmp_path, "t.cube")
    sf = os.path.join(tmp_path, "s.txt")
    synth.write_cube(cf, cube)
    synth.write_symmetry_file(sf, cube.symm_groups)
    cmd = [sys.executable, "-m", "pyrepeat_gb300", cf, "--gpu", "0", "--fit-type", "0", "--symm-file", sf,
           "--total-charge", str(cube.total_charge)]
    if cube.resp:
        rf = os.path.join(tmp_path, "r.txt")
        synth.write_resp_file(rf, cube.resp)
        cmd += ["--resp-file", rf]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = re.findall(r"^\s*(\d+)\s+([A-Z][a-z]?)\s+(-?\d+\.\d+)\s*$", r.stdout, re.M)
    q = np.array([float(x[2]) for x in rows])
    assert len(q) == cube.n_atoms
    assert np.abs(q - q0).max() <= 1e-5 + 5e-7
