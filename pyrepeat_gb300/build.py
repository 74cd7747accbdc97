"""In-tree build of the native parts.

* ``librepeat_gb300.so``  the CUDA kernels behind the C ABI (``include/repeat_gb300.h``),
  compiled by nvcc for sm_103a only.
* ``_synth_host.so``      host helper of the synthetic-cube generator (gcc, pthreads).
* ``_cube_io.so``         parallel parser of cube / LOCPOT value blocks (gcc, pthreads).

Translation units are compiled in parallel; nothing here needs a GPU.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "librepeat_gb300.so")
SYNTH_PATH = os.path.join(HERE, "_synth_host.so")
CUBE_IO_PATH = os.path.join(HERE, "_cube_io.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = [
    "rp_capi.cu",
    "filter.cu",
    "ewald_tables.cu",
    "phi_fp64.cu",
    "recip_sep.cu",
    "gram_mixed.cu",
    "solve.cu",
    "potential.cu",
    "qeq.cu",
]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _stale(target, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_host_helpers(force: bool = False) -> str:
    src = os.path.join(CSRC, "synth_host.c")
    if force or _stale(SYNTH_PATH, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-o", SYNTH_PATH, src, "-lm", "-lpthread"])
    src = os.path.join(CSRC, "cube_io.c")
    if force or _stale(CUBE_IO_PATH, [src]):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-o", CUBE_IO_PATH, src, "-lpthread"])
    return SYNTH_PATH


def build_cuda(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> str:
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    objs, jobs = [], []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD_DIR, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                if o.strip():
                    print(o)
    if force or jobs or _stale(LIB_PATH, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB_PATH, *objs, "-lcublas", "-lcusolver", "-lcuda"])
    return LIB_PATH


def build_all(force: bool = False, verbose: bool = False) -> None:
    build_host_helpers(force)
    build_cuda(force, verbose)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose=True)
