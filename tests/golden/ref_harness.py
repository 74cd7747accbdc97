"""Import the reference ``repeat.py`` for fixture generation (this container only).

Two adjustments, neither of which edits the reference:

* ``scipy.spatial.erfc = scipy.special.erfc``: ``repeat.py:965`` calls
  ``spatial.erfc``, which SciPy does not have, so the NumPy (``--no-jit``) path
  raises AttributeError without this alias.
* The per-atom Phi columns and the CPU filter run on the reference's thread
  strategy (``nogil_threads``, ``repeat.py:1145-1197``, ``2049-2055``) instead
  of its forkserver/spawn process pools: the arithmetic per column and per
  layer is the same code, and process pools cannot re-import a ``__main__``
  that is not a file.

Bytecode writes are disabled so nothing is written under the reference tree.
"""
import os
import sys


def _reference_dir() -> str:
    """The reference tree: the PYREPEAT_REFERENCE environment variable (required)."""
    d = os.environ.get("PYREPEAT_REFERENCE")
    if not d or not os.path.exists(os.path.join(d, "repeat.py")):
        raise RuntimeError("set PYREPEAT_REFERENCE to the directory that holds the reference's repeat.py")
    return d


def load_reference():
    sys.dont_write_bytecode = True
    reference_dir = _reference_dir()
    import scipy.spatial
    import scipy.special
    scipy.spatial.erfc = scipy.special.erfc
    if reference_dir not in sys.path:
        sys.path.insert(0, reference_dir)
    import repeat as R  # noqa: E402
    R._NOGIL_ENABLED = True
    workers = max(1, os.cpu_count() or 1)

    def _threads(n_grid, n_atoms, use_jit=True, force_strategy=None, prefer_gpu=None):
        return "nogil_threads", workers, False, 0

    R.select_parallel_strategy = _threads
    return R
