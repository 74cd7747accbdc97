"""Drop-in command for repeat.py's --gpu path: ``python repeat_gb300.py X.cube --gpu ...``.

The same program as ``python -m pyrepeat_gb300`` (every flag of repeat.py's main(),
repeat.py:2654-2674, and its stdout and --output formats)."""
import sys

from pyrepeat_gb300.__main__ import main

if __name__ == "__main__":
    sys.exit(main())
