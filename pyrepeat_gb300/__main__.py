"""Command line of the GB300 periodic REPEAT fit: ``python -m pyrepeat_gb300``.

Keeps every flag of repeat.py's ``main()`` (repeat.py:2654-2674) and its stdout and
``--output`` formats (repeat.py:2745-2789), so scripts written for the reference's
``--gpu`` path run unchanged:

    python -m pyrepeat_gb300 X.cube --gpu --total-charge 0 --symm-file s.txt --output esp.txt

Differences, all explicit: the fit always runs on the GPU (there is no CPU path;
without a CUDA device the command fails); ``--gpu`` takes one device id (a list
such as ``0,1`` is rejected: one fit uses one GPU); ``--fp64`` selects the plain
FP64 fit instead of the mixed-precision one; ``--kmax`` (new, default 7, the
reference's KMAX) sets the k-space cutoff; ``--cores``, ``--block-k`` and
``--no-jit`` steer the reference's CPU backends and are accepted without effect;
``--fit-type 0`` fits the non-periodic 1/r basis (the same filter, normal
equations and constraints, no Ewald sum); ``--qeq-file`` restrains the fit as the
reference does when no RESP file is given; ``--charge qeq`` prints (and with
``--output`` writes) QEq charges, with the Coulomb matrix and the solve on the GPU.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np


def build_parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="python -m pyrepeat_gb300",
                                description="REPEAT charges from a periodic ESP cube on a GB300 GPU")
    p.add_argument("cube_file", nargs="?", default=None)
    p.add_argument("--fit-type", type=int, default=1, choices=[0, 1])
    p.add_argument("--vdw-factor", type=float, default=1.0)
    p.add_argument("--vdw-max", type=float, default=1000.0)
    p.add_argument("--cutoff", type=float, default=20.0)
    p.add_argument("--total-charge", type=float, default=0.0)
    p.add_argument("--symm-file", type=str, default=None)
    p.add_argument("--resp-file", type=str, default=None)
    p.add_argument("--qeq-file", type=str, default=None)
    p.add_argument("--cores", type=int, default=None, help="accepted for compatibility (no effect)")
    p.add_argument("--block-k", type=int, default=64, help="accepted for compatibility (no effect)")
    p.add_argument("--no-jit", action="store_true", help="accepted for compatibility (no effect)")
    p.add_argument("--gpu", nargs="?", const="0", default=None, help="CUDA device id (default 0)")
    p.add_argument("--fp64", action="store_true", help="plain FP64 fit instead of the mixed-precision one")
    p.add_argument("--kmax", type=int, default=7, help="k-space cutoff KMAX (the reference's default is 7)")
    p.add_argument("--output", type=str, default=None)
    p.add_argument("--charge", type=str, default="repeat", choices=["repeat", "qeq"])
    p.add_argument("--stats", action="store_true", default=False)
    return p


def parse_device(spec: str | None) -> int:
    """'--gpu' value -> one device id.  Lists and 'all' are refused: one fit, one GPU."""
    if spec is None:
        return 0
    s = str(spec).strip().lower()
    if s == "all" or "," in s:
        raise SystemExit(f"Error: --gpu {spec}: one fit runs on one GPU; give one device id (e.g. --gpu 0)")
    try:
        return int(s)
    except ValueError:
        raise SystemExit(f"Error: --gpu {spec}: not a device id")


def main(argv=None) -> int:
    args = build_parser().parse_args(argv)
    device = parse_device(args.gpu)
    from .calculator import ChargeCalculator
    from .constants import ATOM_SYMBOLS

    print("=" * 60)
    print("REPEAT - GB300")
    print("=" * 60)
    print(f"Python: {sys.version.split()[0]}")
    print(f"GPU: device {device} [{'fp64' if args.fp64 else 'mixed'}]")
    print("=" * 60)
    if (not args.cube_file) or (not os.path.exists(args.cube_file)):
        print(f"Error: Cube file '{args.cube_file}' not found!")
        return 1

    calc = ChargeCalculator(cube_file=args.cube_file, fit_flag=args.fit_type, vdw_factor=args.vdw_factor,
                            vdw_max=args.vdw_max, R_cutoff=args.cutoff, q_tot=args.total_charge,
                            symm_file=args.symm_file, resp_file=args.resp_file, qeq_file=args.qeq_file,
                            n_cores=args.cores, block_k=args.block_k, use_jit=not args.no_jit, device=device,
                            fp64=args.fp64, kmax=args.kmax)
    if args.charge == "qeq":
        print("\n========================================")
        print("Using QEq (Charge Equilibration) method")
        print("========================================")
        charges = calc.compute_qeq_charges()
        print("\nQEq Charges:")
        for i, q in enumerate(charges):
            z = int(calc.cube["atom_index"][i])
            sym = ATOM_SYMBOLS[z] if z < len(ATOM_SYMBOLS) else "X"
            print(f"{i + 1:4d} {sym:2s} {q:12.6f}")
        print(f"\nTotal charge: {np.sum(charges):.6f}")
        if args.output:
            with open(args.output, "w") as f:
                for i, q in enumerate(charges):
                    z = int(calc.cube["atom_index"][i])
                    sym = ATOM_SYMBOLS[z] if z < len(ATOM_SYMBOLS) else "X"
                    pos = calc.cube["atom_pos"][i]
                    f.write(f"{i + 1:4d} {sym:2s} {pos[0]:12.6f} {pos[1]:12.6f} {pos[2]:12.6f} {q:12.6f}\n")
            print(f"QEq charges written to {args.output}")
        return 0
    print("\n========================================")
    print("Using REPEAT method (Streaming)")
    print("========================================")
    charges = calc.fit_charges()
    stats = None
    if args.stats or args.output:
        print("\nComputing statistics...")
        stats = calc.compute_stats(charges, need_v_coul=args.output is not None)
    print("\nREPEAT Charges:")
    for i, q in enumerate(charges):
        z = int(calc.cube["atom_index"][i])
        sym = ATOM_SYMBOLS[z] if z < len(ATOM_SYMBOLS) else "X"
        print(f"{i + 1:4d} {sym:2s} {q:12.6f}")
    print(f"\nTotal charge: {np.sum(charges):.6f}")
    if stats is not None:
        print(f"RMS error: {stats['rms_error']:.6e}")
    if args.output:
        with open(args.output, "w") as f:
            for g, v_qm, v_coul in zip(calc.grid_pos, calc.V_pot, stats["V_coul"]):
                f.write(f"{g[0]:12.6f} {g[1]:12.6f} {g[2]:12.6f} {v_coul:16.8e} {v_qm:16.8e}\n")
        print(f"Output written to {args.output}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
