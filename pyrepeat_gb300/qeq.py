"""QEq parameters: the per-element table and the lookup rules of repeat.py.

Two uses, both per element symbol (Hartree units):

* ``restraint_table`` — the QEq restraint of the REPEAT fit (``_apply_qeq``,
  repeat.py:2522-2535), applied when a ``--qeq-file`` parsed to at least one entry
  and no RESP file did: A_ii += hardness, b_i += electronegativity for every atom
  whose element is in the file, else in the default table; other atoms are left
  alone.  The device solve takes a diagonal restraint as (s, t) with A_ii += s and
  b_i += s*t, so the restraint is passed as s = hardness, t = chi / hardness.
* ``charge_parameters`` — chi and the idempotential J_ii = 2 x hardness of
  ``compute_qeq_charges`` (repeat.py:2553-2573): the file first, then the parameter
  set (the default table, or a caller's set, which also selects the EQeq hydrogen
  rule), else chi 0.15 / J_ii 0.50 with a warning.

``DEFAULT_QEQ_PARAMS`` holds the same numbers as repeat.py:617-650 (chi, hardness =
J_0 / 2, Hartree): the charges and the restrained fit depend on them, so they have
to be the reference's values.
"""
from __future__ import annotations

from .constants import z_to_symbol

EV_TO_HARTREE = 1.0 / 27.211386245988

# element: (chi, hardness), Hartree
DEFAULT_QEQ_PARAMS = {
    "H": (0.166401, 0.255225), "He": (0.449802, 0.899603), "Li": (0.110466, 0.175364),
    "Be": (0.179222, 0.326547), "B": (0.149493, 0.310892), "C": (0.199590, 0.215240),
    "N": (0.245778, 0.243355), "O": (0.320234, 0.314869), "F": (0.235784, 0.409058),
    "Ne": (0.396149, 0.792298), "Na": (0.104476, 0.168749), "Mg": (0.145193, 0.271424),
    "Al": (0.111752, 0.216449), "Si": (0.153168, 0.256284), "P": (0.200757, 0.293988),
    "S": (0.254594, 0.329707), "Cl": (0.213918, 0.267278), "Ar": (0.289578, 0.579156),
    "K": (0.088968, 0.141114), "Ca": (0.118734, 0.211671), "Sc": (0.135014, 0.151110),
    "Ti": (0.142033, 0.166471), "V": (0.150415, 0.154972), "Cr": (0.136447, 0.223945),
    "Mn": (0.169778, 0.182273), "Fe": (0.152763, 0.229605), "Co": (0.156402, 0.233353),
    "Ni": (0.161252, 0.237542), "Cu": (0.199512, 0.127447), "Zn": (0.136010, 0.164010),
    "Ga": (0.110209, 0.220564), "Ge": (0.148868, 0.252683), "As": (0.190651, 0.279950),
    "Se": (0.236219, 0.303616), "Br": (0.209178, 0.321925), "Kr": (0.257239, 0.514479),
    "Rb": (0.085661, 0.135675), "Sr": (0.111127, 0.179333), "Y": (0.144017, 0.165515),
    "Zr": (0.141408, 0.208143), "Nb": (0.141004, 0.216375), "Mo": (0.144164, 0.233500),
    "Tc": (0.153425, 0.236293), "Ru": (0.154711, 0.232250), "Rh": (0.158349, 0.233132),
    "Pd": (0.166618, 0.222475), "Ag": (0.163016, 0.230340), "Cd": (0.184992, 0.290828),
    "In": (0.110135, 0.205057), "Sn": (0.146516, 0.229605), "Sb": (0.180031, 0.245627),
    "Te": (0.213729, 0.259150), "I": (0.199586, 0.210207), "Xe": (0.222696, 0.445392),
    "Cs": (0.080222, 0.125753), "Ba": (0.103410, 0.176099), "La": (0.113553, 0.163898),
    "Ce": (0.113920, 0.161693), "Pr": (0.113920, 0.161693), "Nd": (0.113920, 0.161693),
    "Pm": (0.113920, 0.161693), "Sm": (0.113920, 0.161693), "Eu": (0.113920, 0.161693),
    "Gd": (0.113920, 0.161693), "Th": (0.113920, 0.161693),
}

# EQeq hydrogen (repeat.py:2555-2563): ionisation energy 13.598 eV, electron affinity -2 eV
_H_I1, _H_I0 = 13.598, -2.0


def read_qeq_file(path) -> dict:
    """``element electroneg hardness`` per line (repeat.py:1906-1918): lines with fewer
    than three fields are skipped; any unreadable line makes the whole table empty, as
    the reference's parser does."""
    out = {}
    try:
        with open(path) as f:
            for line in f:
                p = line.split()
                if len(p) >= 3:
                    out[p[0]] = {"electroneg": float(p[1]), "hardness": float(p[2])}
    except Exception:  # noqa: BLE001 - the reference returns an empty table on any error
        return {}
    return out


def restraint_table(Z, qeq_data) -> dict:
    """{element: (s, t)} for the device's diagonal restraint, one entry per element of Z
    that the file or the default table covers."""
    out = {}
    for z in Z:
        sym = z_to_symbol(int(z))
        if sym in out:
            continue
        if qeq_data and sym in qeq_data:
            chi, hard = qeq_data[sym]["electroneg"], qeq_data[sym]["hardness"]
        elif sym in DEFAULT_QEQ_PARAMS:
            chi, hard = DEFAULT_QEQ_PARAMS[sym]
        else:
            continue
        if hard == 0.0:
            if chi != 0.0:
                raise ValueError(f"QEq restraint for {sym}: hardness 0 with electronegativity {chi} "
                                 "shifts only the right-hand side, which the diagonal restraint cannot carry")
            continue
        out[sym] = (float(hard), float(chi) / float(hard))
    return out


def charge_parameters(Z, qeq_data=None, param_set=None):
    """(chi [N], J_ii [N], method name, symbols without parameters) for QEq charges."""
    import numpy as np
    method = "QEq" if param_set is None else "EQeq"
    table = DEFAULT_QEQ_PARAMS if param_set is None else param_set
    chi = np.zeros(len(Z))
    jself = np.zeros(len(Z))
    missing = []
    for i, z in enumerate(Z):
        sym = z_to_symbol(int(z))
        if sym == "H" and method == "EQeq":
            chi[i] = 0.5 * (_H_I1 + _H_I0) * EV_TO_HARTREE
            jself[i] = (_H_I1 - _H_I0) * EV_TO_HARTREE
        elif qeq_data and sym in qeq_data:
            chi[i] = qeq_data[sym]["electroneg"]
            jself[i] = 2.0 * qeq_data[sym]["hardness"]
        elif sym in table:
            c, h = table[sym]
            chi[i] = c
            jself[i] = 2.0 * h
        else:
            chi[i] = 0.15
            jself[i] = 0.50
            missing.append(sym)
    return chi, jself, method, missing
