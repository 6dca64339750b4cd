"""Positional parameter files of the reference (one value per line, comment after).

qw.params: SBEs.py:4978-5002 (SBESolver._read_qw_params); mb.params: SBEs.py:5004-5022
(SBESolver._read_mb_params).  Values are returned in SI units.
"""

import os

from .constants import E0, HBAR, ME0


def _values(path):
    with open(path, "r", encoding="utf-8") as f:
        return [ln.split()[0] for ln in f if ln.strip()]


def read_qw_params(path=os.path.join("params", "qw.params")):
    v = _values(path)
    return dict(L=float(v[0]), Delta0=float(v[1]), gap=float(v[2]) * E0, me=float(v[3]) * ME0,
                mh=float(v[4]) * ME0, HO=float(v[5]) * E0, gam_e=float(v[6]), gam_h=float(v[7]),
                gam_eh=float(v[8]), epsr=float(v[9]), Oph=float(v[10]) * E0 / HBAR,
                Gph=float(v[11]) * E0 / HBAR, Edc=float(v[12]), jmax=int(v[13]),
                ntmax=int(v[14]))


MB_KEYS = ("Optics", "Excitons", "EHs", "Screened", "Phonon", "DCTrans", "LF", "FreePot",
           "DiagDph", "OffDiagDph", "Recomb", "PLSpec", "ignorewire", "Xqwparams", "LorentzDelta")


def read_mb_params(path=os.path.join("params", "mb.params")):
    v = _values(path)
    return {k: bool(int(v[i])) for i, k in enumerate(MB_KEYS)}


def write_qw_params(path, p):
    lines = [p["L"], p["Delta0"], p["gap"] / E0, p["me"] / ME0, p["mh"] / ME0, p["HO"] / E0,
             p["gam_e"], p["gam_h"], p["gam_eh"], p["epsr"], p["Oph"] * HBAR / E0,
             p["Gph"] * HBAR / E0, p.get("Edc", 0.0), p.get("jmax", 1000), p.get("ntmax", 100000)]
    with open(path, "w", encoding="utf-8") as f:
        for x in lines:
            f.write(f"{x!r}\n")


def write_mb_params(path, flags):
    with open(path, "w", encoding="utf-8") as f:
        for k in MB_KEYS:
            f.write(f"{int(bool(flags.get(k, False)))}  # {k}\n")
