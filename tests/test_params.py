"""The positional parameter files the drop-in reads (qw.params: SBEs.py:4978-5002,
mb.params: SBEs.py:5004-5022): one value per line, a comment after it, SI units out."""
import pytest

from pulsesuite_gb300.constants import E0, HBAR, ME0
from pulsesuite_gb300.params import (MB_KEYS, read_mb_params, read_qw_params, write_mb_params,
                                     write_qw_params)

QW_LINES = [("80e-9", "L"), ("6e-9", "Delta0"), ("1.52", "gap (eV)"), ("0.067", "me (me0)"),
            ("0.45", "mh (me0)"), ("100e-3", "HO (eV)"), ("2e12", "gam_e"), ("3e12", "gam_h"),
            ("2.5e12", "gam_eh"), ("12.9", "epsr"), ("36e-3", "Oph (eV/hbar)"),
            ("3e-3", "Gph (eV/hbar)"), ("1e5", "Edc (V/m)"), ("250", "jmax"), ("10000", "ntmax")]


def test_qw_params_units(tmp_path):
    f = tmp_path / "qw.params"
    f.write_text("".join(f"{v:<10} # {c}\n" for v, c in QW_LINES), encoding="utf-8")
    p = read_qw_params(str(f))
    assert p["L"] == 80e-9 and p["Delta0"] == 6e-9
    assert p["gap"] == 1.52 * E0
    assert p["me"] == 0.067 * ME0 and p["mh"] == 0.45 * ME0
    assert p["HO"] == 100e-3 * E0
    assert (p["gam_e"], p["gam_h"], p["gam_eh"]) == (2e12, 3e12, 2.5e12)
    assert p["epsr"] == 12.9
    assert p["Oph"] == 36e-3 * E0 / HBAR and p["Gph"] == 3e-3 * E0 / HBAR
    assert p["Edc"] == 1e5
    assert (p["jmax"], p["ntmax"]) == (250, 10000)
    assert isinstance(p["jmax"], int) and isinstance(p["ntmax"], int)


def test_qw_params_round_trip(tmp_path):
    f = tmp_path / "qw.params"
    f.write_text("".join(f"{v}  # {c}\n" for v, c in QW_LINES), encoding="utf-8")
    p = read_qw_params(str(f))
    g = tmp_path / "again.params"
    write_qw_params(str(g), p)
    q = read_qw_params(str(g))
    for k, v in p.items():
        assert q[k] == pytest.approx(v, rel=1e-15, abs=0), k


def test_mb_params_flags(tmp_path):
    bits = [1, 1, 0, 1, 1, 0, 1, 0, 1, 1, 0, 0, 0, 1, 0]
    f = tmp_path / "mb.params"
    f.write_text("".join(f"{b}          # {k}\n" for b, k in zip(bits, MB_KEYS)), encoding="utf-8")
    flags = read_mb_params(str(f))
    assert list(flags) == list(MB_KEYS)
    assert [int(flags[k]) for k in MB_KEYS] == bits
    g = tmp_path / "again.params"
    write_mb_params(str(g), flags)
    assert read_mb_params(str(g)) == flags
