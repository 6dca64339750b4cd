"""Backup files of the state (SBEs.py:5524-5569 write_sbes_data / read_sbes_data)
through the library's host-side writer and reader: byte-identical to the reference's
files and values read back as the reference reads them.  No GPU needed."""

import numpy as np
import pytest

from tests.conftest import golden

KEYS = ("CC1", "CC2", "CC3", "DD1", "DD2", "DD3", "YY1", "YY2", "YY3")


@pytest.fixture(scope="module")
def lib():
    from pulsesuite_gb300 import _lib, build
    build.build()
    return _lib


def _file_order(arr):
    """(Nk, Nk, Nw) level -> the file's element order: per wire, k2 outer, k1 inner."""
    return np.transpose(arr, (2, 1, 0)).reshape(-1)


def _bits(z):
    return np.ascontiguousarray(z).view(np.int64)


@pytest.mark.parametrize("threads", [1, 3, 0])
def test_write_matches_reference_files(lib, threads):
    g = golden("backup_nk6")
    for k in KEYS:
        text = bytes(lib.backup_format(_file_order(g["arr_" + k]), threads))
        assert text == bytes(g["txt_" + k]), k


@pytest.mark.parametrize("threads", [1, 4])
def test_read_matches_reference_reader(lib, threads):
    g = golden("backup_nk6")
    nk, nw = int(g["nk"]), int(g["nw"])
    for k in KEYS:
        vals = lib.backup_parse(bytes(g["txt_" + k]), nk * nk * nw, threads)
        assert np.array_equal(_bits(vals), _bits(_file_order(g["back_" + k]))), k


def test_format_is_python_repr(lib):
    """Every number as f"{np.float64}" prints it, over the whole float64 range."""
    rng = np.random.default_rng(0)
    n = 200000
    bits = rng.integers(0, 2 ** 63, size=2 * n, dtype=np.int64)
    bits[: n // 2] &= ~(0x7FF << 52)          # subnormals and zeros
    v = bits.view(np.float64)
    v[v != v] = 1.5                           # random NaN payloads aside (repr is "nan")
    extra = [0.0, -0.0, 1e16, 1e15, 9999999999999998.0, 1e-4, 1e-5, 0.1, 5e-324, np.inf,
             -np.inf, np.nan, 1.7976931348623157e308, 2.0 ** 63, 123.0, -1e-300]
    v[: len(extra)] = extra
    z = np.empty(n, dtype=complex)
    z.real = v[0::2]
    z.imag = v[1::2]
    text = bytes(lib.backup_format(z, 0)).decode()
    want = "".join(f"{np.real(x)} {np.imag(x)}\n" for x in z)
    assert text == want


def test_parse_spellings_and_errors(lib):
    text = b"+1.5 -2e3 tail\r\n  0.25\t1e-400\ninf -2\n-0.0 -inf\n-0.0 0.0\n"
    vals = lib.backup_parse(text, 5)
    # what read_sbes_data stores for each line: float(re) + 1j * float(im)
    want = np.array([float(a) + 1j * float(b)
                     for a, b, *_ in (ln.split() for ln in text.decode().splitlines())])
    assert np.array_equal(_bits(vals), _bits(want))
    assert lib.backup_parse(b"1 2\n3 4", 2)[1] == 3 + 4j       # last line without newline
    with pytest.raises(lib.SbeError, match="lines"):
        lib.backup_parse(b"1 2\n", 2)
    with pytest.raises(lib.SbeError, match="line 2"):
        lib.backup_parse(b"1 2\n3\n5 6\n", 3)
    with pytest.raises(lib.SbeError, match="line 1"):
        lib.backup_parse(b"1x 2\n", 1)


ODD_TOKENS = ["+-1", "-+1", "--1", "++1", "1_0", "1__0", "_1", "1_", "1_.5", "1._5", "1.5_",
              "1e1_0", "1e_10", "1_0e-1_1", ".5", "5.", ".", "-.", "1.e5", ".e5", "e5", "1e",
              "1e+", "INF", "-Infinity", "+nan", "-NaN", "nan(1)", "infin", "infinityx",
              "0x1p3", "1.5x", "0_0.0_0", "00012", "1e400", "-1e-400", "1E5", "+.5e-3"]


@pytest.mark.parametrize("tok", ODD_TOKENS)
def test_parse_accepts_what_python_float_accepts(lib, tok):
    """read_sbes_data reads each number with Python float(): every odd ASCII spelling
    is accepted or refused as float() does, with the same value when accepted (float()
    also takes non-ASCII decimal digits, which the library's reader refuses)."""
    text = f"{tok} 2\n".encode()
    try:
        want = float(tok)
    except ValueError:
        with pytest.raises(lib.SbeError, match="line 1"):
            lib.backup_parse(text, 1)
        return
    got = lib.backup_parse(text, 1)[0]
    w = want + 2j
    if np.isnan(want):
        assert np.isnan(got.real) and got.imag == 2.0
    else:
        assert _bits(np.array([got])).tolist() == _bits(np.array([w])).tolist()


def test_large_level_round_trip(lib):
    """A 32-wire Nk = 256 level: threaded write then read gives the values back."""
    rng = np.random.default_rng(1)
    z = rng.standard_normal(32 * 256 * 256) * 1e-3 + 1j * rng.standard_normal(32 * 256 * 256)
    text = lib.backup_format(z, 0)
    back = lib.backup_parse(text, z.size, 0)
    assert np.array_equal(back, z)
