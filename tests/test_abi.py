"""The C-ABI library loads without a GPU and exports every declared entry point."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "sbe_gb300.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"^\s*(?:const char\*|int)\s+(sbe_\w+)\s*\(", src, re.M)))


@pytest.fixture(scope="module")
def lib_path():
    from pulsesuite_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.LIB_PATH


def test_header_matches_binding_list():
    from pulsesuite_gb300 import _lib
    assert _declared() == sorted(_lib.EXPORTS)


def test_library_exports_all_symbols(lib_path):
    lib = ctypes.CDLL(lib_path)
    for name in _declared():
        assert hasattr(lib, name), name


def test_constants_and_errors_without_gpu(lib_path):
    from pulsesuite_gb300 import _lib
    from pulsesuite_gb300.constants import E0, EPS0, HBAR, KB, ME0
    lib = _lib.load(lib_path)
    out = (ctypes.c_double * 5)()
    assert lib.sbe_constants(out) == 0
    assert list(out) == [HBAR, E0, EPS0, ME0, KB]
    # host-side argument checks return an error code instead of touching the device
    assert lib.sbe_constants(None) == 1
    assert b"null" in lib.sbe_last_error()
    assert lib.sbe_dpdt(0, None, None, None, None, None, None, None, None, None, None, None) == 1
    assert lib.sbe_ctx_create(None, 0, None, None) == 1


def test_new_entry_points_check_arguments_without_gpu(lib_path):
    """DC, statistics, backup and coupling entry points reject bad arguments on the
    host, before any device call."""
    from pulsesuite_gb300 import _lib
    lib = _lib.load(lib_path)
    assert lib.sbe_wire_info(None, 0, None, None, None, None, None, None, None) == 1
    assert b"bad context" in lib.sbe_last_error()
    assert lib.sbe_calc_jfx(-1, None, None, 1.0, 1.0, None, None) == 1
    assert lib.sbe_calc_jfx(4, None, None, 1.0, 1.0, None, None) == 1
    assert lib.sbe_calc_jfx(0, None, None, 1.0, 1.0, None, None) == 0     # nothing to do
    assert lib.sbe_qw_placement(2, 2, 2, None, None, None, None, None, None) == 1
    assert lib.sbe_e_at_xyz(None, None, 0, None, 1, None, 1, None, 0, None, None) == 1
    assert lib.sbe_backup_format(None, 3, None, 0, None, 0) == 1
    n = ctypes.c_longlong(-1)
    assert lib.sbe_backup_format(None, 0, None, 0, ctypes.byref(n), 0) == 0 and n.value == 0
    assert lib.sbe_backup_parse(None, 0, None, 0, 0) == 0


def _declared_params():
    """name -> parameter kinds of every declaration in the header ('ptr', 'double',
    'i64', 'int'), comments removed; a (void) list is empty."""
    with open(os.path.join(ROOT, "include", "sbe_gb300.h")) as f:
        src = re.sub(r"/\*.*?\*/", " ", f.read(), flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*(?:const char\*|int)\s+(sbe_\w+)\s*\(([^;]*?)\)\s*;", src, re.M | re.S):
        params = [p.strip() for p in m.group(2).split(",")]
        if params == ["void"] or params == [""]:
            params = []
        kinds = []
        for p in params:
            if "*" in p:
                kinds.append("ptr")
            elif "double" in p:
                kinds.append("double")
            elif "long long" in p:
                kinds.append("i64")
            elif "int" in p:
                kinds.append("int")
            else:
                raise AssertionError(f"unclassified parameter {p!r} of {m.group(1)}")
        out[m.group(1)] = kinds
    return out


def test_binding_signatures_match_header(lib_path):
    """Every ctypes signature in the binding has the header's parameter count and kinds
    (pointer, double, 64-bit or 32-bit integer): a drift between the two would pass
    arguments in the wrong registers."""
    from pulsesuite_gb300 import _lib
    lib = _lib.load(lib_path)
    kind = {ctypes.c_void_p: "ptr", ctypes.c_char_p: "ptr", ctypes.c_double: "double",
            ctypes.c_longlong: "i64", ctypes.c_int: "int"}
    decl = _declared_params()
    assert sorted(decl) == _declared()
    for name, params in decl.items():
        f = getattr(lib, name)
        if f.argtypes is None:
            assert params == [], f"{name}: no binding signature for {len(params)} parameters"
            continue
        assert [kind[t] for t in f.argtypes] == params, name


def test_descriptor_structs_match_the_header(tmp_path):
    """The ctypes descriptor structures have the C structs' size and field offsets
    (gcc compiles offsetof() of every field against the header)."""
    import shutil
    import subprocess
    from pulsesuite_gb300 import _lib
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    structs = [_lib.SbeWireDesc, _lib.SbePstdDesc, _lib.SbePstd3Desc, _lib.SbeCoupleDesc,
               _lib.SbeCouple3Desc]
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sbe_gb300.h"',
             'int main(void) {']
    for st in structs:
        n = st.__name__
        lines.append(f'  printf("{n} size %zu\\n", sizeof({n}));')
        for fname, _ in st._fields_:
            lines.append(f'  printf("{n} {fname} %zu\\n", offsetof({n}, {fname}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n"):
        if ln.strip():
            a, b, c = ln.split()
            got[(a, b)] = int(c)
    for st in structs:
        n = st.__name__
        assert got[(n, "size")] == ctypes.sizeof(st), n
        for fname, _ in st._fields_:
            assert got[(n, fname)] == getattr(st, fname).offset, f"{n}.{fname}"
