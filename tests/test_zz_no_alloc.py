"""sbe_prop2qw_noalloc (static-scratch Prop2QW) against sbe_prop2qw, through the C ABI."""

import numpy as np
import pytest

from pulsesuite_gb300 import _lib


def test_noalloc_rejects_null_context_without_gpu():
    import os
    from pulsesuite_gb300 import build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    lib = _lib.load()
    assert lib.sbe_prop2qw_noalloc(None, 0, None, 0, None, None, None) == 1
    assert b"sbe_prop2qw_noalloc" in lib.sbe_last_error()


def _grid_and_fields(torch, n_rr, half_width, seed):
    rng = np.random.default_rng(seed)
    RR = torch.tensor(np.linspace(-half_width, half_width, n_rr), dtype=torch.float64,
                      device="cuda")
    f = rng.standard_normal((4, n_rr)) + 1j * rng.standard_normal((4, n_rr))
    return RR, torch.tensor(f, dtype=torch.complex128, device="cuda")


def _call(lib, name, ctx, w, RR, f4, out):
    rc = getattr(lib, name)(ctx.handle, w, _lib.ptr(RR), RR.numel(), _lib.ptr(f4), _lib.ptr(out),
                            _lib.stream_handle())
    _lib.check(rc, name)


@pytest.mark.gpu
def test_noalloc_matches_prop2qw_twice_in_a_row():
    torch = pytest.importorskip("torch")
    from pulsesuite_gb300.wires import WireContext, WireSpec
    specs = [WireSpec(nk=32, L=50e-9, wire_index=1), WireSpec(nk=64, L=80e-9, wire_index=2)]
    ctx = WireContext(specs)
    lib = ctx.lib
    for w, n_rr in ((0, 600), (1, _lib_max_grid())):
        RR, f4 = _grid_and_fields(torch, n_rr, 2.5 * specs[w].L, seed=10 + w)
        nr = specs[w].nr
        ref = torch.empty((4, nr), dtype=torch.complex128, device="cuda")
        _call(lib, "sbe_prop2qw", ctx, w, RR, f4, ref)
        outs = []
        for _ in range(2):
            out = torch.full((4, nr), complex(np.nan, np.nan), dtype=torch.complex128,
                             device="cuda")
            _call(lib, "sbe_prop2qw_noalloc", ctx, w, RR, f4, out)
            outs.append(out)
        torch.cuda.synchronize()
        r = ref.cpu().numpy()
        assert np.abs(r).max() > 0
        for out in outs:
            o = out.cpu().numpy()
            assert np.isfinite(o).all()
            assert np.abs(o - r).max() <= 1e-14 * np.abs(r).max()
    ctx.close()


def _lib_max_grid():
    return 8192  # SBE_NOALLOC_MAX_GRID in include/sbe_gb300.h


@pytest.mark.gpu
def test_noalloc_rejects_sizes_beyond_the_static_scratch():
    torch = pytest.importorskip("torch")
    from pulsesuite_gb300.wires import WireContext, WireSpec
    ctx = WireContext([WireSpec(nk=16, L=40e-9, wire_index=1)])
    lib = ctx.lib
    RR, f4 = _grid_and_fields(torch, _lib_max_grid() + 1, 100e-9, seed=3)
    out = torch.zeros((4, 34), dtype=torch.complex128, device="cuda")
    rc = lib.sbe_prop2qw_noalloc(ctx.handle, 0, _lib.ptr(RR), RR.numel(), _lib.ptr(f4),
                                 _lib.ptr(out), _lib.stream_handle())
    assert rc == 1
    assert b"exceeds the static scratch limit" in lib.sbe_last_error()
    torch.cuda.synchronize()
    assert not out.abs().any()
    ctx.close()
