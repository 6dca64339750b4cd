"""sbe_prop2qw_noalloc (static-scratch Prop2QW) against sbe_prop2qw, through the C ABI.

The entry point exists for callers that must not allocate device memory (a host code
whose own pool owns the device memory, or a loop that must not take the allocator's
lock), so besides its values the tests check that it allocates nothing: the high-water
mark of the device's default memory pool (where stream-ordered allocations come from)
and the free device memory are unchanged across calls.
"""

import ctypes

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


class _DefaultPool:
    """Used-memory high-water mark of the current device's default memory pool, read
    through the driver API (cuMemPoolGetAttribute, CU_MEMPOOL_ATTR_USED_MEM_HIGH)."""

    USED_MEM_CURRENT, USED_MEM_HIGH = 7, 8

    def __init__(self, torch):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), torch.cuda.current_device()) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def get(self, attr):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, attr, ctypes.byref(v)) == 0
        return v.value

    def probe_allocation(self, nbytes=1 << 20):
        """One stream-ordered allocation from the default pool and its release (what
        the check must be able to see)."""
        ptr = ctypes.c_uint64()
        assert self.cu.cuMemAllocAsync(ctypes.byref(ptr), ctypes.c_size_t(nbytes), None) == 0
        assert self.cu.cuMemFreeAsync(ptr, None) == 0
        assert self.cu.cuStreamSynchronize(None) == 0

    def reset_high(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_MEM_HIGH,
                                             ctypes.byref(zero)) == 0


@pytest.mark.gpu
def test_noalloc_allocates_nothing_and_covers_its_largest_wire():
    """Nk = 1024 (Nr = 2050, the scratch limit) on the largest grid: equal to
    sbe_prop2qw, while the default pool's high-water mark and the free device memory
    stay where they were; a stream-ordered allocation moves the mark (so the check can
    see one)."""
    torch = pytest.importorskip("torch")
    from pulsesuite_gb300.wires import WireContext, WireSpec
    spec = WireSpec(nk=1024, L=np.pi / (3e9 / 511.5), wire_index=1)
    assert spec.nr == 2050
    ctx = WireContext([spec])
    lib = ctx.lib
    RR, f4 = _grid_and_fields(torch, _lib_max_grid(), 2.5 * spec.L, seed=21)
    ref = torch.empty((4, spec.nr), dtype=torch.complex128, device="cuda")
    outs = [torch.full((4, spec.nr), complex(np.nan, np.nan), dtype=torch.complex128,
                       device="cuda") for _ in range(3)]
    _call(lib, "sbe_prop2qw_noalloc", ctx, 0, RR, f4, outs[0])   # first call in this context
    torch.cuda.synchronize()
    pool = _DefaultPool(torch)
    used0 = pool.get(_DefaultPool.USED_MEM_CURRENT)
    pool.reset_high()
    free0 = torch.cuda.mem_get_info()[0]
    for out in outs[1:]:
        _call(lib, "sbe_prop2qw_noalloc", ctx, 0, RR, f4, out)
    torch.cuda.synchronize()
    assert pool.get(_DefaultPool.USED_MEM_HIGH) <= used0
    assert torch.cuda.mem_get_info()[0] == free0
    pool.probe_allocation()
    assert pool.get(_DefaultPool.USED_MEM_HIGH) > used0
    _call(lib, "sbe_prop2qw", ctx, 0, RR, f4, ref)
    torch.cuda.synchronize()
    r = ref.cpu().numpy()
    assert np.abs(r).max() > 0
    for out in outs:
        o = out.cpu().numpy()
        assert np.isfinite(o).all()
        assert np.abs(o - r).max() <= 1e-14 * np.abs(r).max()
    ctx.close()


@pytest.mark.gpu
def test_noalloc_rejects_a_wire_beyond_the_static_scratch():
    """Nk = 1026 (Nr = 2054 > 2050) is refused before any launch."""
    torch = pytest.importorskip("torch")
    from pulsesuite_gb300.wires import WireContext, WireSpec
    spec = WireSpec(nk=1026, L=np.pi / (3e9 / 512.5), wire_index=1)
    ctx = WireContext([spec])
    lib = ctx.lib
    RR, f4 = _grid_and_fields(torch, 512, 2.5 * spec.L, seed=4)
    out = torch.zeros((4, spec.nr), dtype=torch.complex128, device="cuda")
    rc = lib.sbe_prop2qw_noalloc(ctx.handle, 0, _lib.ptr(RR), RR.numel(), _lib.ptr(f4),
                                 _lib.ptr(out), _lib.stream_handle())
    assert rc == 2
    assert b"exceeds the static scratch limit" in lib.sbe_last_error()
    torch.cuda.synchronize()
    assert not out.abs().any()
    ctx.close()


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
