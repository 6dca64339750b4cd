"""1-D PSTD field grid and wires coupled to it (the field step of the path).

:class:`Pstd1D` owns the grid tables on the GPU; fields are caller-owned complex128
tensors: ``E`` = (Ey, Ez) and ``H`` = (Hz, Hy) of shape (2, nx), ``Ex`` of shape
(nx,).  :class:`CoupledLine` puts the wires of a :class:`~.wires.WireContext` at
positions on the grid and advances wires and fields together (``step`` or a CUDA
graph of one step).  Every call runs on the GPU through ``libsbe_gb300``.
"""

import ctypes
from dataclasses import dataclass

import torch

from . import _lib
from .wires import CDTYPE

C0 = 299792458.0


class Pstd1D:
    """Grid of nx points (power of two), cell dx, background epsr, absorbing
    layers of n_abc cells at both ends (mask exp(-abc_strength s^2))."""

    def __init__(self, nx, dx, epsr, n_abc=0, abc_strength=0.0, device=None):
        if not torch.cuda.is_available():
            raise _lib.SbeError("a CUDA device is required (no CPU fallback)")
        self.lib = _lib.load()
        self.nx, self.dx, self.epsr = int(nx), float(dx), float(epsr)
        self.device = torch.device(device or "cuda")
        d = _lib.SbePstdDesc(self.nx, int(n_abc), 0, 0, self.dx, self.epsr, float(abc_strength))
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.sbe_pstd_create(ctypes.byref(d), _lib.stream_handle(),
                                                ctypes.byref(h)), "sbe_pstd_create")
        self.handle = h
        self.x = torch.empty(self.nx, dtype=torch.float64, device=self.device)
        self.q = torch.empty(self.nx, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_pstd_grid(h, _lib.ptr(self.x), _lib.ptr(self.q),
                                          _lib.stream_handle()), "sbe_pstd_grid")

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.sbe_pstd_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def max_dt(self):
        """Largest stable leapfrog step: c dt pi / (sqrt(epsr) dx) <= 2."""
        return 2.0 * self.dx * self.epsr ** 0.5 / (C0 * 3.141592653589793)

    def zeros(self, ncomp=2):
        return torch.zeros((ncomp, self.nx), dtype=CDTYPE, device=self.device)

    def deriv(self, f):
        """dfdx1D (usefulsubs.py:163-185) of one (nx,) or two (2, nx) fields."""
        f = f.contiguous()
        nf = 1 if f.dim() == 1 else f.shape[0]
        out = torch.empty_like(f)
        _lib.check(self.lib.sbe_pstd_deriv(self.handle, _lib.ptr(f), nf, _lib.ptr(out),
                                           _lib.stream_handle()), "sbe_pstd_deriv")
        return out

    def update_h(self, E, H, dt):
        _lib.check(self.lib.sbe_pstd_update_h(self.handle, _lib.ptr(E), _lib.ptr(H), float(dt),
                                              _lib.stream_handle()), "sbe_pstd_update_h")

    def update_e(self, E, H, J, dt):
        _lib.check(self.lib.sbe_pstd_update_e(self.handle, _lib.ptr(E), _lib.ptr(H),
                                              _lib.ptr(J), float(dt), _lib.stream_handle()),
                   "sbe_pstd_update_e")

    def step(self, E, H, J, dt):
        _lib.check(self.lib.sbe_pstd_step(self.handle, _lib.ptr(E), _lib.ptr(H), _lib.ptr(J),
                                          float(dt), _lib.stream_handle()), "sbe_pstd_step")

    def elong(self, rho, Px):
        out = torch.empty(self.nx, dtype=CDTYPE, device=self.device)
        _lib.check(self.lib.sbe_pstd_elong(self.handle, _lib.ptr(rho), _lib.ptr(Px),
                                           _lib.ptr(out), _lib.stream_handle()), "sbe_pstd_elong")
        return out


class Pstd3D:
    """3-D grid of n = (nx, ny, nz) points (powers of two in [2, 1024]), cells
    d = (dx, dy, dz), background epsr, absorbing layers of n_abc cells per axis; fields
    are caller-owned complex128 tensors of shape (3, nx, ny, nz): E = (Ex, Ey, Ez),
    H = (Hx, Hy, Hz).  ``fp32_work``: transforms between the first and last pass in
    FP32 (the fields stay FP64)."""

    def __init__(self, n, d, epsr, n_abc=(0, 0, 0), abc_strength=0.0, fp32_work=False,
                 device=None):
        if not torch.cuda.is_available():
            raise _lib.SbeError("a CUDA device is required (no CPU fallback)")
        self.lib = _lib.load()
        self.n = tuple(int(v) for v in n)
        self.d = tuple(float(v) for v in d)
        self.epsr = float(epsr)
        self.device = torch.device(device or "cuda")
        desc = _lib.SbePstd3Desc((ctypes.c_int * 3)(*self.n),
                                 (ctypes.c_int * 3)(*[int(v) for v in n_abc]),
                                 int(bool(fp32_work)), 0, (ctypes.c_double * 3)(*self.d),
                                 self.epsr, float(abc_strength))
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.sbe_pstd3_create(ctypes.byref(desc), _lib.stream_handle(),
                                                 ctypes.byref(h)), "sbe_pstd3_create")
        self.handle = h
        self.x, self.q = [], []
        for a in range(3):
            x = torch.empty(self.n[a], dtype=torch.float64, device=self.device)
            q = torch.empty_like(x)
            _lib.check(self.lib.sbe_pstd3_grid(h, a, _lib.ptr(x), _lib.ptr(q),
                                               _lib.stream_handle()), "sbe_pstd3_grid")
            self.x.append(x)
            self.q.append(q)

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.sbe_pstd3_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def zeros(self):
        return torch.zeros((3,) + self.n, dtype=CDTYPE, device=self.device)

    def max_dt(self):
        """Largest stable leapfrog step: v dt |q|max / 2 <= 1."""
        qm = sum((3.141592653589793 / d) ** 2 for d in self.d) ** 0.5
        return 2.0 * self.epsr ** 0.5 / (C0 * qm)

    def curl(self, F):
        out = torch.empty_like(F)
        _lib.check(self.lib.sbe_pstd3_curl(self.handle, _lib.ptr(F.contiguous()), _lib.ptr(out),
                                           _lib.stream_handle()), "sbe_pstd3_curl")
        return out

    def step(self, E, H, J, dt):
        _lib.check(self.lib.sbe_pstd3_step(self.handle, _lib.ptr(E), _lib.ptr(H), _lib.ptr(J),
                                           float(dt), _lib.stream_handle()), "sbe_pstd3_step")

    def update_h(self, E, H, dt):
        """H -= dt/mu0 curl E (masked), the first half of ``step``."""
        _lib.check(self.lib.sbe_pstd3_update_h(self.handle, _lib.ptr(E), _lib.ptr(H), float(dt),
                                               _lib.stream_handle()), "sbe_pstd3_update_h")

    def update_e(self, E, H, J, dt):
        """E += dt/eps (curl H - J) (masked), the second half of ``step``."""
        _lib.check(self.lib.sbe_pstd3_update_e(self.handle, _lib.ptr(E), _lib.ptr(H), _lib.ptr(J),
                                               float(dt), _lib.stream_handle()),
                   "sbe_pstd3_update_e")

    def elong(self, rho, P, qx=None, qy=None, qz=None):
        """ElongfromRho (rhoPJ.py:703-880): returns (out10 (10, nx, ny, nz), P_k (3, ...))
        with out10 = [E_PRho x, y, z, E_P x, y, z, E_Rho x, y, z, RhoBound]; the
        wavenumber tables default to the grid's FFT-order ones."""
        q = [qq if qq is not None else self.q[a] for a, qq in enumerate((qx, qy, qz))]
        q = [torch.as_tensor(v, dtype=torch.float64, device=self.device).contiguous() for v in q]
        out = torch.empty((10,) + self.n, dtype=CDTYPE, device=self.device)
        pk = torch.empty((3,) + self.n, dtype=CDTYPE, device=self.device)
        _lib.check(self.lib.sbe_pstd3_elong(self.handle, _lib.ptr(rho.contiguous()),
                                            _lib.ptr(P.contiguous()), *[_lib.ptr(v) for v in q],
                                            _lib.ptr(out), _lib.ptr(pk), _lib.stream_handle()),
                   "sbe_pstd3_elong")
        return out, pk


@dataclass
class SheetSource:
    """Soft source: a current sheet at grid cell ``index`` launching
    E_inc(t) = E0 exp(-((t - tpeak)/tau)^2) cos(w0 (t - tpeak)) to both sides."""
    index: int
    E0: float
    tau: float
    w0: float
    tpeak: float


class _DeviceArray:
    """__cuda_array_interface__ of a float64 device buffer owned by the library."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = dict(shape=tuple(shape), typestr="<f8",
                                             data=(int(ptr), False), version=3, strides=None)


class _Graph:
    def __init__(self, lib, handle, kernels, keep):
        self.lib, self.handle, self.kernels, self._keep = lib, handle, kernels, keep

    def launch(self):
        _lib.check(self.lib.sbe_graph_launch(self.handle, _lib.stream_handle()),
                   "sbe_graph_launch")

    def close(self):
        if self.handle is not None and self.handle.value:
            self.lib.sbe_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CoupledLine:
    """Wires of ``ctx`` centred at ``wire_x`` (m) on the grid of ``pstd``."""

    def __init__(self, ctx, pstd, wire_x, source=None, t0=0.0, longitudinal=True):
        self.ctx, self.pstd, self.lib = ctx, pstd, pstd.lib
        wx = (ctypes.c_double * ctx.nw)(*[float(v) for v in wire_x])
        if source is None:
            d = _lib.SbeCoupleDesc(-1, int(bool(longitudinal)), 0, 0, 0.0, 1.0, 0.0, 0.0, float(t0))
        else:
            d = _lib.SbeCoupleDesc(int(source.index), int(bool(longitudinal)), 0, 0,
                                   float(source.E0), float(source.tau), float(source.w0),
                                   float(source.tpeak), float(t0))
        h = ctypes.c_void_p()
        _lib.check(self.lib.sbe_couple_create(ctx.handle, pstd.handle, wx, ctypes.byref(d),
                                              _lib.stream_handle(), ctypes.byref(h)),
                   "sbe_couple_create")
        self.handle = h
        ptrs = [ctypes.c_void_p() for _ in range(5)]
        _lib.check(self.lib.sbe_couple_buffers(h, *[ctypes.byref(p) for p in ptrs]),
                   "sbe_couple_buffers")
        self._ptr = dict(zip(("Ek", "src", "Pg", "rho", "J"), [p.value for p in ptrs]))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.sbe_couple_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def view(self, name):
        """Zero-copy tensor view of an internal buffer: Ek (3 total_r), src
        (5 total_r; per wire 5 x Nr, packed like WireContext.zeros_r(5)), Pg (3, nx),
        rho (nx,), J (2, nx)."""
        tr, nx = self.ctx.total_r, self.pstd.nx
        shape = dict(Ek=(3 * tr,), src=(5 * tr,), Pg=(3, nx), rho=(nx,), J=(2, nx))[name]
        raw = torch.as_tensor(_DeviceArray(self._ptr[name], shape + (2,)), device=self.pstd.device)
        return torch.view_as_complex(raw)

    def set_step(self, n):
        _lib.check(self.lib.sbe_couple_set_step(self.handle, int(n), _lib.stream_handle()),
                   "sbe_couple_set_step")

    def reset(self):
        """New run: step 0, previous grid polarisation and current cleared."""
        _lib.check(self.lib.sbe_couple_reset(self.handle, _lib.stream_handle()),
                   "sbe_couple_reset")

    def sample(self, Ex, E):
        _lib.check(self.lib.sbe_couple_sample(self.handle, _lib.ptr(Ex), _lib.ptr(E),
                                              _lib.stream_handle()), "sbe_couple_sample")

    def deposit(self):
        _lib.check(self.lib.sbe_couple_deposit(self.handle, _lib.stream_handle()),
                   "sbe_couple_deposit")

    def step(self, P, C, D, E, H, Ex, dt, precision=_lib.PREC_FP64):
        _lib.check(self.lib.sbe_couple_step(self.handle, _lib.ptr(P), _lib.ptr(C), _lib.ptr(D),
                                            _lib.ptr(E), _lib.ptr(H), _lib.ptr(Ex), float(dt),
                                            int(precision), _lib.stream_handle()),
                   "sbe_couple_step")

    def graph(self, P, C, D, E, H, Ex, dt, precision=_lib.PREC_FP64):
        """CUDA graph of one coupled step on these buffers (launch() replays it)."""
        h = ctypes.c_void_p()
        n = ctypes.c_longlong()
        _lib.check(self.lib.sbe_couple_graph_create(self.handle, _lib.ptr(P), _lib.ptr(C),
                                                    _lib.ptr(D), _lib.ptr(E), _lib.ptr(H),
                                                    _lib.ptr(Ex), float(dt), int(precision),
                                                    ctypes.byref(h), ctypes.byref(n)),
                   "sbe_couple_graph_create")
        return _Graph(self.lib, h, n.value, (P, C, D, E, H, Ex))


class CoupledGrid3:
    """Wires of ``ctx`` along the z axis of the 3-D grid ``pstd`` at positions
    ``wire_xy`` ((x, y) per wire, m), centred at z = 0 (sbe_couple3_*): the wire's
    (x, y, z) components are the grid's (z, x, y).  ``gate``: the transverse SHO gate
    length of the deposit (the reference's 5 nm); ``source``: a current sheet in the
    plane x = x[index] (a :class:`SheetSource`) along component ``pol`` with a
    Gaussian profile of waist ``waist`` (<= 0: uniform)."""

    def __init__(self, ctx, pstd, wire_xy, source=None, pol=1, waist=0.0, gate=5e-9, t0=0.0):
        self.ctx, self.pstd, self.lib = ctx, pstd, pstd.lib
        xy = [float(v) for p in wire_xy for v in p]
        wxy = (ctypes.c_double * len(xy))(*xy)
        if source is None:
            d = _lib.SbeCouple3Desc(-1, int(pol), 0, 0, 0.0, 1.0, 0.0, 0.0, float(t0),
                                    float(waist), float(gate))
        else:
            d = _lib.SbeCouple3Desc(int(source.index), int(pol), 0, 0, float(source.E0),
                                    float(source.tau), float(source.w0), float(source.tpeak),
                                    float(t0), float(waist), float(gate))
        h = ctypes.c_void_p()
        _lib.check(self.lib.sbe_couple3_create(ctx.handle, pstd.handle, wxy, ctypes.byref(d),
                                               _lib.stream_handle(), ctypes.byref(h)),
                   "sbe_couple3_create")
        self.handle = h
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        _lib.check(self.lib.sbe_couple3_buffers(h, *[ctypes.byref(p) for p in ptrs]),
                   "sbe_couple3_buffers")
        self._ptr = dict(zip(("Ek", "src", "J", "rho"), [p.value for p in ptrs]))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.sbe_couple3_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def view(self, name):
        """Zero-copy view of Ek (3 total_r), src (5 total_r), J (3, nx, ny, nz), rho."""
        tr, n = self.ctx.total_r, self.pstd.n
        shape = dict(Ek=(3 * tr,), src=(5 * tr,), J=(3,) + n, rho=n)[name]
        raw = torch.as_tensor(_DeviceArray(self._ptr[name], shape + (2,)), device=self.pstd.device)
        return torch.view_as_complex(raw)

    def reset(self):
        _lib.check(self.lib.sbe_couple3_reset(self.handle, _lib.stream_handle()),
                   "sbe_couple3_reset")

    def sample(self, E, precision=_lib.PREC_FP64):
        _lib.check(self.lib.sbe_couple3_sample(self.handle, _lib.ptr(E), int(precision),
                                               _lib.stream_handle()), "sbe_couple3_sample")

    def deposit(self, dt):
        _lib.check(self.lib.sbe_couple3_deposit(self.handle, float(dt), _lib.stream_handle()),
                   "sbe_couple3_deposit")

    def step(self, P, C, D, E, H, dt, precision=_lib.PREC_FP64):
        _lib.check(self.lib.sbe_couple3_step(self.handle, _lib.ptr(P), _lib.ptr(C), _lib.ptr(D),
                                             _lib.ptr(E), _lib.ptr(H), float(dt), int(precision),
                                             _lib.stream_handle()), "sbe_couple3_step")

    def graph(self, P, C, D, E, H, dt, precision=_lib.PREC_FP64):
        h = ctypes.c_void_p()
        n = ctypes.c_longlong()
        _lib.check(self.lib.sbe_couple3_graph_create(self.handle, _lib.ptr(P), _lib.ptr(C),
                                                     _lib.ptr(D), _lib.ptr(E), _lib.ptr(H),
                                                     float(dt), int(precision), ctypes.byref(h),
                                                     ctypes.byref(n)),
                   "sbe_couple3_graph_create")
        return _Graph(self.lib, h, n.value, (P, C, D, E, H))
