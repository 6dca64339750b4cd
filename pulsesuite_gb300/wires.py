"""Wire descriptors and the device context that owns their tables.

A :class:`WireContext` is a batch of quantum wires (possibly of different Nk)
whose one-time tables (Coulomb V(q), Chi1D, phonon EP/HP, dephasing index maps,
e^{ikr}, window) live on the GPU.  State tensors are owned by the caller and are
packed: wire w's Nk x Nk matrix starts at element ``mat_offset[w]`` of a flat
complex128 tensor; the per-wire field / source vectors (length Nr = 2 Nk + 2)
start at ``r_offset[w]``.  The layout groups the wires by Nk (ascending; the
caller's order within one Nk), so use ``pack`` / ``pack_r`` / ``mat`` / ``rvec``
rather than concatenating per-wire blocks.
"""

import ctypes
from dataclasses import dataclass, field

import torch

from . import _lib
from .constants import E0, HBAR, ME0

CDTYPE = torch.complex128


@dataclass
class WireSpec:
    """One quantum wire in SI units (qw.params fields, SBEs.py:4978-5002)."""
    nk: int
    L: float
    Delta0: float = 5e-9
    gap: float = 1.5 * E0
    me: float = 0.07 * ME0
    mh: float = 0.45 * ME0
    HO: float = 100e-3 * E0
    gam_e: float = 1e12
    gam_h: float = 1e12
    gam_eh: float = 1e12
    epsr: float = 9.1
    Oph: float = 36e-3 * E0 / HBAR
    Gph: float = 3e-3 * E0 / HBAR
    temp: float = 77.0
    Edc: float = 0.0
    wire_index: int = 1
    flags: dict = field(default_factory=lambda: dict(
        Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
        LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False))

    def flag_bits(self):
        bits = 0
        for k, v in self.flags.items():
            if v:
                bits |= _lib.FLAG_BITS[k]
        return bits

    @property
    def nr(self):
        return 2 * self.nk + 2

    def to_c(self):
        return _lib.SbeWireDesc(self.nk, self.wire_index, self.flag_bits(), 0, self.L,
                                self.Delta0, self.gap, self.me, self.mh, self.HO, self.gam_e,
                                self.gam_h, self.gam_eh, self.epsr, self.Oph, self.Gph,
                                self.temp, self.Edc)


class RK4Graph:
    """One captured RK4 step (sbe_rk4_graph_create); launch() replays it on the
    current stream.  ``kernels`` is the number of kernel launches per step."""

    def __init__(self, ctx, P, C, D, Ek0, dEk, dt, src_out, precision):
        self.ctx = ctx
        self._keep = (P, C, D, Ek0, dEk, src_out)
        h = ctypes.c_void_p()
        n = ctypes.c_longlong()
        _lib.check(ctx.lib.sbe_rk4_graph_create(ctx.handle, _lib.ptr(P), _lib.ptr(C),
                                                _lib.ptr(D), _lib.ptr(Ek0), _lib.ptr(dEk),
                                                float(dt), int(precision), _lib.ptr(src_out),
                                                ctypes.byref(h), ctypes.byref(n)),
                   "sbe_rk4_graph_create")
        self.handle = h
        self.kernels = n.value

    def launch(self):
        _lib.check(self.ctx.lib.sbe_graph_launch(self.handle, _lib.stream_handle()),
                   "sbe_graph_launch")

    def close(self):
        if self.handle is not None and self.handle.value:
            self.ctx.lib.sbe_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


TABLES = dict(kr=0, r=1, Ee=2, Eh=3, V0=4, Chi1D=5, qeqh=6, EP=7, HP=8, window=9, maps=10,
              xexh=11, Expikr=12, scalars=13, window_k=14)


class WireContext:
    """Device tables of a batch of wires (sbe_ctx_create)."""

    def __init__(self, specs, device=None):
        if not torch.cuda.is_available():
            raise _lib.SbeError("a CUDA device is required (no CPU fallback)")
        self.lib = _lib.load()
        self.specs = list(specs)
        self.device = torch.device(device or "cuda")
        arr = (_lib.SbeWireDesc * len(self.specs))(*[s.to_c() for s in self.specs])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.sbe_ctx_create(arr, len(self.specs), _lib.stream_handle(),
                                               ctypes.byref(h)), "sbe_ctx_create")
        self.handle = h
        lay = (ctypes.c_longlong * (3 * len(self.specs)))()
        tm = ctypes.c_longlong()
        tr = ctypes.c_longlong()
        _lib.check(self.lib.sbe_ctx_layout(h, lay, ctypes.byref(tm), ctypes.byref(tr)),
                   "sbe_ctx_layout")
        self.nk = [lay[3 * w] for w in range(len(self.specs))]
        self.mat_offset = [lay[3 * w + 1] for w in range(len(self.specs))]
        self.r_offset = [lay[3 * w + 2] for w in range(len(self.specs))]
        self.total_mat = tm.value
        self.total_r = tr.value

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            self.lib.sbe_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nw(self):
        return len(self.specs)

    # ---- packed-state helpers ---------------------------------------------
    def zeros_state(self):
        return torch.zeros(self.total_mat, dtype=CDTYPE, device=self.device)

    def zeros_r(self, ncomp):
        return torch.zeros(ncomp * self.total_r, dtype=CDTYPE, device=self.device)

    def mat(self, flat, w):
        n = self.nk[w]
        o = self.mat_offset[w]
        return flat[o:o + n * n].view(n, n)

    def rvec(self, flat, w, ncomp):
        """View of wire w's ncomp x Nr block of a packed r-vector tensor."""
        nr = 2 * self.nk[w] + 2
        o = ncomp * self.r_offset[w]
        return flat[o:o + ncomp * nr].view(ncomp, nr)

    def pack(self, mats):
        """Packed state tensor of one Nk x Nk matrix per wire (caller's wire order; each
        placed at its wire's offset: the layout groups the wires by Nk)."""
        out = torch.empty(self.total_mat, dtype=CDTYPE, device=self.device)
        for w, m in enumerate(mats):
            self.mat(out, w).copy_(torch.as_tensor(m).reshape(self.nk[w], self.nk[w]))
        return out

    def pack_r(self, vecs, ncomp):
        """Packed r-vector tensor of one (ncomp, Nr) block per wire (caller's order)."""
        out = torch.empty(ncomp * self.total_r, dtype=CDTYPE, device=self.device)
        for w, v in enumerate(vecs):
            self.rvec(out, w, ncomp).copy_(torch.as_tensor(v).reshape(ncomp, -1))
        return out

    # ---- tables ------------------------------------------------------------
    def table(self, w, name):
        which = TABLES[name]
        nk = self.nk[w]
        nr = 2 * nk + 2
        shapes = {0: (nk,), 1: (nr,), 2: (nk,), 3: (nk,), 4: (3, nk), 5: (2, nk), 6: (2, nk),
                  7: (nk, nk), 8: (nk, nk), 9: (nr,), 11: (2, nk), 13: (16,)}
        if which == 10:
            t = torch.empty((6, nk, nk), dtype=torch.int32, device=self.device)
        elif which == 12:
            t = torch.empty((nk, nr), dtype=CDTYPE, device=self.device)
        elif which == 14:
            t = torch.empty((nr,), dtype=CDTYPE, device=self.device)
        else:
            t = torch.empty(shapes[which], dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_ctx_table(self.handle, w, which, _lib.ptr(t),
                                          t.numel() * t.element_size(), _lib.stream_handle()),
                   "sbe_ctx_table")
        return t

    # ---- per-wire reference building blocks ------------------------------
    def screened_arrays(self, w, ne, nh):
        nk = self.nk[w]
        VC = torch.empty((nk, nk, 3), dtype=torch.float64, device=self.device)
        E1D = torch.empty((nk, nk), dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_screened_arrays(self.handle, w, _lib.ptr(ne), _lib.ptr(nh),
                                                _lib.ptr(VC), _lib.ptr(E1D),
                                                _lib.stream_handle()), "sbe_screened_arrays")
        return VC, E1D

    def gamma(self, w, ne, nh, VC):
        nk = self.nk[w]
        ge = torch.empty(nk, dtype=torch.float64, device=self.device)
        gh = torch.empty(nk, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_gamma(self.handle, w, _lib.ptr(ne), _lib.ptr(nh), _lib.ptr(VC),
                                      _lib.ptr(ge), _lib.ptr(gh), _lib.stream_handle()),
                   "sbe_gamma")
        return ge, gh

    def offdiag(self, w, ne, nh, P, VC, g3):
        nk = self.nk[w]
        x = torch.empty((nk, nk), dtype=CDTYPE, device=self.device)
        De = torch.empty((2 * nk + 1, nk), dtype=torch.float64, device=self.device)
        Dh = torch.empty_like(De)
        g = torch.as_tensor(g3, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_offdiag(self.handle, w, _lib.ptr(ne), _lib.ptr(nh), _lib.ptr(P),
                                        _lib.ptr(VC), _lib.ptr(g), _lib.ptr(x), _lib.ptr(De),
                                        _lib.ptr(Dh), _lib.stream_handle()), "sbe_offdiag")
        return x, De, Dh

    def phonon_rates(self, w, ne, nh, VC, E1D, WinE, WoutE, WinH, WoutH):
        _lib.check(self.lib.sbe_phonon_rates(self.handle, w, _lib.ptr(ne), _lib.ptr(nh),
                                             _lib.ptr(VC), _lib.ptr(E1D), _lib.ptr(WinE),
                                             _lib.ptr(WoutE), _lib.ptr(WinH), _lib.ptr(WoutH),
                                             _lib.stream_handle()), "sbe_phonon_rates")

    def carrier_rates(self, w, ne, nh, VC, WinE, WoutE, WinH, WoutH, precision="fp64"):
        """coulomb.py:1298/1313 MBCE/MBCH: adds the carrier-carrier rates to Win/Wout
        (precision "fp64" or "mixed")."""
        prec = _lib.PREC_MIXED if precision == "mixed" else _lib.PREC_FP64
        _lib.check(self.lib.sbe_carrier_rates(self.handle, w, _lib.ptr(ne), _lib.ptr(nh),
                                              _lib.ptr(VC), _lib.ptr(WinE), _lib.ptr(WoutE),
                                              _lib.ptr(WinH), _lib.ptr(WoutH), prec,
                                              _lib.stream_handle()), "sbe_carrier_rates")

    def spont_emission(self, w, ne, nh, VC):
        """emission.py:94 SpontEmission: Rsp of wire w (needs Recomb in its flags)."""
        rsp = torch.empty(self.nk[w], dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_spont_emission(self.handle, w, _lib.ptr(ne), _lib.ptr(nh),
                                               _lib.ptr(VC), _lib.ptr(rsp),
                                               _lib.stream_handle()), "sbe_spont_emission")
        return rsp

    def wire_info(self, w, C2, D2, src, Ek, VC=None):
        """The per-step statistics of wire w (the info and EP columns of SBEs.py:5769-5809)
        as 23 numbers on the host (see sbe_wire_info)."""
        out = torch.empty(23, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_wire_info(self.handle, w, _lib.ptr(C2), _lib.ptr(D2),
                                          _lib.ptr(src), _lib.ptr(Ek), _lib.ptr(VC), _lib.ptr(out),
                                          _lib.stream_handle()), "sbe_wire_info")
        return out.cpu().numpy()

    def wire_pdote(self, w, Ek, src, P0=None):
        """sum_c sum_r (Re P_c - P0_c) Re iFFTG(E_c) of wire w (see sbe_wire_pdote):
        Ek, src the packed wire-k field and real-space sources, P0 (3, Nr) float64 or
        None."""
        out = torch.empty(1, dtype=torch.float64, device=self.device)
        p0 = None if P0 is None else P0.contiguous()
        _lib.check(self.lib.sbe_wire_pdote(self.handle, w, _lib.ptr(Ek), _lib.ptr(src),
                                           _lib.ptr(p0), _lib.ptr(out), _lib.stream_handle()),
                   "sbe_wire_pdote")
        return float(out.item())

    def deph_extrema(self, w):
        """(max Re De, min Re De, max Re Dh, min Re Dh) of wire w's last preparation."""
        out = torch.empty(4, dtype=torch.float64, device=self.device)
        _lib.check(self.lib.sbe_deph_extrema(self.handle, w, _lib.ptr(out), _lib.stream_handle()),
                   "sbe_deph_extrema")
        return out.cpu().numpy()

    def sources(self, w, P, C, D, ne, nh):
        nr = 2 * self.nk[w] + 2
        out = [torch.empty(nr, dtype=CDTYPE, device=self.device) for _ in range(5)]
        _lib.check(self.lib.sbe_sources(self.handle, w, _lib.ptr(P), _lib.ptr(C), _lib.ptr(D),
                                        _lib.ptr(ne), _lib.ptr(nh), *[_lib.ptr(o) for o in out],
                                        _lib.stream_handle()), "sbe_sources")
        return out

    def prop2qw(self, w, RR, fields4):
        nr = 2 * self.nk[w] + 2
        out = torch.empty((4, nr), dtype=CDTYPE, device=self.device)
        _lib.check(self.lib.sbe_prop2qw(self.handle, w, _lib.ptr(RR), RR.numel(),
                                        _lib.ptr(fields4), _lib.ptr(out), _lib.stream_handle()),
                   "sbe_prop2qw")
        return out

    def qw2prop(self, w, RR, src5, plasmonics):
        out = torch.empty((5, RR.numel()), dtype=CDTYPE, device=self.device)
        _lib.check(self.lib.sbe_qw2prop(self.handle, w, _lib.ptr(RR), RR.numel(), _lib.ptr(src5),
                                        _lib.ptr(out), int(bool(plasmonics)),
                                        _lib.stream_handle()), "sbe_qw2prop")
        return out

    # ---- whole-batch steps -------------------------------------------------
    def leapfrog_step(self, state9, Ek, dt, src_out):
        arr = (ctypes.c_void_p * 9)(*[t.data_ptr() for t in state9])
        for t in state9:
            _lib.ptr(t)
        _lib.check(self.lib.sbe_leapfrog_step(self.handle, arr, _lib.ptr(Ek), float(dt),
                                              _lib.ptr(src_out), _lib.stream_handle()),
                   "sbe_leapfrog_step")

    def rk4_step(self, P, C, D, Ek0, dEk, dt, src_out, precision=_lib.PREC_FP64):
        _lib.check(self.lib.sbe_rk4_step(self.handle, _lib.ptr(P), _lib.ptr(C), _lib.ptr(D),
                                         _lib.ptr(Ek0), _lib.ptr(dEk), float(dt), int(precision),
                                         _lib.ptr(src_out), _lib.stream_handle()), "sbe_rk4_step")

    def local_field(self, e0, de=None, comp=1, Ek0=None, dEk=None):
        """Field uniform along every wire (sbe_local_field): component ``comp`` of
        wire w is e0[w] FFTG(window); e0, de: one amplitude per wire (device float64
        tensors or host sequences).  Fills and returns (Ek0, dEk)."""
        def dev(v):
            return torch.as_tensor(v, dtype=torch.float64, device=self.device).contiguous()
        e0 = dev(e0)
        de = None if de is None else dev(de)
        if Ek0 is None:
            Ek0 = self.zeros_r(3)
        if dEk is None and de is not None:
            dEk = self.zeros_r(3)
        _lib.check(self.lib.sbe_local_field(self.handle, _lib.ptr(e0), _lib.ptr(de), int(comp),
                                            _lib.ptr(Ek0), _lib.ptr(dEk),
                                            _lib.stream_handle()), "sbe_local_field")
        return Ek0, dEk

    def rk4_graph(self, P, C, D, Ek0, dEk, dt, src_out, precision=_lib.PREC_FP64):
        """Capture one rk4_step on these buffers into a CUDA graph (RK4Graph)."""
        return RK4Graph(self, P, C, D, Ek0, dEk, dt, src_out, precision)

    def deph(self, C, D, fp32=False):
        """Off-diagonal dephasing matrices (De, Dh), packed [2Nk+1][Nk] per wire, of the
        occupations of C, D: the FP64 reference sums or the mixed path's FP32 sums."""
        n = sum((2 * s.nk + 1) * s.nk for s in self.specs)
        De = torch.empty(n, dtype=torch.float64, device="cuda")
        Dh = torch.empty_like(De)
        _lib.check(self.lib.sbe_deph_selftest(self.handle, _lib.ptr(C), _lib.ptr(D), int(bool(fp32)),
                                              _lib.ptr(De), _lib.ptr(Dh), _lib.stream_handle()),
                   "sbe_deph_selftest")
        return De, Dh

    def autotune(self, cache_json=None):
        """Choose the mixed path's GEMM tiles per Nk bucket (sbe_autotune): time both
        N tiles, or load the choice cached in ``cache_json`` for this device and these
        buckets; returns ``tiles()``."""
        path = None if cache_json is None else str(cache_json).encode()
        _lib.check(self.lib.sbe_autotune(self.handle, path), "sbe_autotune")
        return self.tiles()

    def tiles(self):
        """Per bucket (Nk, wires, exchange tile, commutator tile, source tile,
        hi*hi split)."""
        cap = 6 * self.nw
        out = (ctypes.c_int * cap)()
        nb = ctypes.c_int()
        _lib.check(self.lib.sbe_ctx_tiles(self.handle, out, cap, ctypes.byref(nb)),
                   "sbe_ctx_tiles")
        return [tuple(out[6 * i:6 * i + 6]) for i in range(nb.value)]

    def check(self):
        """Wait for the current stream and raise if a device-side bounded wait gave up."""
        _lib.check(self.lib.sbe_ctx_check(self.handle, _lib.stream_handle()), "sbe_ctx_check")

    def wait_selftest(self):
        """Make one bounded wait give up (~2 s) on a barrier nothing completes; True if
        it did.  The next check() then raises; the context stays usable."""
        g = ctypes.c_int(0)
        _lib.check(self.lib.sbe_wait_selftest(self.handle, ctypes.byref(g), _lib.stream_handle()),
                   "sbe_wait_selftest")
        return g.value == 1

    def charge(self):
        """(n_wires, 2) carrier numbers sum |C_kk|, sum |D_kk| that the charge
        normalisation of the last step found (FP64, before it rescaled them)."""
        out = torch.zeros(len(self.specs), 2, dtype=torch.float64)
        _lib.check(self.lib.sbe_ctx_charge(self.handle, ctypes.c_void_p(out.data_ptr()),
                                           _lib.stream_handle()), "sbe_ctx_charge")
        return out

    def charge_imbalance(self):
        """max over wires of |N_e - N_h| / ((N_e + N_h) / 2) before the last step's
        normalisation (0 for wires without carriers)."""
        q = self.charge()
        mean = 0.5 * (q[:, 0] + q[:, 1])
        r = (q[:, 0] - q[:, 1]).abs() / torch.where(mean > 0, mean, torch.ones_like(mean))
        return float(r.max()) if len(r) else 0.0

    def profile(self, enable=True):
        _lib.check(self.lib.sbe_ctx_profile(self.handle, int(bool(enable))), "sbe_ctx_profile")

    def profile_read(self, category):
        """(total ms, launches) of a timed category since the last read:
        0 commutator GEMMs, 1 exchange GEMMs, 2 source GEMMs, 3 FP32 dephasing."""
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        _lib.check(self.lib.sbe_ctx_profile_read(self.handle, int(category), ctypes.byref(ms),
                                                 ctypes.byref(n)), "sbe_ctx_profile_read")
        return ms.value, n.value

    def rhs(self, P, C, D, Ek, precision=_lib.PREC_FP64):
        dP = torch.empty_like(P)
        dC = torch.empty_like(C)
        dD = torch.empty_like(D)
        _lib.check(self.lib.sbe_rhs(self.handle, _lib.ptr(P), _lib.ptr(C), _lib.ptr(D),
                                    _lib.ptr(Ek), int(precision), _lib.ptr(dP), _lib.ptr(dC),
                                    _lib.ptr(dD), _lib.stream_handle()), "sbe_rhs")
        return dP, dC, dD
