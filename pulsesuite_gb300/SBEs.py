"""GB300 drop-in for ``pulsesuite.PSTD3D.SBEs`` (the quantum-wire SBE module).

The names, arguments and in-place/return conventions follow the reference
(src/pulsesuite/PSTD3D/SBEs.py):

* ``dpdt``, ``dCdt``, ``dDdt`` (SBEs.py:1839, 2210, 2502) return new arrays;
* ``CalcH`` (SBEs.py:658) fills Heh, Hee, Hhh in place;
* ``SBESolver`` (SBEs.py:4619) with ``QWCalculator`` (SBEs.py:5826), ``chiqw``,
  ``getqc``, ``QWArea``, ``ShutOffOptics``, ``write_sbes_data`` /
  ``read_sbes_data`` (SBEs.py:5504-5569);
* the module-level shims ``InitializeSBE``, ``QWCalculator``, ``chiqw``,
  ``getqc``, ``QWArea``, ``ShutOffOptics``, ``WriteSBEsData``, ``ReadSBEsData``
  (SBEs.py:6011-6053).

Arrays may be NumPy (host; results come back as NumPy) or CUDA torch tensors
(results stay on the device).  All arithmetic runs in libsbe_gb300 on the GPU;
there is no CPU path.  With ``write_info`` (on, as in the reference) the solver
appends the reference's per-step text diagnostics: dataQW/info.WW.t.dat and
EP.WW.t.dat (SBEs.py:5769-5809), output/PdotE.p.dat and PdotE.w.dat
(SBEs.py:5924-5975) and dataQW/Wire/info/MaxOffDiag.e.dat and .h.dat
(dephasing.py:538-539, 731-740); the statistics are reduced on the device.
"""

import os

import numpy as np
import torch

from . import _lib
from .constants import C0, E0, EPS0, HBAR, KB, ME0, PI, TWOPI
from .params import read_mb_params, read_qw_params
from .wires import CDTYPE, WireContext, WireSpec

ii = 1j
hbar = HBAR
eV = 1.602176634e-19


def _to_dev(x, dtype):
    if isinstance(x, torch.Tensor):
        if not x.is_cuda:
            x = x.cuda()
        return x.to(dtype).contiguous(), True
    a = np.ascontiguousarray(np.asarray(x))
    return torch.from_numpy(a).to("cuda", dtype).contiguous(), False


def _ret(t, was_torch):
    return t if was_torch else t.cpu().numpy()


def _rhs_call(which, C, D, p, Heh, Hee, Hhh, GamE=None, GamH=None, Off=None):
    lib = _lib.load()
    tC, is_t = _to_dev(C, CDTYPE)
    tD, _ = _to_dev(D, CDTYPE)
    tp, _ = _to_dev(p, CDTYPE)
    th = [_to_dev(h, CDTYPE)[0] for h in (Heh, Hee, Hhh)]
    nk = tp.shape[0]
    out = torch.empty_like(tp)
    s = _lib.stream_handle()
    if which == 0:
        ge = _to_dev(GamE, torch.float64)[0]
        gh = _to_dev(GamH, torch.float64)[0]
        to = _to_dev(Off, CDTYPE)[0] if Off is not None else None
        rc = lib.sbe_dpdt(nk, _lib.ptr(tC), _lib.ptr(tD), _lib.ptr(tp), *[_lib.ptr(h) for h in th],
                          _lib.ptr(ge), _lib.ptr(gh), _lib.ptr(to), _lib.ptr(out), s)
    elif which == 1:
        rc = lib.sbe_dCdt(nk, _lib.ptr(tC), _lib.ptr(tD), _lib.ptr(tp), *[_lib.ptr(h) for h in th],
                          _lib.ptr(out), s)
    else:
        rc = lib.sbe_dDdt(nk, _lib.ptr(tC), _lib.ptr(tD), _lib.ptr(tp), *[_lib.ptr(h) for h in th],
                          _lib.ptr(out), s)
    _lib.check(rc, ("dpdt", "dCdt", "dDdt")[which])
    return _ret(out, is_t)


def dpdt(C, D, p, Heh, Hee, Hhh, GamE, GamH, OffP):
    """SBEs.py:1839 dp/dt (p stored [kh][ke])."""
    return _rhs_call(0, C, D, p, Heh, Hee, Hhh, GamE, GamH, OffP)


def dCdt(Cee, Dhh, Phe, Heh, Hee, Hhh, GamE, GamH, OffE):
    """SBEs.py:2210 dC/dt (GamE, GamH, OffE unused, as in the reference)."""
    return _rhs_call(1, Cee, Dhh, Phe, Heh, Hee, Hhh)


def dDdt(Cee, Dhh, Phe, Heh, Hee, Hhh, GamE, GamH, OffH):
    """SBEs.py:2502 dD/dt (GamE, GamH, OffH unused, as in the reference)."""
    return _rhs_call(2, Cee, Dhh, Phe, Heh, Hee, Hhh)


def calc_h(Meh, Wee, Whh, C, D, p, VC, Heh, Hee, Hhh, Ee, Eh, gap, excitons, lf, freepot):
    """SBEs.py:809-1131 CalcH with explicit grid energies and flags; outputs in place."""
    lib = _lib.load()
    tM, is_t = _to_dev(Meh, CDTYPE)
    tW = _to_dev(Wee, CDTYPE)[0]
    tWh = _to_dev(Whh, CDTYPE)[0]
    tC = _to_dev(C, CDTYPE)[0]
    tD = _to_dev(D, CDTYPE)[0]
    tp = _to_dev(p, CDTYPE)[0]
    tV = _to_dev(VC, torch.float64)[0]
    tEe = _to_dev(Ee, torch.float64)[0]
    tEh = _to_dev(Eh, torch.float64)[0]
    nk = tp.shape[0]
    o = [torch.empty_like(tp) for _ in range(3)]
    _lib.check(lib.sbe_calch(nk, _lib.ptr(tM), _lib.ptr(tW), _lib.ptr(tWh), _lib.ptr(tC),
                             _lib.ptr(tD), _lib.ptr(tp), _lib.ptr(tV), _lib.ptr(tEe),
                             _lib.ptr(tEh), float(gap), int(bool(excitons)), int(bool(lf)),
                             int(bool(freepot)), *[_lib.ptr(x) for x in o],
                             _lib.stream_handle()), "CalcH")
    for dst, src in zip((Heh, Hee, Hhh), o):
        if isinstance(dst, torch.Tensor):
            dst.copy_(src)
        else:
            dst[...] = src.cpu().numpy()


def CalcH(Meh, Wee, Whh, C, D, p, VC, Heh, Hee, Hhh):
    """SBEs.py:658 CalcH with the grid/flags of the initialised solver."""
    s = _default_solver
    if s is None:
        raise RuntimeError("CalcH: call InitializeSBE first")
    calc_h(Meh, Wee, Whh, C, D, p, VC, Heh, Hee, Hhh, s.Ee, s.Eh, s.gap, s.Excitons, s.LF,
           s.FreePot)


def yw(w):
    """qwoptics.py:1093: (-1)**floor((w-1)/2)."""
    return (-1) ** int(np.floor((w - 1) / 2.0))


def QWChi1(lam, dky, Ee, Eh, area, geh, dcv):
    """qwoptics.py:1109-1146: linear susceptibility of the wire (a scalar)."""
    ww = TWOPI * C0 / lam
    d1 = Ee + Eh - ii * HBAR * geh - HBAR * ww
    d2 = Ee + Eh + ii * HBAR * geh + HBAR * ww
    return 4 * dcv ** 2 / EPS0 / area * dky / TWOPI * np.sum((Ee + Eh) / (d1 * d2))


_LEVELS = ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3")


class SBESolver:
    """SBEs.py:4619 SBESolver on the GPU.

    By default every wire has a device context of its own and QWCalculator(w) steps
    wire w, as the reference does.  With ``batch=True`` all wires share one context:
    QWCalculator(w) for w < Nw stages wire w's field and keeps its output arrays, and
    the call for w = Nw steps every wire in one batched leapfrog step and fills the
    output arrays of all of them (the drivers call the wires of a time step in order
    and read the outputs after the last one, sbetestprop.py:181-234,
    rhoPJ.py:306-343)."""

    def __init__(self, q, rr, r0, Emaxxx, lam, Nw, QW, backend="gb300", params=None, flags=None,
                 nk=None, temp=77.0, batch=False):
        self.Nw = Nw
        self.batch = bool(batch)
        self.QW = QW
        self.xxx = 1
        self.jjj = 1
        self.t = 0.0
        self.wireoff = True
        self.small = 1e-200
        if not QW:
            return
        p = params if params is not None else read_qw_params()
        f = flags if flags is not None else read_mb_params()
        for k, v in p.items():
            setattr(self, k, v)
        self.flags = dict(f)
        for k, v in f.items():
            setattr(self, k, v)
        self.Emax0 = Emaxxx
        # the reference appends dataQW/info.WW.t.dat and EP.WW.t.dat every step
        self.write_info = True
        kmax = np.sqrt(1.2 * self.gap * 2.0 * self.me / (HBAR ** 2))
        self.dkr = TWOPI / (2.0 * self.L)
        if nk is None:
            nk = int(np.floor(kmax / self.dkr) * 2 + 1) - 1
        self.Nk = nk
        self.Nr = 2 * nk + 2
        cflags = {k: bool(f.get(k, False)) for k in _lib.FLAG_BITS}
        specs = [WireSpec(nk=nk, L=self.L, Delta0=self.Delta0, gap=self.gap, me=self.me,
                          mh=self.mh, HO=self.HO, gam_e=self.gam_e, gam_h=self.gam_h,
                          gam_eh=self.gam_eh, epsr=self.epsr, Oph=self.Oph, Gph=self.Gph,
                          temp=temp, Edc=float(getattr(self, "Edc", 0.0)), wire_index=w,
                          flags=cflags) for w in range(1, Nw + 1)]
        if self.batch:
            self.contexts = [WireContext(specs)]
        else:
            self.contexts = [WireContext([sp]) for sp in specs]
        c0 = self.contexts[0]
        self.kr = c0.table(0, "kr").cpu().numpy()
        self.r = c0.table(0, "r").cpu().numpy()
        self.Ee = c0.table(0, "Ee").cpu().numpy()
        self.Eh = c0.table(0, "Eh").cpu().numpy()
        sc = c0.table(0, "scalars").cpu().numpy()
        self.dcv, self.alphae, self.alphah, self.ehint, self.area, self.qc = sc[:6]
        self.dr = (self.r[2] - self.r[1]) * (self.Nr - 1) / float(self.Nr)
        self.kkp = np.round((self.kr[:, None] - self.kr[None, :]) / self.dkr).astype(np.int64)
        self.chiw = QWChi1(lam, self.dkr, self.Ee + self.gap, self.Eh, self.area, self.gam_eh,
                           self.dcv)
        # initial state (SBEs.py:4829-4849): Fermi diagonals at Ee + gap/2 (both carriers)
        with np.errstate(over="ignore"):
            fe = 1.0 / (np.exp((self.Ee + self.gap / 2.0) / KB / temp) + 1.0)
        dev = torch.device("cuda")
        d = torch.as_tensor(fe, dtype=CDTYPE, device=dev)
        if self.batch:
            # nine packed levels of all wires; _st[w][i] are views of wire w's blocks
            self._lev = [c0.zeros_state() for _ in range(9)]
            self._st = [[c0.mat(self._lev[i], w) for i in range(9)] for w in range(Nw)]
            self._ek = c0.zeros_r(3)
            self._src = c0.zeros_r(5)
            self._outs = [None] * Nw
        else:
            self._st = [[torch.zeros((nk, nk), dtype=CDTYPE, device=dev) for _ in range(9)]
                        for _ in range(Nw)]
        for w in range(Nw):
            for i in (3, 4, 5, 6, 7, 8):
                self._st[w][i].diagonal().copy_(d)
        self.rr_offset = np.asarray(rr) - r0
        self._rr_dev = None
        # PdotE bookkeeping (SBEs.py:5924-5975): one history of the last two calls'
        # Re P on both grids, shared by all wires as in the reference
        self._pde = None
        self._fld = [None] * Nw
        if self.OffDiagDph and self.write_info:
            # InitializeDephasing opens (truncates) both files (dephasing.py:537-539)
            os.makedirs("dataQW/Wire/info", exist_ok=True)
            for sp in ("e", "h"):
                open(f"dataQW/Wire/info/MaxOffDiag.{sp}.dat", "w", encoding="utf-8").close()

    # reference-shaped state views (Nk, Nk, Nw), copied from/to the GPU
    def _get_level(self, i):
        return np.stack([self._st[w][i].cpu().numpy() for w in range(self.Nw)], axis=2)

    def _set_level(self, i, arr):
        arr = np.asarray(arr)
        for w in range(self.Nw):
            self._st[w][i].copy_(torch.as_tensor(np.ascontiguousarray(arr[:, :, w]), dtype=CDTYPE))

    def chiqw(self):
        return self.chiw

    def getqc(self):
        return self.qc

    def QWArea(self):
        return self.area

    def ShutOffOptics(self):
        """SBEs.py:5516: disable optical coupling (rebuilds the wire contexts' flag)."""
        self.Optics = False
        self.flags["Optics"] = False
        for ctx in self.contexts:
            for spec in ctx.specs:
                spec.flags = dict(spec.flags, Optics=False)
        self.contexts = [WireContext(ctx.specs) for ctx in self.contexts]

    def QWCalculator(self, Exx, Eyy, Ezz, Vrr, rr, q, dt, w, Pxx, Pyy, Pzz, Rho, DoQWP, DoQWDl):
        """SBEs.py:5826-5985: advance wire w by dt and return its sources in place."""
        Pxx[:] = 0.0
        Pyy[:] = 0.0
        Pzz[:] = 0.0
        Rho[:] = 0.0
        if w == 1:
            if self.jjj == self.jmax:
                self.jjj = 0
            self.xxx += 1
            self.jjj += 1
            self.t += dt
        mag = np.max(np.sqrt(np.abs(Exx) ** 2 + np.abs(Eyy) ** 2 + np.abs(Ezz) ** 2))
        if self.wireoff and mag < 1e-3 * self.Emax0:
            return
        self.wireoff = False
        DoQWP[0] = self.Optics
        DoQWDl[0] = self.LF
        RR = torch.as_tensor(np.asarray(rr, dtype=np.float64), device="cuda")
        f4 = torch.as_tensor(np.stack([np.asarray(a, dtype=complex) for a in (Exx, Eyy, Ezz, Vrr)]),
                             dtype=CDTYPE, device="cuda").contiguous()
        if self.batch:
            self._batched(w, RR, f4, dt, (Pxx, Pyy, Pzz, Rho))
            return
        ctx = self.contexts[w - 1]
        Ek = ctx.prop2qw(0, RR, f4)                       # (4, Nr): Ex, Ey, Ez, Vr in wire k space
        src = torch.empty((5, self.Nr), dtype=CDTYPE, device="cuda")
        Ek3 = Ek[:3].contiguous()
        ctx.leapfrog_step(self._st[w - 1], Ek3, dt, src)
        out = ctx.qw2prop(0, RR, src, self.LF).cpu().numpy()
        if self.write_info:
            self._write_info(ctx, w, dt, src, Ek3)
            self._write_maxoffdiag(ctx, 0)
        Pxx[:] = out[0]
        Pyy[:] = out[1]
        Pzz[:] = out[2]
        Rho[:] = out[4] - out[3]
        if self.write_info:
            self._pdote(ctx, 0, (Exx, Eyy, Ezz), (Pxx, Pyy, Pzz), rr, Ek3, src)
        if getattr(self, "ignorewire", False):
            Pxx[:] = 0.0
            Pyy[:] = 0.0
            Pzz[:] = 0.0
            Rho[:] = 0.0

    def _batched(self, w, RR, f4, dt, outs):
        """Stage wire w's field; on the last wire step them all and fill every wire's
        outputs (Pxx, Pyy, Pzz, Rho = RhoH - RhoE, SBEs.py:5917)."""
        ctx = self.contexts[0]
        Ek = ctx.prop2qw(w - 1, RR, f4)
        ctx.rvec(self._ek, w - 1, 3).copy_(Ek[:3])
        self._outs[w - 1] = outs
        self._fld[w - 1] = (f4[0].real.cpu().numpy(), f4[1].real.cpu().numpy(),
                            f4[2].real.cpu().numpy(), RR.cpu().numpy())
        if w != self.Nw:
            return
        ctx.leapfrog_step(self._lev, self._ek, dt, self._src)
        for wi in range(self.Nw):
            o = self._outs[wi]
            if o is None:
                continue
            src = ctx.rvec(self._src, wi, 5).contiguous()
            out = ctx.qw2prop(wi, RR, src, self.LF).cpu().numpy()
            if self.write_info:
                self._write_info(ctx, wi + 1, dt, None, None)
                self._write_maxoffdiag(ctx, wi)
                ex, ey, ez, rr = self._fld[wi]
                self._pdote(ctx, wi, (ex, ey, ez), (out[0], out[1], out[2]), rr, self._ek,
                            self._src)
            ign = getattr(self, "ignorewire", False)
            o[0][:] = 0.0 if ign else out[0]
            o[1][:] = 0.0 if ign else out[1]
            o[2][:] = 0.0 if ign else out[2]
            o[3][:] = 0.0 if ign else out[4] - out[3]
        self._outs = [None] * self.Nw

    def _write_info(self, ctx, w, dt, src, Ek3):
        """SBEs.py:5769-5809: append this step's line to dataQW/info.WW.t.dat and to
        dataQW/EP.WW.t.dat (statistics reduced on the device by sbe_wire_info; the
        CalcI0n columns print as complex numbers, as the reference's do)."""
        st = self._st[w - 1]
        if self.batch:
            # the statistics kernel reads wire w's blocks of the packed buffers
            v = ctx.wire_info(w - 1, self._lev[4], self._lev[7], self._src, self._ek)
        else:
            v = ctx.wire_info(0, st[4], st[7], src, Ek3)
        t = self.xxx * dt
        info = [t] + [float(x) for x in v[:15]] + [complex(v[15], 0.0), complex(v[16], 0.0)]
        os.makedirs("dataQW", exist_ok=True)
        with open(f"dataQW/info.{w:02d}.t.dat", "a", encoding="utf-8") as f:
            f.write("".join(f"{x:18.6e} " for x in info[:-1]) + f"{info[-1]:18.6e}\n")
        with open(f"dataQW/EP.{w:02d}.t.dat", "a", encoding="utf-8") as f:
            f.write(" ".join(f"{x:18.6e}" for x in [t] + [float(x) for x in v[17:23]]) + "\n")

    def _write_maxoffdiag(self, ctx, wc):
        """dephasing.py:731-740: one line per preparation, t and the extrema of Re De
        (MaxOffDiag.e.dat) and Re Dh (MaxOffDiag.h.dat) of the wire just stepped."""
        if not self.OffDiagDph:
            return
        v = ctx.deph_extrema(wc)
        for sp, mx, mn in (("e", v[0], v[1]), ("h", v[2], v[3])):
            with open(f"dataQW/Wire/info/MaxOffDiag.{sp}.dat", "a", encoding="utf-8") as f:
                f.write(f"{float(self.t)!r} {float(mx)!r} {float(mn)!r}\n")

    def _pdote(self, ctx, wc, E3, P3, rr, Ek, src):
        """SBEs.py:5924-5975: accumulate P.E on the propagation grid (host arrays of
        this call) and on the wire grid (sbe_wire_pdote on the device), shift the
        two-call history, append t and the energies / e0 to output/PdotE.{p,w}.dat."""
        nrr, nr = len(P3[0]), self.Nr
        if self._pde is None:
            os.makedirs("output", exist_ok=True)
            for sp in ("p", "w"):
                open(f"output/PdotE.{sp}.dat", "w", encoding="utf-8").close()
            z = np.zeros((3, nrr))
            self._pde = dict(p0=z.copy(), p1=z.copy(), ep=0.0, epw=0.0,
                             w0=torch.zeros((3, nr), dtype=torch.float64, device="cuda"),
                             w1=torch.zeros((3, nr), dtype=torch.float64, device="cuda"))
        h = self._pde
        rr = np.asarray(rr)
        drr = rr[1] - rr[0] if len(rr) > 1 else 1.0
        inc = 0.0
        for c in range(3):
            inc = inc + np.sum((np.real(P3[c]) - h["p0"][c]) * np.real(E3[c]) * 0.5) * drr * self.area
        h["ep"] += inc
        h["epw"] += ctx.wire_pdote(wc, Ek, src, h["w0"]) * 0.5 * self.dr * self.area
        h["p0"], h["p1"] = h["p1"], np.stack([np.real(np.asarray(p)) for p in P3])
        h["w0"], h["w1"] = h["w1"], ctx.rvec(src.reshape(-1), wc, 5)[:3].real.contiguous()
        with open("output/PdotE.p.dat", "a", encoding="utf-8") as f:
            f.write(f"{float(self.t)!r} {float(h['ep'] / E0)!r}\n")
        with open("output/PdotE.w.dat", "a", encoding="utf-8") as f:
            f.write(f"{float(self.t)!r} {float(h['epw'] / E0)!r}\n")

    def write_sbes_data(self, n):
        """SBEs.py:5524-5546: dataQW/backup/{CC,DD,YY}{1,2,3}.n.dat, 're im' per line
        (Python float repr), loop order w, k2, k1.  The level is transposed on the
        GPU, copied once and formatted by the library's threaded writer."""
        os.makedirs("dataQW/backup/", exist_ok=True)
        for key in ("CC1", "CC2", "CC3", "DD1", "DD2", "DD3", "YY1", "YY2", "YY3"):
            i = _LEVELS.index(key)
            lev = torch.stack([self._st[w][i].t() for w in range(self.Nw)]).contiguous()
            text = _lib.backup_format(lev.cpu().numpy())
            with open(f"dataQW/backup/{key}.{n}.dat", "wb") as f:
                f.write(text)

    def read_sbes_data(self, Nt):
        """SBEs.py:5548-5569: inverse of write_sbes_data."""
        nk, nw = self.Nk, self.Nw
        for key in ("CC1", "CC2", "CC3", "DD1", "DD2", "DD3", "YY1", "YY2", "YY3"):
            i = _LEVELS.index(key)
            with open(f"dataQW/backup/{key}.{Nt}.dat", "rb") as f:
                vals = _lib.backup_parse(f.read(), nw * nk * nk).reshape(nw, nk, nk)
            for w in range(nw):
                lev = torch.as_tensor(vals[w], dtype=CDTYPE, device="cuda")
                self._st[w][i].copy_(lev.t())

    def close(self):
        for c in getattr(self, "contexts", []):
            c.close()


def _level_prop(i):
    return property(lambda self: self._get_level(i), lambda self, v: self._set_level(i, v))


for _i, _n in enumerate(_LEVELS):
    setattr(SBESolver, _n, _level_prop(_i))


_default_solver = None


def InitializeSBE(q, rr, r0, Emaxxx, lam, Nw, QW):
    """SBEs.py:6011: create the default solver from ./params/*.params."""
    global _default_solver
    _default_solver = SBESolver(q, rr, r0, Emaxxx, lam, Nw, QW)


def QWCalculator(Exx, Eyy, Ezz, Vrr, rr, q, dt, w, Pxx, Pyy, Pzz, Rho, DoQWP, DoQWDl):
    """SBEs.py:6017: delegate to the default solver."""
    _default_solver.QWCalculator(Exx, Eyy, Ezz, Vrr, rr, q, dt, w, Pxx, Pyy, Pzz, Rho, DoQWP,
                                 DoQWDl)


def chiqw():
    return _default_solver.chiqw()


def getqc():
    return _default_solver.getqc()


def QWArea():
    return _default_solver.QWArea()


def ShutOffOptics():
    _default_solver.ShutOffOptics()


def WriteSBEsData(n):
    _default_solver.write_sbes_data(n)


def ReadSBEsData(Nt):
    _default_solver.read_sbes_data(Nt)
