"""Generate the golden vectors that pin the oracle to the PulseSuite reference.

Run from the repository root in a container that holds the reference source::

    python tests/golden/make_golden.py /path/to/pulsesuite/src

The reference is pure Python but imports ``numba`` and ``pyfftw``, neither of
which is installed here.  This script writes two tiny stand-in packages into a
temporary directory: ``numba.jit`` returns the function unchanged (the mode the
reference's own ``NUMBA_DISABLE_JIT=1`` tox target uses) and
``pyfftw.interfaces.numpy_fft`` is ``numpy.fft`` (same DFT).  Every output below
is produced by the reference's own functions on seeded inputs; the inputs and
outputs are stored as ``.npz`` files next to this script.

Cases
-----
kernels_nkN     CalcH (``SBEs._CalcH_fallback``) for every flag combination and
                dpdt/dCdt/dDdt (``SBEs._dpdt_fallback`` ...), random inputs.
coulomb_nkN     ``coulomb.CoulombModule`` tables (V0, Chi1D, qe, qh) and
                ``CalcScreenedArrays`` with and without screening; K0 samples.
phonon_nkN      ``phonons.InitializePhonons`` tables and ``MBPE``/``MBPH``.
mbc_nkN         ``coulomb.CoulombModule`` carrier-carrier scattering ``MBCE``/``MBCH``
                (and the ``CalcMBArrays`` tables) with Gaussian and Lorentzian
                broadening.  ``make_golden.py <src> mbc`` writes these alone.
emission_nkN    ``emission.InitializeEmission`` tables and ``SpontEmission`` (Recomb);
                ``make_golden.py <src> emission`` writes these alone.
dc_nkN          ``dcfield.DCFieldModule.Transport`` (DCTrans) of a matrix with and
                without LF; ``make_golden.py <src> dc`` writes these alone.
backup_nk6      ``SBESolver.write_sbes_data`` files of nine levels (text and arrays);
                ``make_golden.py <src> backup`` writes it alone.
coupling3d      rhoPJ CalcJfx / QWPlacement and usefulsubs EAtXYZ on seeded inputs;
                ``make_golden.py <src> coupling3d`` writes it alone.
info_nkN        the statistics of dataQW/info.WW.t.dat and EP.WW.t.dat from the
                reference's helpers; ``make_golden.py <src> info`` writes these alone.
dephasing_nkN   ``dephasing.DephasingModule`` index maps, ``CalcGammaE/H`` and
                ``OffDiagDephasing2``.
qwoptics_nkN    ``qwoptics.QWOptics`` polarisation/charge sources, ``Prop2QW``
                and ``QW2Prop`` (cubic-spline resampling + FFTG).
solver_step     ``SBEs.SBESolver`` built from params files, several
                ``QWCalculator`` leapfrog steps on two wires.
solver_100      the same solver run for 100 leapfrog steps: the fields of every step,
                the sources of every tenth step and the nine state levels at the end;
                ``make_golden.py <src> solver100`` writes it alone.
pstd            Pieces of the field step: ``usefulsubs.dfdx1D`` on FFT-order
                wavenumbers (``libpulsesuite.helpers.GetKArray``), the grids of
                ``typespace`` and ``helpers``, and ``rhoPJ.ElongfromRho`` on an
                (Nx, 1, 1) grid.
pstd3d          Pieces of the 3-D field step: ``rhoPJ.ElongfromRho`` on a 3-D grid
                (all ten outputs and the in-place transformed P), the q-space
                derivatives ``usefulsubs.dfdx1D_q``/``dfdy1D_q``/``dfdx2D_q``/``dfdy2D_q``,
                ``dfdy2D`` and the axis grids of ``typespace`` and ``helpers`` at
                256 x 128 x 128 x 20 nm; ``make_golden.py <src> pstd3d`` writes it alone.
"""

import io
import os
import sys
import tempfile
import types
import contextlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_NUMBA_STUB = '''
def jit(*a, **k):
    if len(a) == 1 and callable(a[0]) and not k:
        return a[0]
    return lambda f: f
njit = jit
prange = range
def float64(*a, **k):
    return None
class _Cuda:
    @staticmethod
    def is_available():
        return False
    @staticmethod
    def jit(*a, **k):
        if len(a) == 1 and callable(a[0]):
            return a[0]
        return lambda f: f
cuda = _Cuda()
'''

_PYFFTW_STUB = '''
import numpy.fft as numpy_fft
class cache:
    enable = staticmethod(lambda: None)
    set_keepalive_time = staticmethod(lambda *a: None)
'''


def _install_stubs(tmp):
    os.makedirs(os.path.join(tmp, "numba"))
    os.makedirs(os.path.join(tmp, "pyfftw", "interfaces"))
    with open(os.path.join(tmp, "numba", "__init__.py"), "w") as f:
        f.write(_NUMBA_STUB)
    with open(os.path.join(tmp, "pyfftw", "__init__.py"), "w") as f:
        f.write("from . import interfaces\n")
    with open(os.path.join(tmp, "pyfftw", "interfaces", "__init__.py"), "w") as f:
        f.write(_PYFFTW_STUB)


# Material used for the component cases (GaAs-like wire, Appendix values of the
# synthetic workload): masses in me0, energies in eV.
MAT = dict(me=0.067, mh=0.45, gap=1.52, epsr=12.9, Delta0=6e-9, HO=100e-3,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, Oph=36e-3, Gph=3e-3)


def herm_state(rng, n, scale):
    z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    q, _ = np.linalg.qr(z)
    lam = rng.uniform(0.0, scale, n)
    return (q * lam) @ q.conj().T


def cnormal(rng, shape, sigma):
    return sigma * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2.0)


def wire_grid(nk, kabs=3e9):
    """Half-offset k grid with |k|max = kabs; grid arrays as SBESolver builds them."""
    from pulsesuite.PSTD3D.typespace import GetKArray, GetSpaceArray
    from pulsesuite.PSTD3D.usefulsubs import GetArray0Index
    dnk = (nk - 1) // 2
    dkr = kabs / (nk - 1 - dnk - 0.5) if nk > 1 else 1.0
    L = np.pi / dkr
    nr = 2 * nk + 2
    kr = np.array([dkr * (-dnk + k - 0.5) for k in range(nk)])
    r = GetSpaceArray(nr, 2 * L)
    Qr = GetKArray(nr, 2 * L)
    Qr = np.roll(Qr, nr // 2)
    Qr[0] = -Qr[0]
    NQ0 = GetArray0Index(Qr)
    kkp = np.zeros((nk, nk), dtype=np.int64)
    for k in range(nk):
        for kp in range(nk):
            kkp[k, kp] = int(np.round((kr[k] - kr[kp]) / dkr)) + NQ0
    return dict(nk=nk, nr=nr, dkr=dkr, L=L, kr=kr, r=r, Qr=Qr, kkp=kkp, NQ0=NQ0)


def derived(g):
    from scipy.constants import e as e0, hbar, m_e as me0
    me = MAT["me"] * me0
    mh = MAT["mh"] * me0
    gap = MAT["gap"] * e0
    HO = MAT["HO"] * e0
    Ee = hbar ** 2 * g["kr"] ** 2 / (2.0 * me)
    Eh = hbar ** 2 * g["kr"] ** 2 / (2.0 * mh)
    dcv = np.sqrt((e0 * hbar) ** 2 / (6.0 * me0 * gap) * (me0 / me - 1.0))
    ae = np.sqrt(me * HO) / hbar
    ah = np.sqrt(mh * HO) / hbar
    ehint = np.sqrt(2.0 * ae * ah / (ae ** 2 + ah ** 2))
    area = np.sqrt(2.0 * np.pi) / np.sqrt(ae ** 2 + ah ** 2) * MAT["Delta0"]
    return dict(me=me, mh=mh, gap=gap, Ee=Ee, Eh=Eh, dcv=dcv, alphae=ae,
                alphah=ah, ehint=ehint, area=area)


def case_kernels(nk, seed):
    from pulsesuite.PSTD3D import SBEs
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    C = herm_state(rng, nk, 0.1)
    D = herm_state(rng, nk, 0.1)
    P = cnormal(rng, (nk, nk), 1e-3)
    Meh = cnormal(rng, (nk, nk), 1e-22)
    Wee = cnormal(rng, (nk, nk), 1e-22)
    Whh = cnormal(rng, (nk, nk), 1e-22)
    VC = rng.uniform(0.5e-21, 2e-21, (nk, nk, 3))
    out = dict(C=C, D=D, P=P, Meh=Meh, Wee=Wee, Whh=Whh, VC=VC, Ee=d["Ee"],
               Eh=d["Eh"], gap=d["gap"])
    for exc in (0, 1):
        for lf in (0, 1):
            for fp in (0, 1):
                Heh = np.zeros((nk, nk), complex)
                Hee = np.zeros((nk, nk), complex)
                Hhh = np.zeros((nk, nk), complex)
                SBEs._CalcH_fallback(Meh, Wee, Whh, C, D, P, VC, Heh, Hee, Hhh, nk,
                                     d["Ee"], d["Eh"], d["gap"], bool(exc), bool(lf),
                                     bool(fp))
                tag = f"e{exc}l{lf}f{fp}"
                out[f"Heh_{tag}"] = Heh
                out[f"Hee_{tag}"] = Hee
                out[f"Hhh_{tag}"] = Hhh
    # RHS with Hamiltonians from the full-flag CalcH and random rates
    Heh, Hee, Hhh = out["Heh_e1l1f0"], out["Hee_e1l1f0"], out["Hhh_e1l1f0"]
    GamE = rng.uniform(0.5e12, 2e12, nk)
    GamH = rng.uniform(0.5e12, 2e12, nk)
    OffP = cnormal(rng, (nk, nk), 1e-37)
    out.update(GamE=GamE, GamH=GamH, OffP=OffP)
    out["dP"] = SBEs._dpdt_fallback(C, D, P, Heh, Hee, Hhh, GamE, GamH, OffP)
    out["dC"] = SBEs._dCdt_fallback(C, D, P, Heh, Hee, Hhh, GamE, GamH, OffP)
    out["dD"] = SBEs._dDdt_fallback(C, D, P, Heh, Hee, Hhh, GamE, GamH, OffP)
    return out


def case_coulomb(nk, seed):
    from pulsesuite.PSTD3D import coulomb
    from pulsesuite.PSTD3D.usefulsubs import K03
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    cm = coulomb.CoulombModule(g["r"], g["kr"], g["L"], MAT["Delta0"], d["me"], d["mh"],
                               d["Ee"], d["Eh"], MAT["gam_e"], MAT["gam_h"], d["alphae"],
                               d["alphah"], MAT["epsr"], g["Qr"], g["kkp"], True)
    out = dict(kr=g["kr"], r=g["r"], Qr=g["Qr"], kkp=g["kkp"], L=g["L"],
               Delta0=MAT["Delta0"], me=d["me"], mh=d["mh"], alphae=d["alphae"],
               alphah=d["alphah"], epsr=MAT["epsr"], Veh0=cm.Veh0, Vee0=cm.Vee0,
               Vhh0=cm.Vhh0, Chi1De=cm.Chi1De, Chi1Dh=cm.Chi1Dh, qe=cm.qe, qh=cm.qh)
    for i, (lo, hi) in enumerate(((0.0, 0.02), (0.05, 0.5))):
        ne = rng.uniform(lo, hi, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
        nh = rng.uniform(lo, hi, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
        out[f"ne{i}"] = ne
        out[f"nh{i}"] = nh
        for scr in (0, 1):
            VC = np.zeros((nk, nk, 3))
            E1D = np.zeros((nk, nk))
            cm.CalcScreenedArrays(bool(scr), g["L"], ne, nh, VC, E1D)
            out[f"VC{i}_s{scr}"] = VC
            out[f"E1D{i}_s{scr}"] = E1D
    xs = np.concatenate([np.geomspace(1e-3, 150.0, 200), [1.0, 2.0, 9.0, 18.0, 35.0, 50.0, 99.9]])
    out["k0_x"] = xs
    out["k0_jit"] = np.array([coulomb._K03_jit(x) for x in xs])
    out["k0_cik"] = np.array([K03(x) for x in xs])
    return out


def case_phonon(nk, temp, seed, VC, E1D):
    from pulsesuite.PSTD3D import phonons
    from scipy.constants import e as e0, hbar
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    phonons._Temp = temp
    Oph = MAT["Oph"] * e0 / hbar
    Gph = MAT["Gph"] * e0 / hbar
    phonons.InitializePhonons(g["kr"], d["Ee"], d["Eh"], g["L"], MAT["epsr"], Gph, Oph)
    ne = rng.uniform(0.0, 0.3, nk)
    nh = rng.uniform(0.0, 0.3, nk)
    WinE = rng.uniform(0, 1e11, nk)
    WoutE = rng.uniform(0, 1e11, nk)
    WinH = rng.uniform(0, 1e11, nk)
    WoutH = rng.uniform(0, 1e11, nk)
    out = dict(temp=temp, Oph=Oph, Gph=Gph, ne=ne, nh=nh, VC=VC, E1D=E1D,
               WinE0=WinE.copy(), WoutE0=WoutE.copy(), WinH0=WinH.copy(),
               WoutH0=WoutH.copy(), EP=phonons._EP, HP=phonons._HP,
               Vscale=phonons._Vscale, N0=phonons._NO)
    phonons.MBPE(ne, VC, E1D, WinE, WoutE)
    phonons.MBPH(nh, VC, E1D, WinH, WoutH)
    out.update(WinE=WinE, WoutE=WoutE, WinH=WinH, WoutH=WoutH)
    fermi = phonons.FermiDistr(d["Ee"] + d["gap"] / 2.0)
    out["fermi"] = fermi
    phonons._Temp = 77.0
    return out


def case_mbc(nk, seed, VC):
    """coulomb.CoulombModule(...).MBCE / MBCH with both broadenings."""
    from pulsesuite.PSTD3D import coulomb
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    ne = rng.uniform(0.0, 0.4, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
    nh = rng.uniform(0.0, 0.4, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
    out = dict(kr=g["kr"], Ee=d["Ee"], Eh=d["Eh"], ge=MAT["gam_e"] * 1.3, gh=MAT["gam_h"] * 0.8,
               VC=VC, ne=ne, nh=nh)
    for lz in (0, 1):
        cm = coulomb.CoulombModule(g["r"], g["kr"], g["L"], MAT["Delta0"], d["me"], d["mh"],
                                   d["Ee"], d["Eh"], out["ge"], out["gh"], d["alphae"],
                                   d["alphah"], MAT["epsr"], g["Qr"], g["kkp"], True,
                                   LorentzDelta=bool(lz))
        w = [rng.uniform(0, 1e11, nk) for _ in range(4)]
        out.update({f"WinE0_l{lz}": w[0].copy(), f"WoutE0_l{lz}": w[1].copy(),
                    f"WinH0_l{lz}": w[2].copy(), f"WoutH0_l{lz}": w[3].copy()})
        cm.MBCE(np.real(ne), np.real(nh), g["kr"], d["Ee"], d["Eh"], VC, MAT["gam_eh"],
                out["ge"], w[0], w[1])
        cm.MBCH(np.real(ne), np.real(nh), g["kr"], d["Ee"], d["Eh"], VC, MAT["gam_eh"],
                out["gh"], w[2], w[3])
        out.update({f"WinE_l{lz}": w[0], f"WoutE_l{lz}": w[1], f"WinH_l{lz}": w[2],
                    f"WoutH_l{lz}": w[3], f"Ceh_l{lz}": cm.Ceh, f"Cee_l{lz}": cm.Cee,
                    f"Chh_l{lz}": cm.Chh})
    return out


def case_emission(nk, seed, VC):
    """emission.InitializeEmission + SpontEmission (Recomb)."""
    from pulsesuite.PSTD3D import emission
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    ne = rng.uniform(0.0, 0.4, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
    nh = rng.uniform(0.0, 0.4, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
    geh = MAT["gam_eh"] * 1.2
    emission.InitializeEmission(g["kr"], d["Ee"], d["Eh"], abs(d["dcv"]), MAT["epsr"], geh,
                                d["ehint"])
    Rsp = np.zeros(nk)
    emission.SpontEmission(ne, nh, d["Ee"], d["Eh"], d["gap"], geh, VC, Rsp)
    return dict(kr=g["kr"], Ee=d["Ee"], Eh=d["Eh"], gap=d["gap"], dcv=d["dcv"],
                ehint=d["ehint"], epsr=MAT["epsr"], geh=geh, VC=VC, ne=ne, nh=nh, Rsp=Rsp,
                HOmega=emission._HOmega, square=emission._square, RScale=emission._RScale)


def case_dc(nk, seed):
    """dcfield.DCFieldModule.Transport (DCTrans) with and without LF."""
    from pulsesuite.PSTD3D import dcfield
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    dm = dcfield.DCFieldModule(g["kr"], d["me"], d["mh"], datadir=None)
    out = dict(kr=g["kr"], Edc=3.0e5, Eac=-1.2e5, dt=0.5e-15, Y=dm.Y)
    for lf in (0, 1):
        C = herm_state(rng, nk, 0.3) + cnormal(rng, (nk, nk), 1e-3)
        out[f"C_in_l{lf}"] = C.copy()
        dm.Transport(C, out["Edc"], out["Eac"], out["dt"], True, bool(lf))
        out[f"C_out_l{lf}"] = C
    return out


def backup_values(rng, shape):
    """Complex values over the float64 range for the backup-format case: random
    mantissas at exponents from subnormal to near overflow, plus the edges of the
    repr's positional/scientific switch, signed zeros and integers."""
    n = int(np.prod(shape))
    mag = 10.0 ** rng.uniform(-320, 307, 2 * n)
    v = rng.standard_normal(2 * n) * mag
    edge = [0.0, -0.0, 1.0, -2.0, 0.1 + 0.2, 1e-4, 1e-5, 9.999e-5, 1e15, 1e16, 9999999999999998.0,
            123456789012345678.0, 5e-324, -2.2250738585072014e-308, 1.7976931348623157e308,
            0.5, 1 / 3, 2.0 ** 52, 2.0 ** 53 + 2, 1e22, 1e23, 3.0e-7, 12345.678]
    v[:len(edge)] = edge
    z = np.empty(n, dtype=complex)
    z.real = v[0::2]   # (re + 1j * im would drop the sign of -0.0)
    z.imag = v[1::2]
    return z.reshape(shape)


def case_backup(nk, nw, seed):
    """SBESolver.write_sbes_data (SBEs.py:5524-5546) of nine levels: the files' text
    and the arrays it was written from."""
    from pulsesuite.PSTD3D import SBEs
    rng = np.random.default_rng(seed)
    keys = ["CC1", "CC2", "CC3", "DD1", "DD2", "DD3", "YY1", "YY2", "YY3"]
    obj = types.SimpleNamespace(Nk=nk)
    for k in keys:
        setattr(obj, k, backup_values(rng, (nk, nk, nw)))
    SBEs.SBESolver.write_sbes_data(obj, 7)
    out = dict(nk=nk, nw=nw, n=7)
    for k in keys:
        out["arr_" + k] = getattr(obj, k)
        with open(f"dataQW/backup/{k}.7.dat", "rb") as f:
            out["txt_" + k] = np.frombuffer(f.read(), dtype=np.uint8)
    # read_sbes_data forms float(re) + 1j * float(im): signed zeros do not all survive
    back = types.SimpleNamespace(Nk=nk, **{k: np.zeros((nk, nk, nw), complex) for k in keys})
    SBEs.SBESolver.read_sbes_data(back, 7)
    for k in keys:
        out["back_" + k] = getattr(back, k)
    return out


def case_info(nk, seed):
    """The statistics of dataQW/info.WW.t.dat and EP.WW.t.dat from the reference's
    own helpers (dcfield CalcVD, CalcI0, CalcI0n; usefulsubs TotalEnergy, Temperature,
    iFFTG) on seeded occupations, sources, fields and a screened VC."""
    from scipy.constants import e as E0, hbar as HBAR
    from pulsesuite.PSTD3D import dcfield, usefulsubs
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    kr, L = g["kr"], g["L"]
    nr = 2 * nk + 2
    me, mh, gap = d["me"], d["mh"], 1.52 * E0
    Ee = (HBAR * kr) ** 2 / (2 * me)
    Eh = (HBAR * kr) ** 2 / (2 * mh)
    ne2 = np.abs(rng.uniform(0, 0.3, nk) * np.exp(-(kr / kr.max()) ** 2)).astype(complex)
    nh2 = np.abs(rng.uniform(0, 0.2, nk) * np.exp(-(kr / kr.max() - 0.1) ** 2)).astype(complex)
    VC = np.abs(rng.standard_normal((nk, nk, 3))) * 1e-21
    re = cnormal(rng, nr, 1e3)
    rh = cnormal(rng, nr, 2e3)
    Ek = [cnormal(rng, nr, 1e6) for _ in range(3)]
    src3 = [cnormal(rng, nr, 1e-3) for _ in range(3)]
    dkr = np.pi / L
    dm = dcfield.DCFieldModule(kr, me, mh, datadir=None)
    dcfield._instance = dm
    info = [dcfield.CalcVD(kr, me, ne2), dcfield.CalcVD(kr, mh, nh2),
            np.real(2 * np.sum(ne2) / L), np.real(2 * np.sum(nh2) / L),
            usefulsubs.TotalEnergy(ne2, Ee + gap) / E0, usefulsubs.TotalEnergy(nh2, Eh) / E0,
            usefulsubs.Temperature(ne2, Ee), usefulsubs.Temperature(nh2, Eh),
            np.max(np.abs(re)), np.max(np.abs(rh)), dm.GetEDrift(),
            np.real(HBAR * np.sum((ne2 - nh2) * kr)) * 2.0, np.real(HBAR * np.sum(ne2 * kr)),
            np.real(-HBAR * np.sum(nh2 * kr)),
            np.real(dm.CalcI0(ne2, nh2, Ee, Eh, VC, dkr, kr, 0.0)),
            dcfield.CalcI0n(ne2, me, kr), dcfield.CalcI0n(1 - nh2, -mh, kr)]
    ep = []   # SBEs.py:5793-5809: iFFTG of the wire-k fields and sources, then [Nr // 2]
    for E in Ek + src3:
        x = E.copy()
        usefulsubs.iFFTG(x)
        ep.append(np.real(x[nr // 2]))
    return dict(kr=kr, L=L, me=me, mh=mh, gap=gap, Ee=Ee, Eh=Eh, ne2=ne2, nh2=nh2, VC=VC,
                re=re, rh=rh, Ek=np.array(Ek), src3=np.array(src3), dkr=dkr,
                info=np.array(info, dtype=complex), ep=np.array(ep))


def case_coupling3d(seed):
    """rhoPJ CalcJfx and QWPlacement, usefulsubs EAtXYZ of the reference on seeded
    inputs (points inside, on and outside the grid)."""
    from pulsesuite.PSTD3D import rhoPJ, usefulsubs
    rng = np.random.default_rng(seed)
    n = 257
    rn, rp = cnormal(rng, n, 1.0), cnormal(rng, n, 1.0)
    J = rhoPJ.CalcJfx(rn.copy(), rp.copy(), 1e-16, 5e-9)
    nx, ny, nz = 7, 5, 4
    fw = cnormal(rng, nx, 1.0)
    gx, gy, gz = rng.uniform(0, 1, nx), rng.uniform(-1, 1, ny), np.exp(-rng.uniform(0, 3, nz))
    grid = np.zeros((nx, ny, nz), dtype=complex)
    rhoPJ.QWPlacement(fw, gx, gy, gz, grid)
    x = np.sort(rng.uniform(-1, 1, 9))
    y = np.linspace(-2.0, 3.0, 6)
    z = np.cumsum(rng.uniform(0.1, 1.0, 5))
    f = cnormal(rng, (9, 6, 5), 1.0)
    pts = np.stack([rng.uniform(-1.3, 1.3, 40), rng.uniform(-2.5, 3.5, 40),
                    rng.uniform(0.0, z[-1] + 0.5, 40)], axis=1)
    pts[:5] = [[x[0], y[0], z[0]], [x[-1], y[-1], z[-1]], [x[3], y[2], z[1]],
               [-5.0, 10.0, 0.0], [x[4], y[4] + 1e-9, z[2]]]
    val = np.array([usefulsubs.EAtXYZ(f, x, y, z, *p) for p in pts])
    return dict(rn=rn, rp=rp, J=J, dt=1e-16, dx=5e-9, fw=fw, gx=gx, gy=gy, gz=gz, grid=grid,
                x=x, y=y, z=z, f=f, pts=pts, val=val)


def case_dephasing(nk, seed, VC):
    from pulsesuite.PSTD3D import dephasing
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    dm = dephasing.DephasingModule()
    dm.InitializeDephasing(g["kr"], d["me"], d["mh"])
    ne = rng.uniform(0.0, 0.4, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
    nh = rng.uniform(0.0, 0.4, nk) + 1j * rng.uniform(-1e-3, 1e-3, nk)
    P = cnormal(rng, (nk, nk), 1e-3)
    GamE = np.zeros(nk)
    GamH = np.zeros(nk)
    dm.CalcGammaE(g["kr"], ne, nh, VC, GamE)
    dm.CalcGammaH(g["kr"], ne, nh, VC, GamH)
    gvec = np.array([1.3e12, 0.9e12, 1.1e12])
    x = np.zeros((nk, nk), complex)
    dm.OffDiagDephasing2(ne, nh, P, g["kr"], d["Ee"], d["Eh"], gvec, VC, 0.0, x)
    De = dephasing.CalcOffDiagDeph_E2(ne, nh, g["kr"], d["Ee"], d["Eh"], gvec[0], gvec[2], VC, nk)
    Dh = dephasing.CalcOffDiagDeph_H2(ne, nh, g["kr"], d["Ee"], d["Eh"], gvec[1], gvec[2], VC, nk)
    return dict(kr=g["kr"], me=d["me"], mh=d["mh"], Ee=d["Ee"], Eh=d["Eh"], VC=VC,
                ne=ne, nh=nh, P=P, g=gvec, GamE=GamE, GamH=GamH, OffP=x, De=De, Dh=Dh,
                k_p_q=dm._k_p_q, k_m_q=dm._k_m_q, k1p=dm._k1p, k1p_m_q=dm._k1p_m_q,
                k1=dm._k1, k1_m_q=dm._k1_m_q, xe=dm._xe, xh=dm._xh)


def case_qwoptics(nk, seed):
    from pulsesuite.PSTD3D import qwoptics
    rng = np.random.default_rng(seed)
    g = wire_grid(nk)
    d = derived(g)
    qw = qwoptics.QWOptics(g["r"], g["L"], d["dcv"], g["kr"], g["Qr"], d["Ee"], d["Eh"],
                           d["ehint"], d["area"], d["gap"])
    nr = g["nr"]
    P = cnormal(rng, (nk, nk), 1e-3)
    C = herm_state(rng, nk, 0.1)
    D = herm_state(rng, nk, 0.1)
    out = dict(kr=g["kr"], r=g["r"], Qr=g["Qr"], kkp=g["kkp"], L=g["L"], dcv=d["dcv"],
               ehint=d["ehint"], area=d["area"], P=P, C=C, D=D,
               window=qw._QWWindow, Expikr=qw._Expikr)
    for w in (1, 2, 3, 4):
        Px = np.zeros(nr, complex)
        Py = np.zeros(nr, complex)
        Pz = np.zeros(nr, complex)
        qw.QWPolarization3(g["r"], g["kr"], P, d["ehint"], d["area"], g["L"], Px, Py, Pz, 1, w)
        out[f"Px_w{w}"] = Px
        out[f"Py_w{w}"] = Py
        out[f"Pz_w{w}"] = Pz
    ne = np.abs(np.diag(C)).astype(complex)
    nh = np.abs(np.diag(D)).astype(complex)
    re = np.zeros(nr, complex)
    rh = np.zeros(nr, complex)
    qw.QWRho5(g["Qr"], g["kr"], g["r"], g["L"], g["kkp"], P, C, D, ne, nh, re, rh, 1, 1)
    out.update(ne=ne, nh=nh, re=re, rh=rh)
    # propagation grid covering the wire and beyond, smooth random fields
    nrr = 3 * nr + 7
    RR = np.linspace(-1.6 * g["L"], 1.4 * g["L"], nrr)
    fld = {}
    for nm in ("Exx", "Eyy", "Ezz", "Vrr"):
        a = rng.standard_normal(4)
        fld[nm] = (1e6 * (a[0] * np.cos(RR / g["L"] * 3.1 + a[1]) + a[2] * np.sin(RR / g["L"] * 1.7))
                   + 1j * 1e5 * a[3] * np.cos(RR / g["L"]))
    Ex = np.zeros(nr, complex)
    Ey = np.zeros(nr, complex)
    Ez = np.zeros(nr, complex)
    Vr = np.zeros(nr, complex)
    qw.Prop2QW(RR, fld["Exx"], fld["Eyy"], fld["Ezz"], fld["Vrr"], 0.0, g["r"], Ex, Ey, Ez, Vr, 0.0, 1)
    out.update(RR=RR, Exx=fld["Exx"], Eyy=fld["Eyy"], Ezz=fld["Ezz"], Vrr=fld["Vrr"],
               Ex=Ex.copy(), Ey=Ey.copy(), Ez=Ez.copy(), Vr=Vr.copy())
    for plas in (0, 1):
        srcs = {}
        for nm in ("Px", "Py", "Pz", "re", "rh"):
            srcs[nm] = cnormal(rng, nr, 1.0)
            out[f"q2p_in_{nm}_{plas}"] = srcs[nm].copy()
        Pxx = np.zeros(nrr, complex)
        Pyy = np.zeros(nrr, complex)
        Pzz = np.zeros(nrr, complex)
        RhoE = np.zeros(nrr, complex)
        RhoH = np.zeros(nrr, complex)
        Exc, Eyc, Ezc, Vrc = Ex.copy(), Ey.copy(), Ez.copy(), Vr.copy()
        qw.QW2Prop(g["r"], g["Qr"], Exc, Eyc, Ezc, Vrc, srcs["Px"], srcs["Py"], srcs["Pz"],
                   srcs["re"], srcs["rh"], RR, Pxx, Pyy, Pzz, RhoE, RhoH, 1, 1, False, bool(plas))
        out.update({f"q2p_Pxx_{plas}": Pxx, f"q2p_Pyy_{plas}": Pyy, f"q2p_Pzz_{plas}": Pzz,
                    f"q2p_RhoE_{plas}": RhoE, f"q2p_RhoH_{plas}": RhoH})
    return out


QW_PARAMS = """{L}     # L
6e-9      # Delta0
1.52      # gap
0.067     # me
0.45      # mh
100e-3    # HO
1e12      # gam_e
1e12      # gam_h
1e12      # gam_eh
12.9      # epsr
36e-3     # Oph
3e-3      # Gph
0.0       # Edc
100000    # jmax
100000    # ntmax
"""

MB_PARAMS = """1 # Optics
1 # Excitons
0 # EHs
1 # Screened
1 # Phonon
0 # DCTrans
1 # LF
0 # FreePot
1 # DiagDph
1 # OffDiagDph
0 # Recomb
0 # PLSpec
0 # Ignorewire
0 # Xqwparams
0 # LorentzDelta
"""


def case_solver(L, nsteps, dt, E0, seed):
    """Full reference leapfrog steps: SBESolver + QWCalculator on two wires."""
    from pulsesuite.PSTD3D import SBEs
    rng = np.random.default_rng(seed)
    os.makedirs("params", exist_ok=True)
    with open("params/qw.params", "w") as f:
        f.write(QW_PARAMS.format(L=repr(L)))
    with open("params/mb.params", "w") as f:
        f.write(MB_PARAMS)
    nrr = 64
    drr = 2.5 * L / (nrr - 1)
    rr = np.linspace(-1.25 * L, 1.25 * L, nrr)
    qrr = np.zeros(nrr)
    lam = 800e-9
    s = SBEs.SBESolver(qrr, rr, 0.0, E0, lam, 2, True)
    nk = s.Nk
    # a non-trivial starting state so that every term of the step is exercised
    for w in range(2):
        for arr in (s.YY1, s.YY2, s.YY3):
            arr[:, :, w] = cnormal(rng, (nk, nk), 1e-3)
        for arr in (s.CC1, s.CC2, s.CC3, s.DD1, s.DD2, s.DD3):
            arr[:, :, w] = herm_state(rng, nk, 0.05)
    out = dict(L=L, dt=dt, E0=E0, rr=rr, nk=nk, nr=s.Nr, kr=s.kr, r=s.r, Qr=s.Qr,
               kkp=s.kkp, dcv=s.dcv, ehint=s.ehint, area=s.area, alphae=s.alphae,
               alphah=s.alphah)
    init = {}
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        init[nm] = getattr(s, nm).copy()
        out[f"init_{nm}"] = init[nm]
    amp = rng.uniform(0.5, 1.5, (nsteps, 3, 2))
    t = 0.0
    for n in range(nsteps):
        flds = []
        for c in range(3):
            f = (E0 * amp[n, c, 0] * np.cos(2 * np.pi * rr / (3 * L) + amp[n, c, 1])
                 + 0j)
            flds.append(f)
        Exx, Eyy, Ezz = flds
        Vrr = np.zeros(nrr, complex)
        out[f"s{n}_Exx"] = Exx
        out[f"s{n}_Eyy"] = Eyy
        out[f"s{n}_Ezz"] = Ezz
        for w in (1, 2):
            Pxx = np.zeros(nrr, complex)
            Pyy = np.zeros(nrr, complex)
            Pzz = np.zeros(nrr, complex)
            Rho = np.zeros(nrr, complex)
            s.QWCalculator(Exx, Eyy, Ezz, Vrr, rr, qrr, dt, w, Pxx, Pyy, Pzz, Rho, [True], [False])
            out[f"s{n}_w{w}_Pxx"] = Pxx
            out[f"s{n}_w{w}_Pyy"] = Pyy
            out[f"s{n}_w{w}_Pzz"] = Pzz
            out[f"s{n}_w{w}_Rho"] = Rho
        for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
            out[f"s{n}_{nm}"] = getattr(s, nm).copy()
        t += dt
    s.close()
    return out


def case_solver100(L, nsteps, dt, E0, seed):
    """nsteps reference leapfrog steps (SBESolver + QWCalculator, two wires): fields of
    every step (real, along rr), sources of every tenth step and the last, and the nine
    state levels after the last step."""
    from pulsesuite.PSTD3D import SBEs
    rng = np.random.default_rng(seed)
    os.makedirs("params", exist_ok=True)
    with open("params/qw.params", "w") as f:
        f.write(QW_PARAMS.format(L=repr(L)))
    with open("params/mb.params", "w") as f:
        f.write(MB_PARAMS)
    nrr = 64
    rr = np.linspace(-1.25 * L, 1.25 * L, nrr)
    qrr = np.zeros(nrr)
    s = SBEs.SBESolver(qrr, rr, 0.0, E0, 800e-9, 2, True)
    nk = s.Nk
    for w in range(2):
        for arr in (s.YY1, s.YY2, s.YY3):
            arr[:, :, w] = cnormal(rng, (nk, nk), 1e-3)
        for arr in (s.CC1, s.CC2, s.CC3, s.DD1, s.DD2, s.DD3):
            arr[:, :, w] = herm_state(rng, nk, 0.05)
    out = dict(L=L, dt=dt, E0=E0, rr=rr, nk=nk, nsteps=nsteps)
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        out[f"init_{nm}"] = getattr(s, nm).copy()
    amp = rng.uniform(0.5, 1.5, (nsteps, 3, 2))
    fields = np.empty((nsteps, 3, nrr))
    for n in range(nsteps):
        for c in range(3):
            fields[n, c] = E0 * amp[n, c, 0] * np.cos(2 * np.pi * rr / (3 * L) + amp[n, c, 1])
    out["fields"] = fields
    for n in range(nsteps):
        Exx, Eyy, Ezz = (fields[n, c] + 0j for c in range(3))
        Vrr = np.zeros(nrr, complex)
        for w in (1, 2):
            srcs = [np.zeros(nrr, complex) for _ in range(4)]
            s.QWCalculator(Exx, Eyy, Ezz, Vrr, rr, qrr, dt, w, *srcs, [True], [False])
            if n % 10 == 9 or n == nsteps - 1:
                for a, nm in zip(srcs, ("Pxx", "Pyy", "Pzz", "Rho")):
                    out[f"s{n}_w{w}_{nm}"] = a
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        out[f"end_{nm}"] = getattr(s, nm).copy()
    s.close()
    # the text diagnostics the reference appended on the way (SBEs.py:5940-5975,
    # dephasing.py:538-539 and 731-740)
    for key, path in (("pdote_p", "output/PdotE.p.dat"), ("pdote_w", "output/PdotE.w.dat"),
                      ("maxoff_e", "dataQW/Wire/info/MaxOffDiag.e.dat"),
                      ("maxoff_h", "dataQW/Wire/info/MaxOffDiag.h.dat")):
        with open(path, "rb") as f:
            out["txt_" + key] = np.frombuffer(f.read(), dtype=np.uint8)
    return out


def case_pstd(nx, dx, seed):
    from pulsesuite.PSTD3D import rhoPJ, typespace, usefulsubs
    from pulsesuite.libpulsesuite import helpers
    rng = np.random.default_rng(seed)
    q = helpers.GetKArray(nx, nx * dx)
    x_h = helpers.GetSpaceArray(nx, (nx - 1) * dx)
    x_t = typespace.GetSpaceArray(nx, (nx - 1) * dx)
    f = cnormal(rng, (nx,), 1.0)
    df = usefulsubs.dfdx1D(f.copy(), q)
    sp = typespace.ss(1, nx, 1, 1, dx, 1.0, 1.0, 12.9)
    qx = typespace.GetKxArray(sp)
    epsr_used = typespace.GetEpsr(sp)
    rho = cnormal(rng, (nx, 1, 1), 1.0)
    px = cnormal(rng, (nx, 1, 1), 1e-9)
    outs = [np.zeros((nx, 1, 1), complex) for _ in range(10)]
    z = np.zeros((nx, 1, 1), complex)
    rhoPJ.ElongfromRho(sp, rho.copy(), px.copy(), z.copy(), z.copy(), *outs)
    return dict(nx=nx, dx=dx, q=q, x_helpers=x_h, x_typespace=x_t, f=f, df=df, qx_space=qx,
                epsr_space=epsr_used, rho=rho[:, 0, 0], px=px[:, 0, 0],
                Exl_PRho=outs[0][:, 0, 0], Exl_P=outs[3][:, 0, 0], Exl_Rho=outs[6][:, 0, 0])


def case_pstd3d(seed):
    from pulsesuite.PSTD3D import rhoPJ, typespace, usefulsubs
    from pulsesuite.libpulsesuite import helpers
    rng = np.random.default_rng(seed)
    nx, ny, nz = 8, 4, 16
    dx, dy, dz = 20e-9, 25e-9, 15e-9
    sp = typespace.ss(3, nx, ny, nz, dx, dy, dz, 12.9)
    qx, qy, qz = typespace.GetKxArray(sp), typespace.GetKyArray(sp), typespace.GetKzArray(sp)
    rho = cnormal(rng, (nx, ny, nz), 1.0)
    P = [cnormal(rng, (nx, ny, nz), 1e-9) for _ in range(3)]
    Pin = [a.copy() for a in P]
    outs = [np.zeros((nx, ny, nz), complex) for _ in range(10)]
    rhoPJ.ElongfromRho(sp, rho.copy(), P[0], P[1], P[2], *outs)
    out = dict(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, epsr=typespace.GetEpsr(sp), qx=qx,
               qy=qy, qz=qz, rho=rho, Px=Pin[0], Py=Pin[1], Pz=Pin[2], Pk_x=P[0], Pk_y=P[1],
               Pk_z=P[2])
    names = ("ExlfromPRho", "EylfromPRho", "EzlfromPRho", "ExlfromP", "EylfromP", "EzlfromP",
             "ExlfromRho", "EylfromRho", "EzlfromRho", "RhoBound")
    for nm, a in zip(names, outs):
        out[nm] = a
    # q-space and FFT derivatives
    f1 = cnormal(rng, (24,), 1.0)
    f2 = cnormal(rng, (24, 10), 1.0)
    qa = helpers.GetKArray(24, 24 * 7e-9)
    qb = helpers.GetKArray(10, 10 * 9e-9)
    out.update(f1=f1, f2=f2, qa=qa, qb=qb, dfdx1D_q=usefulsubs.dfdx1D_q(f1, qa),
               dfdy1D_q=usefulsubs.dfdy1D_q(f1, qa), dfdx2D_q=usefulsubs.dfdx2D_q(f2, qa),
               dfdy2D_q=usefulsubs.dfdy2D_q(f2, qb), dfdy2D=usefulsubs.dfdy2D(f2.copy(), qb))
    # the axes of the 256 x 128 x 128 x 20 nm grid
    for ax, n in (("x", 256), ("y", 128), ("z", 128)):
        out[f"grid_{ax}"] = typespace.GetSpaceArray(n, (n - 1) * 20e-9)
        out[f"q_{ax}"] = helpers.GetKArray(n, n * 20e-9)
    return out


def main():
    ref_src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PULSESUITE_SRC")
    if not ref_src or not os.path.isdir(ref_src):
        raise SystemExit("usage: make_golden.py /path/to/pulsesuite/src")
    only = sys.argv[2] if len(sys.argv) > 2 else None   # e.g. "mbc": that case alone
    with tempfile.TemporaryDirectory() as tmp:
        _install_stubs(tmp)
        sys.path.insert(0, tmp)
        sys.path.insert(1, os.path.abspath(ref_src))
        work = os.path.join(tmp, "run")
        os.makedirs(work)
        cwd = os.getcwd()
        os.chdir(work)
        sink = io.StringIO()
        try:
            with contextlib.redirect_stdout(sink):
                for nk, seed in ((8, 20), (13, 21)):
                    if only in (None, "mbc"):
                        co = case_coulomb(nk, seed)
                        mb = case_mbc(nk, seed + 400, co["VC1_s1"])
                        np.savez_compressed(os.path.join(HERE, f"mbc_nk{nk}.npz"), **mb)
                    if only in (None, "emission"):
                        co = case_coulomb(nk, seed)
                        em = case_emission(nk, seed + 500, co["VC1_s1"])
                        np.savez_compressed(os.path.join(HERE, f"emission_nk{nk}.npz"), **em)
                    if only in (None, "dc"):
                        np.savez_compressed(os.path.join(HERE, f"dc_nk{nk}.npz"),
                                            **case_dc(nk, seed + 600))
                if only in (None, "info"):
                    for nk, seed in ((8, 800), (13, 801)):
                        np.savez_compressed(os.path.join(HERE, f"info_nk{nk}.npz"),
                                            **case_info(nk, seed))
                if only in (None, "coupling3d"):
                    np.savez_compressed(os.path.join(HERE, "coupling3d.npz"),
                                        **case_coupling3d(900))
                if only in (None, "backup"):
                    np.savez_compressed(os.path.join(HERE, "backup_nk6.npz"),
                                        **case_backup(6, 2, 700))
                if only in (None, "solver100"):
                    np.savez_compressed(os.path.join(HERE, "solver_100.npz"),
                                        **case_solver100(14.5e-9, 100, 0.1e-15, 2e7, 41))
                if only in (None, "pstd3d"):
                    np.savez_compressed(os.path.join(HERE, "pstd3d.npz"), **case_pstd3d(60))
                if only in ("mbc", "emission", "dc", "backup", "info", "coupling3d",
                            "solver100", "pstd3d"):
                    return
                for nk, seed in ((7, 10), (16, 11), (30, 12)):
                    np.savez_compressed(os.path.join(HERE, f"kernels_nk{nk}.npz"), **case_kernels(nk, seed))
                for nk, seed in ((8, 20), (16, 21), (30, 22)):
                    co = case_coulomb(nk, seed)
                    np.savez_compressed(os.path.join(HERE, f"coulomb_nk{nk}.npz"), **co)
                    ph = case_phonon(nk, 77.0 if nk != 16 else 300.0, seed + 100, co["VC1_s1"], co["E1D1_s1"])
                    np.savez_compressed(os.path.join(HERE, f"phonon_nk{nk}.npz"), **ph)
                    de = case_dephasing(nk, seed + 200, co["VC1_s1"])
                    np.savez_compressed(os.path.join(HERE, f"dephasing_nk{nk}.npz"), **de)
                    qo = case_qwoptics(nk, seed + 300)
                    np.savez_compressed(os.path.join(HERE, f"qwoptics_nk{nk}.npz"), **qo)
                np.savez_compressed(os.path.join(HERE, "pstd.npz"), **case_pstd(256, 10e-9, 50))
                so = case_solver(14.5e-9, 3, 0.1e-15, 2e7, 40)
                np.savez_compressed(os.path.join(HERE, "solver_step.npz"), **so)
        finally:
            os.chdir(cwd)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
