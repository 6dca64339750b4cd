"""FP64 GPU path vs the reference's golden vectors and the oracle (needs a GPU).

Every call goes through the C ABI of libsbe_gb300 (ctypes, torch device
buffers).  Tolerances are relative Frobenius errors; the FP64 GPU path sums in a
different order from NumPy, and the K0 series of the reference loses ~8 digits
to cancellation near x = 9 (its Chi1D entries there agree to ~1e-9), so
screening-dependent results use 1e-10.
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from oracle import sbe_oracle as O  # noqa: E402
from tests.conftest import golden  # noqa: E402

TIGHT = 1e-12
SCREEN = 1e-10


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pulsesuite_gb300 import build
    build.build()


def dev(x, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(x))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda().contiguous()


def host(t):
    return t.detach().cpu().numpy()


MAT = dict(me=0.067 * O.ME0, mh=0.45 * O.ME0, gap=1.52 * O.E0, HO=100e-3 * O.E0, Delta0=6e-9,
           gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR,
           Gph=3e-3 * O.E0 / O.HBAR)
ALL = dict(Optics=True, Excitons=True, EHs=False, Screened=True, Phonon=True, DCTrans=False,
           LF=True, FreePot=False, DiagDph=True, OffDiagDph=True, Recomb=False)


def ctx_for(nk, L, nw=1, temp=77.0, flags=None):
    from pulsesuite_gb300.wires import WireContext, WireSpec
    specs = [WireSpec(nk=nk, L=L, temp=temp, wire_index=w + 1, flags=dict(flags or ALL), **MAT)
             for w in range(nw)]
    return WireContext(specs)


@pytest.mark.parametrize("nk", [7, 16, 30])
def test_rhs_functions_vs_golden(nk):
    from pulsesuite_gb300 import SBEs
    g = golden(f"kernels_nk{nk}")
    H = (g["Heh_e1l1f0"], g["Hee_e1l1f0"], g["Hhh_e1l1f0"])
    dP = SBEs.dpdt(g["C"], g["D"], g["P"], *H, g["GamE"], g["GamH"], g["OffP"])
    dC = SBEs.dCdt(g["C"], g["D"], g["P"], *H, g["GamE"], g["GamH"], g["OffP"])
    dD = SBEs.dDdt(g["C"], g["D"], g["P"], *H, g["GamE"], g["GamH"], g["OffP"])
    assert rel(dP, g["dP"]) < TIGHT
    assert rel(dC, g["dC"]) < TIGHT
    assert rel(dD, g["dD"]) < TIGHT


@pytest.mark.parametrize("nk", [7, 16, 30])
def test_calch_vs_golden(nk):
    from pulsesuite_gb300 import SBEs
    g = golden(f"kernels_nk{nk}")
    for exc in (0, 1):
        for lf in (0, 1):
            for fp in (0, 1):
                tag = f"e{exc}l{lf}f{fp}"
                out = [np.zeros((nk, nk), complex) for _ in range(3)]
                SBEs.calc_h(g["Meh"], g["Wee"], g["Whh"], g["C"], g["D"], g["P"], g["VC"], *out,
                            g["Ee"], g["Eh"], float(g["gap"]), exc, lf, fp)
                for a, n in zip(out, ("Heh", "Hee", "Hhh")):
                    assert rel(a, g[f"{n}_{tag}"]) < TIGHT, (tag, n)


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_tables_vs_golden(nk):
    g = golden(f"coulomb_nk{nk}")
    ph = golden(f"phonon_nk{nk}")
    de = golden(f"dephasing_nk{nk}")
    qo = golden(f"qwoptics_nk{nk}")
    c = ctx_for(nk, float(g["L"]), temp=float(ph["temp"]))
    assert rel(host(c.table(0, "kr")), g["kr"]) < 1e-15
    assert rel(host(c.table(0, "r")), g["r"]) == 0.0
    v0 = host(c.table(0, "V0"))
    for i, n in enumerate(("Veh0", "Vee0", "Vhh0")):
        assert rel(v0[i], g[n][:, 0]) < 1e-13, n
    chi = host(c.table(0, "Chi1D"))
    assert rel(chi[0], g["Chi1De"][:, 0]) < SCREEN
    assert rel(chi[1], g["Chi1Dh"][:, 0]) < SCREEN
    assert rel(host(c.table(0, "EP")), ph["EP"]) < 1e-13
    assert rel(host(c.table(0, "HP")), ph["HP"]) < 1e-13
    maps = host(c.table(0, "maps"))
    for i, n in enumerate(("k_p_q", "k_m_q", "k1p", "k1p_m_q", "k1", "k1_m_q")):
        assert np.array_equal(maps[i], de[n]), n
    xx = host(c.table(0, "xexh"))
    assert rel(xx[0], de["xe"]) < 1e-14 and rel(xx[1], de["xh"]) < 1e-14
    assert rel(host(c.table(0, "window")), qo["window"]) < 1e-14
    assert rel(host(c.table(0, "Expikr")), qo["Expikr"]) < 1e-14


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_screening_vs_golden(nk):
    g = golden(f"coulomb_nk{nk}")
    for scr in (0, 1):
        c = ctx_for(nk, float(g["L"]), flags=dict(ALL, Screened=bool(scr)))
        for i in (0, 1):
            VC, E1D = c.screened_arrays(0, dev(g[f"ne{i}"]), dev(g[f"nh{i}"]))
            assert rel(host(VC), g[f"VC{i}_s{scr}"]) < SCREEN
            assert rel(host(E1D), g[f"E1D{i}_s{scr}"]) < SCREEN


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_dephasing_vs_golden(nk):
    g = golden(f"dephasing_nk{nk}")
    cg = golden(f"coulomb_nk{nk}")
    c = ctx_for(nk, float(cg["L"]))
    ge, gh = c.gamma(0, dev(g["ne"]), dev(g["nh"]), dev(g["VC"]))
    assert rel(host(ge), g["GamE"]) < TIGHT
    assert rel(host(gh), g["GamH"]) < TIGHT
    x, De, Dh = c.offdiag(0, dev(g["ne"]), dev(g["nh"]), dev(g["P"]), dev(g["VC"]), g["g"])
    assert rel(host(De), g["De"]) < TIGHT
    assert rel(host(Dh), g["Dh"]) < TIGHT
    assert rel(host(x), g["OffP"]) < TIGHT


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_phonon_rates_vs_golden(nk):
    g = golden(f"phonon_nk{nk}")
    cg = golden(f"coulomb_nk{nk}")
    c = ctx_for(nk, float(cg["L"]), temp=float(g["temp"]))
    w = [dev(g[n]) for n in ("WinE0", "WoutE0", "WinH0", "WoutH0")]
    c.phonon_rates(0, dev(g["ne"].astype(complex)), dev(g["nh"].astype(complex)), dev(g["VC"]),
                   dev(g["E1D"]), *w)
    for t, n in zip(w, ("WinE", "WoutE", "WinH", "WoutH")):
        assert rel(host(t), g[n]) < TIGHT, n


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_sources_and_resampling_vs_golden(nk):
    g = golden(f"qwoptics_nk{nk}")
    c = ctx_for(nk, float(g["L"]), nw=4)
    rho_scale = 2.0 * O.E0 * float(g["ehint"]) / float(g["area"])
    for w in (1, 2, 3, 4):
        Px, Py, Pz, re, rh = c.sources(w - 1, dev(g["P"]), dev(g["C"]), dev(g["D"]),
                                       dev(g["ne"]), dev(g["nh"]))
        for a, n in zip((Px, Py, Pz), ("Px", "Py", "Pz")):
            assert rel(O.fftg(host(a)), g[f"{n}_w{w}"]) < TIGHT, (w, n)
        assert rel(O.fftg(host(re)) / rho_scale, g["re"]) < TIGHT
        assert rel(O.fftg(host(rh)) / rho_scale, g["rh"]) < TIGHT
    RR = dev(g["RR"])
    f4 = dev(np.stack([g["Exx"], g["Eyy"], g["Ezz"], g["Vrr"]]))
    Ek = host(c.prop2qw(0, RR, f4))
    for i, n in enumerate(("Ex", "Ey", "Ez", "Vr")):
        assert rel(Ek[i], g[n]) < 1e-13, n
    for pl in (0, 1):
        src = np.stack([O.ifftg(g[f"q2p_in_{n}_{pl}"]) for n in ("Px", "Py", "Pz", "re", "rh")])
        out = host(c.qw2prop(0, RR, dev(src), pl))
        for i, n in enumerate(("Pxx", "Pyy", "Pzz", "RhoE", "RhoH")):
            assert rel(out[i], g[f"q2p_{n}_{pl}"]) < 1e-13, (pl, n)


SOLVER_FLAGS = dict(Optics=1, Excitons=1, EHs=0, Screened=1, Phonon=1, DCTrans=0, LF=1,
                    FreePot=0, DiagDph=1, OffDiagDph=1, Recomb=0, ignorewire=0)


def test_solver_leapfrog_vs_golden(tmp_path, monkeypatch):
    """Three reference QWCalculator steps on two wires (SBESolver drop-in)."""
    from pulsesuite_gb300 import SBEs
    monkeypatch.chdir(tmp_path)   # the solver appends dataQW/info and EP files
    g = golden("solver_step")
    prm = dict(L=float(g["L"]), Delta0=6e-9, gap=1.52 * O.E0, me=0.067 * O.ME0,
               mh=0.45 * O.ME0, HO=100e-3 * O.E0, gam_e=1e12, gam_h=1e12, gam_eh=1e12,
               epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR, Gph=3e-3 * O.E0 / O.HBAR, Edc=0.0,
               jmax=100000, ntmax=100000)
    rr = g["rr"]
    s = SBEs.SBESolver(np.zeros(len(rr)), rr, 0.0, float(g["E0"]), 800e-9, 2, True, params=prm,
                       flags=SOLVER_FLAGS)
    assert s.Nk == int(g["nk"])
    assert rel(s.kr, g["kr"]) == 0.0
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        setattr(s, nm, g["init_" + nm])
    dt = float(g["dt"])
    for n in range(3):
        for w in (1, 2):
            outs = [np.zeros(len(rr), complex) for _ in range(4)]
            s.QWCalculator(g[f"s{n}_Exx"], g[f"s{n}_Eyy"], g[f"s{n}_Ezz"],
                           np.zeros(len(rr), complex), rr, None, dt, w, *outs, [False], [False])
            for a, nm in zip(outs, ("Pxx", "Pyy", "Pzz", "Rho")):
                assert rel(a, g[f"s{n}_w{w}_{nm}"]) < SCREEN, (n, w, nm)
        for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
            assert rel(getattr(s, nm), g[f"s{n}_{nm}"]) < SCREEN, (n, nm)
    s.close()


def test_batched_solver_leapfrog_vs_golden(tmp_path, monkeypatch):
    """SBESolver(batch=True): both wires in one context, stepped together on the call
    for wire 2, outputs of wire 1 filled then; the reference driver's call order gives
    the reference's three steps."""
    from pulsesuite_gb300 import SBEs
    monkeypatch.chdir(tmp_path)
    g = golden("solver_step")
    prm = dict(L=float(g["L"]), Delta0=6e-9, gap=1.52 * O.E0, me=0.067 * O.ME0,
               mh=0.45 * O.ME0, HO=100e-3 * O.E0, gam_e=1e12, gam_h=1e12, gam_eh=1e12,
               epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR, Gph=3e-3 * O.E0 / O.HBAR, Edc=0.0,
               jmax=100000, ntmax=100000)
    rr = g["rr"]
    s = SBEs.SBESolver(np.zeros(len(rr)), rr, 0.0, float(g["E0"]), 800e-9, 2, True, params=prm,
                       flags=SOLVER_FLAGS, batch=True)
    assert len(s.contexts) == 1
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        setattr(s, nm, g["init_" + nm])
    dt = float(g["dt"])
    for n in range(3):
        outs = {}
        for w in (1, 2):
            outs[w] = [np.zeros(len(rr), complex) for _ in range(4)]
            s.QWCalculator(g[f"s{n}_Exx"], g[f"s{n}_Eyy"], g[f"s{n}_Ezz"],
                           np.zeros(len(rr), complex), rr, None, dt, w, *outs[w], [False], [False])
        for w in (1, 2):
            for a, nm in zip(outs[w], ("Pxx", "Pyy", "Pzz", "Rho")):
                assert rel(a, g[f"s{n}_w{w}_{nm}"]) < SCREEN, (n, w, nm)
        for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
            assert rel(getattr(s, nm), g[f"s{n}_{nm}"]) < SCREEN, (n, nm)
    s.close()


def _diagnostic_files_match(g):
    """The text diagnostics of the run against the reference's files: the same lines,
    the times equal, the values within 1e-8 of their column's largest magnitude."""
    for key, path in (("pdote_p", "output/PdotE.p.dat"), ("pdote_w", "output/PdotE.w.dat"),
                      ("maxoff_e", "dataQW/Wire/info/MaxOffDiag.e.dat"),
                      ("maxoff_h", "dataQW/Wire/info/MaxOffDiag.h.dat")):
        want = np.array([[float(v) for v in ln.split()]
                         for ln in bytes(g["txt_" + key]).decode().splitlines()])
        with open(path, encoding="utf-8") as fh:
            got = np.array([[float(v) for v in ln.split()] for ln in fh.read().splitlines()])
        assert got.shape == want.shape, (key, got.shape, want.shape)
        assert np.array_equal(got[:, 0], want[:, 0]), key
        for c in range(1, want.shape[1]):
            scale = np.abs(want[:, c]).max()
            assert np.abs(got[:, c] - want[:, c]).max() <= 1e-8 * scale, (key, c)


@pytest.mark.parametrize("batch", [False, True])
def test_solver_leapfrog_100_steps_vs_golden(tmp_path, monkeypatch, batch):
    """100 reference QWCalculator steps on two wires (SBESolver drop-in, FP64 path):
    the sources of every tenth step and the nine state levels at the end <= 1e-10,
    and the PdotE and MaxOffDiag files the reference wrote on the way."""
    from pulsesuite_gb300 import SBEs
    monkeypatch.chdir(tmp_path)
    g = golden("solver_100")
    prm = dict(L=float(g["L"]), Delta0=6e-9, gap=1.52 * O.E0, me=0.067 * O.ME0,
               mh=0.45 * O.ME0, HO=100e-3 * O.E0, gam_e=1e12, gam_h=1e12, gam_eh=1e12,
               epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR, Gph=3e-3 * O.E0 / O.HBAR, Edc=0.0,
               jmax=100000, ntmax=100000)
    rr, f = g["rr"], g["fields"]
    s = SBEs.SBESolver(np.zeros(len(rr)), rr, 0.0, float(g["E0"]), 800e-9, 2, True, params=prm,
                       flags=SOLVER_FLAGS, batch=batch)
    assert s.Nk == int(g["nk"])
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        setattr(s, nm, g["init_" + nm])
    dt = float(g["dt"])
    for n in range(int(g["nsteps"])):
        step_outs = {}
        for w in (1, 2):
            outs = [np.zeros(len(rr), complex) for _ in range(4)]
            s.QWCalculator(f[n, 0] + 0j, f[n, 1] + 0j, f[n, 2] + 0j, np.zeros(len(rr), complex),
                           rr, None, dt, w, *outs, [False], [False])
            step_outs[w] = outs
        # (batched: every wire's outputs are filled on the call for the last wire)
        for w in (1, 2):
            if f"s{n}_w{w}_Pxx" in g:
                for a, nm in zip(step_outs[w], ("Pxx", "Pyy", "Pzz", "Rho")):
                    assert rel(a, g[f"s{n}_w{w}_{nm}"]) < SCREEN, (n, w, nm)
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        assert rel(getattr(s, nm), g[f"end_{nm}"]) < SCREEN, nm
    s.close()
    _diagnostic_files_match(g)


def _seeded_state(rng, nk):
    z = rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk))
    q, _ = np.linalg.qr(z)
    C = (q * rng.uniform(0, 0.1, nk)) @ q.conj().T
    z = rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk))
    q, _ = np.linalg.qr(z)
    D = (q * rng.uniform(0, 0.1, nk)) @ q.conj().T
    P = 1e-3 * (rng.standard_normal((nk, nk)) + 1j * rng.standard_normal((nk, nk))) / np.sqrt(2)
    return P, C, D


def _uniform_field_k(wire, E):
    """Wire-k-space field of a spatially uniform field E along y (Prop2QW of a
    constant): E * FFTG(window)."""
    wk = O.fftg(wire.window)
    z = np.zeros_like(wk)
    return [z, E * wk, z]


@pytest.mark.parametrize("nk", [16, 34])
def test_batched_rhs_and_rk4_vs_oracle(nk):
    """Full RHS (preparation included) and one RK4 step, 3 wires, FP64 path."""
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    nw = 3
    c = ctx_for(nk, L, nw=nw)
    rng = np.random.default_rng(5)
    wires = [O.Wire(nk, L, MAT, ALL) for _ in range(nw)]
    states = [_seeded_state(rng, nk) for _ in range(nw)]
    fields = [_uniform_field_k(wires[w], 1e7 * (w + 1)) for w in range(nw)]
    dfields = [_uniform_field_k(wires[w], -3e5 * (w + 1)) for w in range(nw)]
    P = c.pack([s[0] for s in states])
    C = c.pack([s[1] for s in states])
    D = c.pack([s[2] for s in states])
    Ek = c.pack_r([np.stack(f) for f in fields], 3)
    dEk = c.pack_r([np.stack(f) for f in dfields], 3)
    dP, dC, dD = c.rhs(P, C, D, Ek)
    for w in range(nw):
        rP, rC, rD, _ = wires[w].rhs(*states[w], *fields[w], w + 1)
        assert rel(host(c.mat(dP, w)), rP) < SCREEN
        assert rel(host(c.mat(dC, w)), rC) < SCREEN
        assert rel(host(c.mat(dD, w)), rD) < SCREEN
    dt = 0.1e-15
    src = c.zeros_r(5)
    c.rk4_step(P, C, D, Ek, dEk, dt, src)
    charge = c.charge().numpy()
    for w in range(nw):
        ref = wires[w].rk4_step(*states[w], fields[w], dfields[w], dt, w + 1)
        assert rel(host(c.mat(P, w)), ref[0]) < SCREEN
        assert rel(host(c.mat(C, w)), ref[1]) < SCREEN
        assert rel(host(c.mat(D, w)), ref[2]) < SCREEN
        # the conservation record: carrier numbers before the normalisation, and the
        # normalised diagonals summing to their mean
        assert rel(charge[w], np.array(wires[w].last_charge)) < SCREEN
        ne = np.abs(np.diag(host(c.mat(C, w)))).sum()
        assert abs(ne - charge[w].mean()) <= 1e-12 * ne
        s5 = host(c.rvec(src, w, 5))
        for i in range(5):
            assert rel(O.fftg(s5[i]), ref[3 + i]) < SCREEN, (w, i)


@pytest.mark.parametrize("nk", [8, 13])
@pytest.mark.parametrize("lorentz", [0, 1])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_carrier_rates_vs_golden(nk, lorentz, precision):
    """MBCE / MBCH through sbe_carrier_rates against the reference's own rates
    (FP64: 1e-12; FP32 with exact integer energy sums: 1e-6 of the added rates)."""
    from pulsesuite_gb300.wires import WireContext, WireSpec
    g = golden(f"mbc_nk{nk}")
    L = np.pi / (g["kr"][1] - g["kr"][0])
    mat = dict(MAT, gam_e=float(g["ge"]), gam_h=float(g["gh"]))
    flags = dict(ALL, EHs=True, LorentzDelta=bool(lorentz))
    c = WireContext([WireSpec(nk=nk, L=L, wire_index=1, flags=flags, **mat)])
    w = [dev(g[f"{n}0_l{lorentz}"]) for n in ("WinE", "WoutE", "WinH", "WoutH")]
    c.carrier_rates(0, dev(g["ne"]), dev(g["nh"]), dev(g["VC"]), *w, precision=precision)
    for t, n in zip(w, ("WinE", "WoutE", "WinH", "WoutH")):
        add_ref = g[f"{n}_l{lorentz}"] - g[f"{n}0_l{lorentz}"]
        add = host(t) - g[f"{n}0_l{lorentz}"]
        tol = TIGHT if precision == "fp64" else 1e-6
        assert rel(add, add_ref) < (tol if precision == "mixed" else 1e-11), n
        if precision == "fp64":
            assert rel(host(t), g[f"{n}_l{lorentz}"]) < TIGHT, n


@pytest.mark.parametrize("lorentz", [0, 1])
def test_rk4_with_carrier_scattering_vs_oracle(lorentz):
    """One RK4 step with EHs on (carrier-carrier rates in the relaxation), FP64 path."""
    nk = 16
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    nw = 2
    flags = dict(ALL, EHs=True, LorentzDelta=bool(lorentz))
    c = ctx_for(nk, L, nw=nw, flags=flags)
    rng = np.random.default_rng(9)
    wires = [O.Wire(nk, L, MAT, flags) for _ in range(nw)]
    states = [_seeded_state(rng, nk) for _ in range(nw)]
    fields = [_uniform_field_k(wires[w], 1e7 * (w + 1)) for w in range(nw)]
    dfields = [_uniform_field_k(wires[w], -3e5 * (w + 1)) for w in range(nw)]
    P = c.pack([s[0] for s in states])
    C = c.pack([s[1] for s in states])
    D = c.pack([s[2] for s in states])
    Ek = c.pack_r([np.stack(f) for f in fields], 3)
    dEk = c.pack_r([np.stack(f) for f in dfields], 3)
    dt = 0.1e-15
    src = c.zeros_r(5)
    c.rk4_step(P, C, D, Ek, dEk, dt, src)
    for w in range(nw):
        ref = wires[w].rk4_step(*states[w], fields[w], dfields[w], dt, w + 1)
        # the carrier-carrier rates moved the occupations measurably
        ref_ph = O.Wire(nk, L, MAT, dict(ALL)).rk4_step(*states[w], fields[w], dfields[w], dt,
                                                        w + 1)
        assert rel(np.diag(ref[1]), np.diag(ref_ph[1])) > 1e-8
        assert rel(host(c.mat(P, w)), ref[0]) < SCREEN
        assert rel(host(c.mat(C, w)), ref[1]) < SCREEN
        assert rel(host(c.mat(D, w)), ref[2]) < SCREEN


@pytest.mark.parametrize("nk", [8, 13])
def test_spont_emission_vs_golden(nk):
    """SpontEmission (Recomb) through sbe_spont_emission against the reference's Rsp."""
    from pulsesuite_gb300.wires import WireContext, WireSpec
    g = golden(f"emission_nk{nk}")
    L = np.pi / (g["kr"][1] - g["kr"][0])
    mat = dict(MAT, gam_eh=float(g["geh"]))
    c = WireContext([WireSpec(nk=nk, L=L, wire_index=1, flags=dict(ALL, Recomb=True), **mat)])
    rsp = c.spont_emission(0, dev(g["ne"]), dev(g["nh"]), dev(g["VC"]))
    assert rel(host(rsp), g["Rsp"]) < TIGHT


def test_rk4_with_recombination_vs_oracle():
    """One RK4 step with Recomb (and EHs) on, FP64 path, against the oracle."""
    nk = 16
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    nw = 2
    flags = dict(ALL, Recomb=True, EHs=True)
    c = ctx_for(nk, L, nw=nw, flags=flags)
    rng = np.random.default_rng(13)
    wires = [O.Wire(nk, L, MAT, flags) for _ in range(nw)]
    states = [_seeded_state(rng, nk) for _ in range(nw)]
    fields = [_uniform_field_k(wires[w], 1e7 * (w + 1)) for w in range(nw)]
    dfields = [_uniform_field_k(wires[w], -3e5 * (w + 1)) for w in range(nw)]
    P = c.pack([s[0] for s in states])
    C = c.pack([s[1] for s in states])
    D = c.pack([s[2] for s in states])
    Ek = c.pack_r([np.stack(f) for f in fields], 3)
    dEk = c.pack_r([np.stack(f) for f in dfields], 3)
    dt = 0.1e-15
    src = c.zeros_r(5)
    c.rk4_step(P, C, D, Ek, dEk, dt, src)
    for w in range(nw):
        ref = wires[w].rk4_step(*states[w], fields[w], dfields[w], dt, w + 1)
        assert rel(host(c.mat(P, w)), ref[0]) < SCREEN
        assert rel(host(c.mat(C, w)), ref[1]) < SCREEN
        assert rel(host(c.mat(D, w)), ref[2]) < SCREEN


@pytest.mark.parametrize("lf", [True, False])
def test_rk4_with_dc_transport_vs_oracle(lf):
    """One RK4 step with DCTrans on (the shift of P, C, D after the relaxation; with LF
    off only the diagonals), FP64 path, against the oracle.  LF off also runs Recomb
    without Phonon or EHs: no relaxation, so no decay."""
    from pulsesuite_gb300.wires import WireContext, WireSpec
    nk = 16
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    nw = 2
    flags = dict(ALL, DCTrans=True, LF=lf)
    if not lf:
        flags.update(Phonon=False, EHs=False, Recomb=True)
    edc = [4e7, -2.5e7]
    c = WireContext([WireSpec(nk=nk, L=L, temp=77.0, wire_index=w + 1, flags=dict(flags),
                              Edc=edc[w], **MAT) for w in range(nw)])
    rng = np.random.default_rng(17)
    wires = [O.Wire(nk, L, dict(MAT, Edc=edc[w]), flags) for w in range(nw)]
    states = [_seeded_state(rng, nk) for _ in range(nw)]

    def fld(w, ex, ey):
        wk = O.fftg(wires[w].window)
        return [ex * wk, ey * wk, np.zeros_like(wk)]

    fields = [fld(w, 3e7 * (w + 1), 1e7) for w in range(nw)]
    dfields = [fld(w, -2e5, 3e5) for w in range(nw)]
    P = c.pack([s[0] for s in states])
    C = c.pack([s[1] for s in states])
    D = c.pack([s[2] for s in states])
    Ek = c.pack_r([np.stack(f) for f in fields], 3)
    dEk = c.pack_r([np.stack(f) for f in dfields], 3)
    dt = 0.1e-15
    src = c.zeros_r(5)
    c.rk4_step(P, C, D, Ek, dEk, dt, src)
    for w in range(nw):
        ref = wires[w].rk4_step(*states[w], fields[w], dfields[w], dt, w + 1)
        nodc = O.Wire(nk, L, dict(MAT, Edc=edc[w]), dict(flags, DCTrans=False)).rk4_step(
            *states[w], fields[w], dfields[w], dt, w + 1)
        assert rel(nodc[1], ref[1]) > 1e-4   # the shift is visible at this tolerance
        assert rel(host(c.mat(P, w)), ref[0]) < SCREEN
        assert rel(host(c.mat(C, w)), ref[1]) < SCREEN
        assert rel(host(c.mat(D, w)), ref[2]) < SCREEN


def _last_line(path):
    with open(path, encoding="utf-8") as f:
        return f.read().splitlines()[-1].split()


def _close_printed(tokens, want):
    """Printed %18.6e values against the expected numbers (7 significant digits)."""
    assert len(tokens) == len(want)
    for tok, w in zip(tokens, want):
        got = complex(tok) if tok.endswith("j") else float(tok)
        assert abs(got - w) <= 1e-6 * abs(w) + 1e-300, (tok, w)


def test_solver_leapfrog_dc_vs_oracle(tmp_path, monkeypatch):
    """Three QWCalculator steps with DCTrans on (and Edc), SBESolver against the
    oracle's solver, from the reference's saved initial state and fields; each step's
    dataQW/info.WW.t.dat and EP.WW.t.dat lines against the oracle's statistics."""
    from pulsesuite_gb300 import SBEs
    monkeypatch.chdir(tmp_path)
    g = golden("solver_step")
    prm = dict(L=float(g["L"]), Delta0=6e-9, gap=1.52 * O.E0, me=0.067 * O.ME0,
               mh=0.45 * O.ME0, HO=100e-3 * O.E0, gam_e=1e12, gam_h=1e12, gam_eh=1e12,
               epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR, Gph=3e-3 * O.E0 / O.HBAR, Edc=6e7,
               jmax=100000, ntmax=100000)
    flags = dict(SOLVER_FLAGS, DCTrans=1)
    rr = g["rr"]
    s = SBEs.SBESolver(np.zeros(len(rr)), rr, 0.0, float(g["E0"]), 800e-9, 2, True, params=prm,
                       flags=flags)
    ref = O.Solver(s.Nk, prm["L"], prm, {k: bool(v) for k, v in flags.items()}, 2,
                   float(g["E0"]))
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        setattr(s, nm, g["init_" + nm])
        setattr(ref, nm, g["init_" + nm].copy())
    dt = float(g["dt"])
    for n in range(3):
        for w in (1, 2):
            outs = [np.zeros(len(rr), complex) for _ in range(4)]
            s.QWCalculator(g[f"s{n}_Exx"], g[f"s{n}_Eyy"], g[f"s{n}_Ezz"],
                           np.zeros(len(rr), complex), rr, None, dt, w, *outs, [False], [False])
            exp = ref.qw_calculator(g[f"s{n}_Exx"], g[f"s{n}_Eyy"], g[f"s{n}_Ezz"],
                                    np.zeros(len(rr), complex), rr, dt, w)
            for a, b, nm in zip(outs, exp, ("Pxx", "Pyy", "Pzz", "Rho")):
                assert rel(a, b) < SCREEN, (n, w, nm)
            info, ep = ref.last_info
            t = s.xxx * dt
            _close_printed(_last_line(f"dataQW/info.{w:02d}.t.dat"), [t] + list(info))
            _close_printed(_last_line(f"dataQW/EP.{w:02d}.t.dat"), [t] + list(ep))
        for nm in ("YY1", "CC1", "DD1", "CC3"):
            assert rel(getattr(s, nm), getattr(ref, nm)) < SCREEN, (n, nm)
    assert rel(ref.CC3, g["s2_CC3"]) > 1e-6   # the transport changed the state
    s.close()


def test_dc_transport_leaves_other_wires_untouched():
    """A context of one wire with DCTrans + LF and one without: the second wire's RK4
    step (FP64 path) is bit for bit the step of that wire in a context of its own (the
    transport's circulant products run on the DCTrans wires only)."""
    from pulsesuite_gb300.wires import WireContext, WireSpec
    nk = 16
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    dc = dict(ALL, DCTrans=True)
    both = WireContext([WireSpec(nk=nk, L=L, temp=77.0, wire_index=1, flags=dc, Edc=5e7, **MAT),
                        WireSpec(nk=nk, L=L, temp=77.0, wire_index=2, flags=dict(ALL), **MAT)])
    alone = WireContext([WireSpec(nk=nk, L=L, temp=77.0, wire_index=2, flags=dict(ALL), **MAT)])
    rng = np.random.default_rng(17)
    st = [_seeded_state(rng, nk) for _ in range(2)]
    wire = O.Wire(nk, L, MAT, ALL)
    fld = [_uniform_field_k(wire, 2e7), _uniform_field_k(wire, 1e7)]
    dfld = [_uniform_field_k(wire, -1e5), _uniform_field_k(wire, 3e5)]
    P2, C2, D2 = (both.pack([s[i] for s in st]) for i in range(3))
    P1, C1, D1 = (alone.pack([st[1][i]]) for i in range(3))
    both.rk4_step(P2, C2, D2, both.pack_r([np.stack(f) for f in fld], 3),
                  both.pack_r([np.stack(f) for f in dfld], 3), 0.1e-15, both.zeros_r(5))
    alone.rk4_step(P1, C1, D1, alone.pack_r([np.stack(fld[1])], 3),
                   alone.pack_r([np.stack(dfld[1])], 3), 0.1e-15, alone.zeros_r(5))
    torch.cuda.synchronize()
    for a, b in ((P2, P1), (C2, C1), (D2, D1)):
        assert torch.equal(both.mat(a, 1), alone.mat(b, 0))
    assert not torch.equal(both.mat(C2, 0), both.pack([st[0][1]])[:nk * nk].view(nk, nk))


def test_solver_backup_files_round_trip(tmp_path, monkeypatch):
    """write_sbes_data / read_sbes_data (SBEs.py:5524-5569) of the GPU solver's nine
    levels: the files hold the reference writer's text of the levels, and reading
    them back restores every level."""
    from pulsesuite_gb300 import SBEs
    g = golden("solver_step")
    prm = dict(L=float(g["L"]), Delta0=6e-9, gap=1.52 * O.E0, me=0.067 * O.ME0,
               mh=0.45 * O.ME0, HO=100e-3 * O.E0, gam_e=1e12, gam_h=1e12, gam_eh=1e12,
               epsr=12.9, Oph=36e-3 * O.E0 / O.HBAR, Gph=3e-3 * O.E0 / O.HBAR, Edc=0.0,
               jmax=100000, ntmax=100000)
    rr = g["rr"]
    s = SBEs.SBESolver(np.zeros(len(rr)), rr, 0.0, float(g["E0"]), 800e-9, 2, True, params=prm,
                       flags=SOLVER_FLAGS)
    levels = ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3")
    for nm in levels:
        setattr(s, nm, g["s1_" + nm])
    monkeypatch.chdir(tmp_path)
    s.write_sbes_data(12)
    for nm in levels:
        arr = getattr(s, nm)
        want = "".join(f"{np.real(arr[k1, k2, w])} {np.imag(arr[k1, k2, w])}\n"
                       for w in range(arr.shape[2]) for k2 in range(s.Nk) for k1 in range(s.Nk))
        with open(f"dataQW/backup/{nm}.12.dat", encoding="utf-8") as f:
            assert f.read() == want, nm
    for nm in levels:
        setattr(s, nm, np.zeros_like(g["s1_" + nm]))
    s.read_sbes_data(12)
    for nm in levels:
        assert np.array_equal(getattr(s, nm), g["s1_" + nm]), nm
    s.close()


def test_wire_info_vs_oracle():
    """sbe_wire_info on a seeded state, sources and field against the oracle's
    statistics (FP64, all 23 numbers), with the format of the reference's lines."""
    from pulsesuite_gb300.wires import WireContext, WireSpec
    nk = 16
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    c = WireContext([WireSpec(nk=nk, L=L, temp=77.0, wire_index=1, flags=dict(ALL), **MAT)])
    wire = O.Wire(nk, L, MAT, ALL)
    rng = np.random.default_rng(31)
    P, C, D = _seeded_state(rng, nk)
    nr = 2 * nk + 2
    src = (rng.standard_normal((5, nr)) + 1j * rng.standard_normal((5, nr))) * 1e-3
    Ek = [(rng.standard_normal(nr) + 1j * rng.standard_normal(nr)) * 1e6 for _ in range(3)]
    ne = np.abs(np.diag(C)).astype(complex)
    nh = np.abs(np.diag(D)).astype(complex)
    VC, _ = O.screened_arrays(wire.ct, True, L, ne, nh)
    v = c.wire_info(0, c.pack([C]), c.pack([D]), dev(src.reshape(-1)),
                    dev(np.concatenate(Ek)), dev(VC.reshape(-1)))
    # the oracle takes the sources in wire-k space, as the reference holds them
    ks = [O.fftg(x) for x in src]
    info, ep = O.wire_info(ne, nh, ks[3], ks[4], Ek, ks[:3], wire.g["kr"], MAT["me"],
                           MAT["mh"], wire.c["Ee"], wire.c["Eh"], MAT["gap"], L, np.pi / L, VC)
    want = [np.real(x) for x in info] + list(ep)
    for i, (a, b) in enumerate(zip(v, want)):
        assert abs(a - b) <= 1e-12 * abs(b) + 1e-300, (i, a, b)
    assert np.imag(info[15]) == 0.0 and np.imag(info[16]) == 0.0


def test_wire_pdote_and_deph_extrema_vs_oracle():
    """sbe_wire_pdote against sum (Re P - P0) Re iFFTG(E) of the oracle, and
    sbe_deph_extrema against the De, Dh the library's preparation produced."""
    from pulsesuite_gb300.wires import WireContext, WireSpec
    nk = 16
    L = np.pi / (3e9 / (nk / 2 - 0.5))
    c = WireContext([WireSpec(nk=nk, L=L, temp=77.0, wire_index=w + 1, flags=dict(ALL), **MAT)
                     for w in range(2)])
    rng = np.random.default_rng(33)
    nr = 2 * nk + 2
    src = [(rng.standard_normal((5, nr)) + 1j * rng.standard_normal((5, nr))) * 1e-3
           for _ in range(2)]
    Ek = [(rng.standard_normal((3, nr)) + 1j * rng.standard_normal((3, nr))) * 1e6
          for _ in range(2)]
    P0 = rng.standard_normal((3, nr)) * 1e-3
    for w in range(2):
        got = c.wire_pdote(w, c.pack_r(Ek, 3), c.pack_r(src, 5), dev(P0))
        want = sum(np.sum((src[w][i].real - P0[i]) * O.ifftg(Ek[w][i]).real) for i in range(3))
        assert abs(got - want) <= 1e-12 * np.abs(src[w][:3].real * O.ifftg(Ek[w][0]).real).sum()
        got0 = c.wire_pdote(w, c.pack_r(Ek, 3), c.pack_r(src, 5), None)
        want0 = sum(np.sum(src[w][i].real * O.ifftg(Ek[w][i]).real) for i in range(3))
        assert abs(got0 - want0) <= 1e-12 * abs(want0) + 1e-300
    states = [_seeded_state(rng, nk) for _ in range(2)]
    De, Dh = c.deph(c.pack([s[1] for s in states]), c.pack([s[2] for s in states]), fp32=False)
    off = 0
    for w in range(2):
        n = (2 * nk + 1) * nk
        e, h = De[off:off + n], Dh[off:off + n]
        v = c.deph_extrema(w)
        assert list(v) == [float(e.max()), float(e.min()), float(h.max()), float(h.min())]
        off += n
    c.close()
