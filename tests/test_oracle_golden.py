"""Pin the CPU oracle to the reference's own outputs (golden vectors).

The vectors in tests/golden were produced by tests/golden/make_golden.py from
the reference's functions (CalcH, dpdt/dCdt/dDdt, CoulombModule, phonons,
dephasing, QWOptics, SBESolver.QWCalculator).  Tolerances are relative
Frobenius errors; the oracle reorders sums (vectorised), so 1e-13 is used where
the arithmetic is well conditioned.
"""

import numpy as np
import pytest

from oracle import sbe_oracle as O
from tests.conftest import golden

TOL = 1e-13


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("nk", [7, 16, 30])
def test_calch_and_rhs(nk):
    g = golden(f"kernels_nk{nk}")
    for exc in (0, 1):
        for lf in (0, 1):
            for fp in (0, 1):
                tag = f"e{exc}l{lf}f{fp}"
                H = O.calc_h(g["Meh"], g["Wee"], g["Whh"], g["C"], g["D"], g["P"], g["VC"],
                             g["Ee"], g["Eh"], float(g["gap"]), exc, lf, fp)
                for a, n in zip(H, ("Heh", "Hee", "Hhh")):
                    assert rel(a, g[f"{n}_{tag}"]) < TOL, (tag, n)
    H = (g["Heh_e1l1f0"], g["Hee_e1l1f0"], g["Hhh_e1l1f0"])
    z = np.zeros_like(g["P"])
    assert rel(O.dpdt(g["C"], g["D"], g["P"], *H, g["GamE"], g["GamH"], g["OffP"]), g["dP"]) < TOL
    assert rel(O.dCdt(g["C"], g["D"], g["P"], *H, g["GamE"], g["GamH"], z), g["dC"]) < TOL
    assert rel(O.dDdt(g["C"], g["D"], g["P"], *H, g["GamE"], g["GamH"], z), g["dD"]) < TOL


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_coulomb_tables_and_screening(nk):
    g = golden(f"coulomb_nk{nk}")
    grid = O.wire_grid(nk, float(g["L"]))
    assert np.array_equal(grid["kkp"], g["kkp"])
    assert rel(grid["kr"], g["kr"]) < 1e-15 and rel(grid["r"], g["r"]) == 0.0
    c = dict(alphae=float(g["alphae"]), alphah=float(g["alphah"]))
    ct = O.coulomb_tables(grid, c, float(g["epsr"]), float(g["Delta0"]), float(g["me"]),
                          float(g["mh"]))
    for n in ("Veh0", "Vee0", "Vhh0", "qe", "qh"):
        assert rel(ct[n], g[n]) < TOL, n
    # upper triangle of V0 is zero in the reference (kkp < 0 is skipped)
    assert np.all(np.triu(g["Veh0"], 1) == 0.0)
    for n in ("Chi1De", "Chi1Dh"):
        assert rel(ct[n], g[n]) < 1e-12, n
    for i in (0, 1):
        for s in (0, 1):
            VC, E1D = O.screened_arrays(ct, s, float(g["L"]), g[f"ne{i}"], g[f"nh{i}"])
            assert rel(VC, g[f"VC{i}_s{s}"]) < 1e-12
            assert rel(E1D, g[f"E1D{i}_s{s}"]) < 1e-12
    kj = np.array([O.k0_truncated(x) for x in g["k0_x"]])
    kc = np.array([O.k0_cik(x) for x in g["k0_x"]])
    assert np.max(np.abs(kj - g["k0_jit"]) / np.maximum(np.abs(g["k0_jit"]), 1e-300)) < 1e-14
    assert np.max(np.abs(kc - g["k0_cik"]) / np.maximum(np.abs(g["k0_cik"]), 1e-300)) < 1e-13


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_phonons(nk):
    g = golden(f"phonon_nk{nk}")
    cg = golden(f"coulomb_nk{nk}")
    kr = cg["kr"]
    me, mh = 0.067 * O.ME0, 0.45 * O.ME0
    Ee = O.HBAR ** 2 * kr ** 2 / (2 * me)
    Eh = O.HBAR ** 2 * kr ** 2 / (2 * mh)
    pt = O.phonon_tables(Ee, Eh, 12.9, float(g["Gph"]), float(g["Oph"]), float(g["temp"]))
    for n in ("EP", "HP", "Vscale", "N0"):
        assert rel(pt[n], g[n]) < TOL, n
    wi, wo = O.mbpe(g["ne"], g["VC"], g["E1D"], pt)
    hi, ho = O.mbph(g["nh"], g["VC"], g["E1D"], pt)
    assert rel(g["WinE0"] + wi, g["WinE"]) < TOL
    assert rel(g["WoutE0"] + wo, g["WoutE"]) < TOL
    assert rel(g["WinH0"] + hi, g["WinH"]) < TOL
    assert rel(g["WoutH0"] + ho, g["WoutH"]) < TOL


@pytest.mark.parametrize("nk", [8, 13])
@pytest.mark.parametrize("lorentz", [0, 1])
def test_carrier_scattering(nk, lorentz):
    """MBCE / MBCH (carrier-carrier scattering, EHs) and the CalcMBArrays tables."""
    g = golden(f"mbc_nk{nk}")
    mb = dict(Ee=g["Ee"], Eh=g["Eh"], ge=float(g["ge"]), gh=float(g["gh"]), lorentz=bool(lorentz))
    a, b, d = np.meshgrid(np.arange(nk), np.arange(nk), np.arange(nk), indexing="ij")
    for kind, key in (("eh", "Ceh"), ("ee", "Cee"), ("hh", "Chh")):
        ref = g[f"{key}_l{lorentz}"]
        assert not ref[0].any() and not ref[:, 0].any() and not ref[:, :, 0].any()
        assert rel(O.mb_value(kind, a, b, d, g["Ee"], g["Eh"], mb["ge"], mb["gh"], mb["lorentz"]),
                   ref[1:, 1:, 1:]) < TOL, key
    wi, wo = O.mbce(g["ne"], g["nh"], g["VC"], mb)
    hi, ho = O.mbch(g["ne"], g["nh"], g["VC"], mb)
    for name, mine in (("WinE", wi), ("WoutE", wo), ("WinH", hi), ("WoutH", ho)):
        assert rel(g[f"{name}0_l{lorentz}"] + mine, g[f"{name}_l{lorentz}"]) < TOL, name


@pytest.mark.parametrize("nk", [8, 13])
def test_spont_emission(nk):
    """InitializeEmission tables and SpontEmission (Recomb)."""
    g = golden(f"emission_nk{nk}")
    et = O.emission_tables(abs(float(g["dcv"])), float(g["epsr"]), float(g["geh"]),
                           float(g["ehint"]))
    assert rel(et["HOmega"], g["HOmega"]) < TOL and rel(et["square"], g["square"]) < TOL
    rsp = O.spont_emission(g["ne"], g["nh"], g["Ee"], g["Eh"], float(g["gap"]), g["VC"], et)
    assert rel(rsp, g["Rsp"]) < TOL


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_dephasing(nk):
    g = golden(f"dephasing_nk{nk}")
    dt = O.dephasing_tables(g["kr"], float(g["me"]), float(g["mh"]))
    for n in ("k_p_q", "k_m_q", "k1p", "k1p_m_q", "k1", "k1_m_q"):
        assert np.array_equal(dt[n], g[n]), n
    assert rel(dt["xe"], g["xe"]) < TOL and rel(dt["xh"], g["xh"]) < TOL
    assert rel(O.gamma_e(g["kr"], g["ne"], g["nh"], g["VC"], dt), g["GamE"]) < TOL
    assert rel(O.gamma_h(g["kr"], g["ne"], g["nh"], g["VC"], dt), g["GamH"]) < TOL
    x, De, Dh = O.offdiag_dephasing2(g["ne"], g["nh"], g["P"], g["Ee"], g["Eh"], g["g"], g["VC"])
    assert rel(De, g["De"]) < TOL and rel(Dh, g["Dh"]) < TOL
    assert rel(x, g["OffP"]) < TOL


@pytest.mark.parametrize("nk", [8, 16, 30])
def test_qwoptics(nk):
    g = golden(f"qwoptics_nk{nk}")
    L = float(g["L"])
    win = O.qw_window(g["r"], L)
    E = O.expikr(g["kr"], g["r"])
    assert rel(win, g["window"]) == 0.0 and rel(E, g["Expikr"]) == 0.0
    for w in (1, 2, 3, 4):
        P3 = O.qw_polarization3(g["r"], g["kr"], g["P"], float(g["ehint"]), float(g["area"]), L, w,
                                float(g["dcv"]), win, E)
        for a, n in zip(P3, ("Px", "Py", "Pz")):
            assert rel(a, g[f"{n}_w{w}"]) < 1e-13, (w, n)
    re, rh = O.qw_rho5(g["r"], L, g["C"], g["D"], g["ne"], g["nh"], win, E)
    assert rel(re, g["re"]) < 1e-13 and rel(rh, g["rh"]) < 1e-13
    outs = O.prop2qw(g["RR"], g["Exx"], g["Eyy"], g["Ezz"], g["Vrr"], g["r"], win)
    for a, n in zip(outs, ("Ex", "Ey", "Ez", "Vr")):
        assert rel(a, g[n]) < 1e-14, n
    for pl in (0, 1):
        res = O.qw2prop(g["r"], *[g[f"q2p_in_{n}_{pl}"] for n in ("Px", "Py", "Pz", "re", "rh")],
                        g["RR"], pl)
        for a, n in zip(res, ("Pxx", "Pyy", "Pzz", "RhoE", "RhoH")):
            assert rel(a, g[f"q2p_{n}_{pl}"]) < 1e-14, (pl, n)


@pytest.mark.parametrize("nk", [8, 13])
def test_dc_transport(nk):
    """DCFieldModule.Transport (DCTrans) with and without LF, and its k array."""
    g = golden(f"dc_nk{nk}")
    dky = g["kr"][2] - g["kr"][1]
    assert rel(O.dc_karray(nk, dky), g["Y"]) < 1e-15
    for lf in (0, 1):
        out = O.dc_transport(g[f"C_in_l{lf}"], float(g["Edc"]), float(g["Eac"]), float(g["dt"]),
                             dky, lf)
        assert rel(out, g[f"C_out_l{lf}"]) < 1e-14, lf
        if not lf:   # off the diagonal the matrix is untouched
            off = ~np.eye(nk, dtype=bool)
            assert np.array_equal(out[off], g[f"C_in_l{lf}"][off])


@pytest.mark.parametrize("nk", [8, 13])
def test_wire_info_statistics(nk):
    """The info.WW.t.dat / EP.WW.t.dat statistics against the reference's helpers,
    and the line format of SBEs.py:5772-5809."""
    g = golden(f"info_nk{nk}")
    info, ep = O.wire_info(g["ne2"], g["nh2"], g["re"], g["rh"], list(g["Ek"]), list(g["src3"]),
                           g["kr"], float(g["me"]), float(g["mh"]), g["Ee"], g["Eh"],
                           float(g["gap"]), float(g["L"]), float(g["dkr"]), g["VC"])
    for i, (a, b) in enumerate(zip(info, g["info"])):
        assert abs(a - b) <= 1e-13 * abs(b), i
    assert rel(np.array(ep), g["ep"]) < 1e-15
    line = O.info_line(2e-15, info)
    assert line == O.info_line(2e-15, list(g["info"][:15].real) + list(g["info"][15:]))
    assert len(line.split()) == 18 and line.split()[-1].endswith("j")
    assert O.ep_line(2e-15, ep).count("e") == 7


def test_coupling3d_pieces():
    """CalcJfx, QWPlacement and EAtXYZ (with locator) against the reference."""
    g = golden("coupling3d")
    assert np.array_equal(O.calc_jfx(g["rn"], g["rp"], float(g["dt"]), float(g["dx"])), g["J"])
    grid = O.qw_placement(g["fw"], g["gx"], g["gy"], g["gz"])
    assert np.array_equal(grid.view(np.int64), g["grid"].view(np.int64))
    val = np.array([O.e_at_xyz(g["f"], g["x"], g["y"], g["z"], *p) for p in g["pts"]])
    assert np.array_equal(val.view(np.int64), g["val"].view(np.int64))


SOLVER_PARAMS = dict(gap=1.52 * O.E0, me=0.067 * O.ME0, mh=0.45 * O.ME0, HO=100e-3 * O.E0,
                     Delta0=6e-9, gam_e=1e12, gam_h=1e12, gam_eh=1e12, epsr=12.9,
                     Oph=36e-3 * O.E0 / O.HBAR, Gph=3e-3 * O.E0 / O.HBAR)
SOLVER_FLAGS = dict(Optics=1, Excitons=1, EHs=0, Screened=1, Phonon=1, DCTrans=0, LF=1,
                    FreePot=0, DiagDph=1, OffDiagDph=1, Recomb=0)


def test_solver_leapfrog_steps():
    """Three QWCalculator steps on two wires: outputs and all nine state levels."""
    g = golden("solver_step")
    L = float(g["L"])
    nk = O.grid_from_params(L, SOLVER_PARAMS["gap"], SOLVER_PARAMS["me"])
    assert nk == int(g["nk"])
    s = O.Solver(nk, L, SOLVER_PARAMS, SOLVER_FLAGS, 2, float(g["E0"]))
    assert rel(s.wire.g["kr"], g["kr"]) == 0.0
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        setattr(s, nm, g["init_" + nm].copy())
    rr, dt = g["rr"], float(g["dt"])
    for n in range(3):
        for w in (1, 2):
            out = s.qw_calculator(g[f"s{n}_Exx"], g[f"s{n}_Eyy"], g[f"s{n}_Ezz"],
                                  np.zeros(len(rr), complex), rr, dt, w)
            for a, nm in zip(out, ("Pxx", "Pyy", "Pzz", "Rho")):
                assert rel(a, g[f"s{n}_w{w}_{nm}"]) < 1e-13, (n, w, nm)
        for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
            assert rel(getattr(s, nm), g[f"s{n}_{nm}"]) < 1e-14, (n, nm)


def test_solver_leapfrog_100_steps():
    """100 QWCalculator steps on two wires: sources of every tenth step and the nine
    state levels at the end (the reference scheme over a long run)."""
    g = golden("solver_100")
    L = float(g["L"])
    nk = O.grid_from_params(L, SOLVER_PARAMS["gap"], SOLVER_PARAMS["me"])
    assert nk == int(g["nk"])
    s = O.Solver(nk, L, SOLVER_PARAMS, SOLVER_FLAGS, 2, float(g["E0"]))
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        setattr(s, nm, g["init_" + nm].copy())
    rr, dt, f = g["rr"], float(g["dt"]), g["fields"]
    nsteps = int(g["nsteps"])
    for n in range(nsteps):
        for w in (1, 2):
            out = s.qw_calculator(f[n, 0] + 0j, f[n, 1] + 0j, f[n, 2] + 0j,
                                  np.zeros(len(rr), complex), rr, dt, w)
            if f"s{n}_w{w}_Pxx" in g:
                for a, nm in zip(out, ("Pxx", "Pyy", "Pzz", "Rho")):
                    assert rel(a, g[f"s{n}_w{w}_{nm}"]) < 1e-12, (n, w, nm)
    for nm in ("YY1", "YY2", "YY3", "CC1", "CC2", "CC3", "DD1", "DD2", "DD3"):
        assert rel(getattr(s, nm), g[f"end_{nm}"]) < 1e-12, nm


def test_constants_match_scipy():
    sc = pytest.importorskip("scipy.constants")
    assert O.HBAR == sc.hbar and O.E0 == sc.e and O.KB == sc.k
    assert O.EPS0 == sc.epsilon_0 and O.ME0 == sc.m_e
